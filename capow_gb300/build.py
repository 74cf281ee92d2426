"""Build recipe for libcapow_gpu.so (CUDA, sm_103a) and the `capow` C driver.

Everything is compiled in-tree into capow_gb300/_build (library) and capow_gb300/bin
(driver); both folders are git-ignored. Translation units compile in parallel.
Host code is compiled with -ffp-contract=off so the double-precision threshold and
frequency tables reproduce the reference's x86-64 (no FMA) arithmetic on any host.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
DRV = os.path.join(HERE, "driver")
BUILD = os.path.join(HERE, "_build")
BIN = os.path.join(HERE, "bin")
LIB = os.path.join(BUILD, "libcapow_gpu.so")
DRIVER = os.path.join(BIN, "capow")

CU_SOURCES = ["capow_api.cu", "paint.cu", "bin.cu", "noalloc.cu", "adjoint.cu", "batch.cu", "survey.cu"]
C_SOURCES = ["params.c", "catalogue.c", "output.c", "survey_io.c"]
DRIVER_SOURCES = ["main.c"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcapow_gpu")


def _cuda_include(nvcc: str) -> str:
    """The toolkit's include directory (the host C sources call the CUDA runtime for pinned memory)."""
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + [
        os.path.join(ROOT, "include", "capow.h")]


def build_library(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", s, "-o", o])
    for src in C_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".c", ".o"))
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            jobs.append(["gcc", "-O2", "-std=gnu99", "-fPIC", "-ffp-contract=off", "-Wall", "-pthread", "-I",
                         os.path.join(ROOT, "include"), "-I", _cuda_include(nvcc), "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return r

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _newer(LIB, objs):
        run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcufft", "-lpthread"])
    return LIB


def build_driver(force: bool = False) -> str:
    os.makedirs(BIN, exist_ok=True)
    srcs = [os.path.join(DRV, f) for f in DRIVER_SOURCES]
    deps = srcs + [os.path.join(DRV, f) for f in os.listdir(DRV) if f.endswith(".h")] + [
        os.path.join(ROOT, "include", "capow.h"), LIB]
    if force or _newer(DRIVER, deps):
        cmd = ["gcc", "-O2", "-std=gnu99", "-ffp-contract=off", "-Wall", "-I", os.path.join(ROOT, "include"), "-o",
               DRIVER, *srcs, "-L", BUILD, "-lcapow_gpu", "-Wl,-rpath," + BUILD, "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("driver build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return DRIVER


def build(force: bool = False, verbose: bool = False) -> None:
    build_library(force=force, verbose=verbose)
    build_driver(force=force)


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
    print(DRIVER)
