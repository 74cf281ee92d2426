"""Benchmark: ms per P0/P2/P4(k) evaluation of the periodic power-spectrum path.

Workload (the headline configuration): 256^3 = 16,777,216 Zel'dovich-displaced lattice particles
(float32, seeded synthetic; no dataset), box L = 1000 Mpc/h, TSC on a 512^3 grid with interlacing,
density-density, density-momentum and momentum-momentum spectra from one paint, LOS = z (RSD shift),
NK = 161 linear bins to k = 1.61 h/Mpc.

One step = one full evaluation: paint (4 grids) -> z pass (k_zr2c) and cuFFT y pass -> fused x-axis
FFT + bin kernel -> device-to-host copy of the bins. ``value`` times steps with the particles already
resident in HBM (CUDA events on the context stream, barrier + synchronize on both sides, max over
ranks); ``e2e`` times the same evaluations through the public C-ABI calls with pinned HOST particle
buffers, each step's host-to-device copy and read-back inside the timed region, as a stream of
catalogues (capow_power_enqueue / capow_power_result, each copy overlapping the previous evaluation);
``e2e_sequential`` the same one call after the other. Grids (2.15 GB) and particles (268 MB) exceed
L2, so no separate flush is needed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

With N > 1 (torchrun) every rank runs an independent replica (the path does not shard without an
exchange step); value = max-over-ranks time / (N * K).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms per P0/2/4(k) at 512³ grid, 16.7M particles: FP32-mixed vs FP64 GPU vs CPU"
UNIT = "ms"
WORKLOAD = ("256^3 Zel'dovich particles (16,777,216, f32), L=1000 Mpc/h, TSC 512^3, interlaced, "
            "dd+dp+pp P0/P2/P4, LOS=z (RSD), NK=161 to k=1.61")

PARAMS = dict(NX=512, NY=512, NZ=512, XMIN=0.0, XMAX=1000.0, YMIN=0.0, YMAX=1000.0, ZMIN=0.0, ZMAX=1000.0,
              InterpOrder=3, DoInterlacing=1, NK=161, NMU=1, Output2D=0, OutputLog=0, Mink=0.0, Maxk=1.61,
              Omega_m=0.3089, Redshift=0.1, LOS=3, Momentum=0, Odd_Multipoles=0)
N_SIDE = 256
SEED = 2
PRECISION = ("fp32-mixed: FP32 grids, FFT, per-thread bin runs and per-CTA bin copies; FP64 global bin sums, "
             "scalars and near-edge indices; exact k-bins")
# DRAM read + write bytes of one launch at this workload, from one ncu capture of it
TRAFFIC_TILE_REC = 512893000 + 2119952000
TRAFFIC_XFFT_BIN = 1768743000 + 3229000


def algorithmic_bytes(n_particles: int, ng: int, nc: int, grids: int, b_p: int, b_r: int, b_c: int) -> int:
    """B = N_p b_p + G N_g b_r + G (N_g b_r + N_c b_c) + G N_c b_c (paint write, FFT read+write, bin read)."""
    return n_particles * b_p + grids * ng * b_r + grids * (ng * b_r + nc * b_c) + grids * nc * b_c


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.rows.append([c.strip() for c in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    except Exception:
        return {"hbm_gbs": 6800.0, "source": "fallback"}


def make_particles():
    """The workload's particles, generated on the host (both arms get the same values)."""
    from capow_gb300 import synth

    return synth.zeldovich(N_SIDE, L=1000.0, mesh=512, rms_cells=1.5, seed=SEED)


def dist_init():
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(world, v: float, device) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------------------------------ CPU
def cpu_model() -> dict:
    """Host cores and CPU model of this box (for the reference arm's line)."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                model = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if not model:
        import platform

        model = platform.processor() or platform.machine()
    return {"nproc": os.cpu_count(), "model": model}


def config_dict(n_particles: int) -> dict:
    return {"workload": WORKLOAD, "grid": 512, "particles": n_particles, "interp": "TSC", "interlacing": True,
            "spectra": ["dd", "dp", "pp"], "l2": "inputs larger than L2 (grids 2.15 GB, particles 268 MB)",
            "parallelism": "replicas"}


def cpu_reference(steps: int, warmup: int, parts, log=print) -> dict:
    """The reference's algorithm on the host cores: the CPU oracle (the periodic path of the reference
    restated in C, single threaded as the reference's periodic path is without MPI). One step is one
    full evaluation of the workload: the three reference runs that give dd, dp and pp (Momentum 0, 1,
    2), each with its own paint, mean subtraction, FFTs, binning and normalisation, run side by side as
    three single-threaded processes. The FFT is scipy's pocketfft (the reference links FFTW, absent
    here). The step time is the longest of the three runs (they start together); particle loading is
    outside it, as the GPU arm's particles are resident. Returns the median step and the runs' raw sums
    of the last step."""
    import tempfile

    import oracle as orc

    p = orc.Params(**{k: v for k, v in PARAMS.items() if k in orc.Params.__dataclass_fields__})
    samples, last = [], None
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "parts.npz")
        orc.save_particles(path, *parts)
        with orc.ParallelRuns(3) as pool:
            for it in range(warmup + steps):
                t0 = time.perf_counter()
                out = pool.run(p, path, [0, 1, 2], timeout=1800)
                wall = (time.perf_counter() - t0) * 1e3
                per = [o[1] * 1e3 for o in out]
                if it >= warmup:
                    samples.append((max(per), wall, per))
                last = out
                log(f"cpu step {it}{' (warm-up)' if it < warmup else ''}: {max(per):.0f} ms "
                    f"(Momentum 0/1/2 runs {per[0]:.0f} / {per[1]:.0f} / {per[2]:.0f} ms, wall {wall:.0f} ms)")
    val = statistics.median(s[0] for s in samples)
    info = cpu_model()
    return {"value": val, "unit": UNIT, "cores": 3, "kind": "port",
            "sample": ("per step: one full evaluation, the three reference runs for dd, dp, pp (Momentum 0, 1, 2) "
                       "of all 16,777,216 particles on the 512^3 TSC grid, each single threaded, run side by side; "
                       "FFT scipy.fft pocketfft (the reference links FFTW)"),
            "runs_ms": {f"momentum_{m}": statistics.median(s[2][m] for s in samples) for m in (0, 1, 2)},
            "wall_ms": statistics.median(s[1] for s in samples), "nproc": info["nproc"], "cpu_model": info["model"],
            "raw": {m: last[m][0] for m in (0, 1, 2)}}


def accuracy_vs_oracle(res, raw) -> dict:
    """Max over bins of the normalised |P_l(GPU) - P_l(oracle)| per spectrum (parity_util's measure: l = 0
    against P0 + shot/norm, l = 2, 4 times (2l+1); dp normalised by sqrt(P_dd P_pp)), and whether the
    mode counts are equal."""
    dd, pp = np.abs(raw[0]["raw"]["Pk0"]), np.abs(raw[2]["raw"]["Pk0"])
    acc = {}
    for q, (name, norm0) in enumerate((("dd", dd), ("dp", np.sqrt(dd * pp)), ("pp", pp))):
        ref = raw[q]["raw"]
        m = (np.asarray(ref["Nmodes"]) > 0) & (norm0 > 0)
        acc[name] = {f"l{l}": float(np.max((2 * l + 1) * np.abs(np.asarray(res[q][f"Pk{l}"])[m] - ref[f"Pk{l}"][m])
                                            / norm0[m])) for l in (0, 2, 4)}
        acc[name]["nmodes_equal"] = bool(np.array_equal(np.asarray(res[q]["Nmodes"], np.int64),
                                                        np.asarray(ref["Nmodes"], np.int64)))
    return acc


# ------------------------------------------------------------------------------------------ GPU
def profile_case(args):
    """The workload scaled down by 8 for profiler captures: 128^3 Zel'dovich particles (2,097,152, f32) on
    a 256^3 TSC grid with the same settings otherwise (grids 270 MB: above L2, a few hundred MB on the
    device). Runs warm-up + steps evaluations and prints the last one's stage times; no JSON line."""
    import torch

    import capow_gb300 as cg
    from capow_gb300 import synth

    dev = torch.device("cuda", 0)
    x, y, z, vx, vy, vz = synth.zeldovich(N_SIDE // 2, L=1000.0, mesh=256, rms_cells=1.5, seed=SEED,
                                          torch_device=dev)
    d = [torch.from_numpy(a).to(dev) for a in (x, y, z, vz)]
    params = cg.Params(**dict(PARAMS, NX=256, NY=256, NZ=256, NK=81, Maxk=0.81))
    with cg.PowerSpectrum(params, precision="fp32", spectra=["dd", "dp", "pp"], fft_path=args.fft_path) as ps:
        for _ in range(args.warmup + args.steps):
            ps.paint(*d)
            ps.power()
        print("profile case (2,097,152 particles, 256^3): paint %.3f ms, fft %.3f ms, bin %.3f ms" % ps.stage_ms())


def batch_bench(args):
    """The batched-mocks workload: 256 mocks, box L ~ U[500, 1500] Mpc/h, grid from {128^3, 192^3, 256^3},
    particle counts log-uniform in [0.5M, 8M] (cube lattices), Zel'dovich-displaced as the main workload
    (rms 1.5 cells of each grid), CIC and TSC alternating, interlaced, density P0/P2/P4 with LOS = z,
    FP32. capow_batch calls (tile autotuner; direct enqueue and the cached CUDA graph; the first call,
    which sets the batch up, timed apart) against 256 sequential plain-path runs (create, paint, power,
    destroy per mock). Prints one JSON line in mocks per second."""
    import torch

    import capow_gb300 as cg
    from capow_gb300 import synth

    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(1000)
    mocks = []
    for i in range(args.mocks):
        L = float(rng.uniform(500.0, 1500.0))
        ng = int(rng.choice([128, 192, 256]))
        side = max(8, int(round(np.exp(rng.uniform(np.log(0.5e6), np.log(8e6))) ** (1.0 / 3.0))))
        x, y, z, vx, vy, vz = synth.zeldovich(side, L=L, mesh=ng, rms_cells=1.5, seed=1000 + i, torch_device=dev)
        parts = tuple(torch.from_numpy(a).to(dev) for a in (x, y, z, vz)) + (None,)
        nk = int(np.floor((np.pi * ng / L) / 0.01))
        p = cg.Params(NX=ng, NY=ng, NZ=ng, XMIN=0.0, XMAX=L, YMIN=0.0, YMAX=L, ZMIN=0.0, ZMAX=L,
                      InterpOrder=2 + (i % 2), DoInterlacing=1, NK=nk, Maxk=nk * 0.01, LOS=3, Momentum=0)
        mocks.append((p, parts))
    npart = sum(len(m[1][0]) for m in mocks)
    torch.cuda.synchronize()

    def timed(graph):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = cg.run_batch(mocks, precision="fp32", graph=graph, autotune=True)
        torch.cuda.synchronize()
        return time.perf_counter() - t0, out

    # the first call sets up the batch (shared contexts, tables, the autotuner's tile choice); later
    # calls with the same mocks reuse that state; the first graph call also captures the graph
    cg.release_batch()
    t_cold, _ = timed(False)
    t_direct = statistics.median(timed(False)[0] for _ in range(3))
    t_graph_first, _ = timed(True)
    reps = [timed(True) for _ in range(3)]
    t_graph = statistics.median(r[0] for r in reps)
    out = reps[-1][1]
    cg.release_batch()
    times = {False: t_direct, True: t_graph}
    graph_best = times[True] < times[False]
    t_batch = times[graph_best]
    ok = sum(1 for s, _ in out if s == cg.OK)
    t0 = time.perf_counter()
    for p, parts in mocks:
        with cg.PowerSpectrum(p, precision="fp32") as ps:
            ps.paint(*parts[:4])
            ps.power()
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0
    line = {"metric": "mocks per second, 256 uneven periodic mocks (batched)", "value": round(len(mocks) / t_batch, 2),
            "unit": "mocks/s", "higher_is_better": True, "n_gpus": 1, "mocks": len(mocks), "mocks_ok": ok,
            "particles": int(npart), "batch_s": round(t_batch, 3), "batch_s_graph": round(times[True], 3),
            "batch_s_direct": round(times[False], 3), "batch_s_first_call": round(t_cold, 3),
            "batch_s_first_graph_call": round(t_graph_first, 3), "sequential_s": round(t_seq, 3),
            "sequential_mocks_per_s": round(len(mocks) / t_seq, 2), "speedup": round(t_seq / t_batch, 2),
            "data": "synthetic (seeded Zel'dovich lattices)", "dtype": "f32",
            "config": {"workload": "256 mocks, L~U[500,1500], grid in {128,192,256}^3, N_p log-uniform 0.5M-8M, "
                                   "CIC/TSC alternating, interlaced, density P0/P2/P4, LOS=z",
                       "graph": bool(graph_best), "autotune": True}}
    print(json.dumps(line), flush=True)


def scale_bench(args):
    """The large single-mock workload: a 512^3 Zel'dovich lattice (134,217,728 particles, f32), L = 2000 Mpc/h,
    CIC on a 1024^3 grid, interlaced, density and LOS-momentum multipoles (dd, dp, pp). FP32-mixed and
    deterministic int64 modes timed and compared bin by bin with the FP64 path. Prints one JSON line."""
    import torch

    import capow_gb300 as cg
    from capow_gb300 import synth

    dev = torch.device("cuda", 0)
    x, y, z, vx, vy, vz = synth.zeldovich(512, L=2000.0, mesh=1024, rms_cells=1.5, seed=2, torch_device=dev)
    d = [torch.from_numpy(a).to(dev) for a in (x, y, z, vz)]
    del x, y, z, vx, vy
    p = cg.Params(**dict(PARAMS, NX=1024, NY=1024, NZ=1024, XMAX=2000.0, YMAX=2000.0, ZMAX=2000.0, InterpOrder=2,
                         NK=160, Maxk=1.6))
    ts = torch.cuda.Stream(device=dev)
    res, ms = {}, {}
    for prec in ("fp32", "det", "fp64"):
        with cg.PowerSpectrum(p, precision=prec, spectra=["dd", "dp", "pp"], stream=ts.cuda_stream) as ps:
            reps = 2 if prec == "fp64" else 4
            times = []
            for it in range(reps + 1):
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(ts)
                ps.paint(*d)
                r = ps.power()
                e1.record(ts)
                torch.cuda.synchronize()
                if it:
                    times.append(e0.elapsed_time(e1))
            res[prec], ms[prec] = r, statistics.median(times)
    acc = {}
    for prec in ("fp32", "det"):
        acc[prec] = {}
        for q, name in enumerate(("dd", "dp", "pp")):
            r, r64 = res[prec][q], res["fp64"][q]
            m = np.asarray(r64["Nmodes"]) > 0
            n0 = np.abs(r64["Pk0"]) if name != "dp" else np.sqrt(np.abs(res["fp64"][0]["Pk0"] * res["fp64"][2]["Pk0"]))
            acc[prec][name] = {f"l{l}": float(np.max((2 * l + 1) * np.abs(r[f"Pk{l}"][m] - r64[f"Pk{l}"][m]) / n0[m]))
                               for l in (0, 2, 4)}
            acc[prec][name]["nmodes_equal"] = bool(np.array_equal(r["Nmodes"], r64["Nmodes"]))
    line = {"metric": "ms per dd+dp+pp P0/2/4(k), 1024^3 CIC, 134M particles", "unit": "ms", "higher_is_better": False,
            "fp32_ms": round(ms["fp32"], 2), "det_ms": round(ms["det"], 2), "fp64_ms": round(ms["fp64"], 2),
            "accuracy_vs_fp64": acc, "n_gpus": 1, "data": "synthetic (seeded Zel'dovich lattice, f32)",
            "config": {"workload": "512^3 lattice (134,217,728 particles), L=2000 Mpc/h, CIC 1024^3, interlaced, "
                                   "dd+dp+pp, LOS=z, NK=160 to k=1.6"}}
    print(json.dumps(line), flush=True)


PARAM_TAGS = ("NumFilesInParallel NX NY NZ XMIN XMAX YMIN YMAX ZMIN ZMAX DoInterlacing InterpOrder NK NMU Output2D "
              "OutputLog Mink Maxk Omega_m Redshift Periodic LOS Survey Momentum X_Origin Y_Origin Z_Origin REDMININ "
              "REDMAXIN NOBJ_Max Coord_Type x_Column y_Column z_Column NBAR_Column SkyArea FKP_Column FKP_Pk "
              "FKP_Pk_mom FKP_Pk_cross Odd_Multipoles").split()


def write_params_file(path: str, params: dict) -> None:
    """A run_parameters.dat with the 41 tags the reference's reader requires (src/read_params.c:65-227):
    the given values, the periodic estimator, and neutral survey tags."""
    v = {t: 0 for t in PARAM_TAGS}
    v.update(NumFilesInParallel=1, Periodic=1, Survey=0, NOBJ_Max=1, x_Column=1, y_Column=2, z_Column=3,
             NBAR_Column=4, SkyArea=1.0, FKP_Column=5, FKP_Pk=1.0, FKP_Pk_mom=1.0, FKP_Pk_cross=1.0, REDMAXIN=1.0)
    v.update(params)
    with open(path, "w") as f:
        for t in PARAM_TAGS:
            f.write(f"{t} {v[t]!r}\n" if isinstance(v[t], float) else f"{t} {v[t]}\n")


def cli_bench(args):
    """The drop-in driver end to end: `capow <params> <data> none <out>` as a user runs it, timed as whole
    processes (CUDA context creation included) with the driver's own phase times (CAPOW_TIMING=1).
    Two runs: the headline workload (16,777,216 Zel'dovich particles, TSC 512^3, dd+dp+pp through
    CAPOW_SPECTRA) from a binary column catalogue (float32), and the plain run's workload (2,097,152
    uniform particles, CIC 128^3, LOS = z) from a text catalogue written with %.9g. Median of
    `--steps` runs each (at least 3). Prints one JSON line."""
    import tempfile

    import capow_gb300 as cg
    from capow_gb300 import synth

    reps = max(args.steps, 3)

    def run(pf, df, env_extra):
        env = dict(os.environ, CAPOW_TIMING="1", **env_extra)
        walls, phases = [], []
        with tempfile.TemporaryDirectory() as tmp:
            for _ in range(reps):
                t0 = time.perf_counter()
                r = subprocess.run([cg.DRIVER_PATH, pf, df, "none", os.path.join(tmp, "out.txt")],
                                   capture_output=True, text=True, env=env, timeout=600)
                walls.append(time.perf_counter() - t0)
                if r.returncode != 0:
                    raise RuntimeError(r.stdout[-2000:] + r.stderr[-2000:])
                line = [s for s in r.stderr.splitlines() if s.startswith("capow timing")][-1]
                toks = line.split(":", 1)[1].split()
                phases.append({toks[i]: float(toks[i + 1]) for i in range(0, len(toks), 2)})
        med = {k: round(statistics.median(p[k] for p in phases), 4) for k in phases[0]}
        return {"wall_s": round(statistics.median(walls), 4), "phases_s": med}

    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        x, y, z, vx, vy, vz = make_particles()
        pf, df = os.path.join(tmp, "c1.dat"), os.path.join(tmp, "c1.bin")
        write_params_file(pf, PARAMS)
        cg.write_soa_catalogue(df, x, y, z, vx, vy, vz, dtype=np.float32)
        out["c1_binary"] = run(pf, df, {"CAPOW_SPECTRA": "dd,dp,pp", "CAPOW_PRECISION": "fp32"})
        out["c1_binary"]["catalogue_bytes"] = os.path.getsize(df)
        rng = np.random.default_rng(1)
        n0 = 2_097_152
        pos = rng.uniform(0.0, 1000.0, size=(n0, 3))
        vel = rng.normal(0.0, 300.0, size=(n0, 3))
        p0 = dict(PARAMS, NX=128, NY=128, NZ=128, InterpOrder=2, NK=41, Maxk=0.41)
        pf0, df0 = os.path.join(tmp, "c0.dat"), os.path.join(tmp, "c0.txt")
        write_params_file(pf0, p0)
        np.savetxt(df0, np.hstack([pos, vel]), fmt="%.9g")
        out["c0_text"] = run(pf0, df0, {"CAPOW_PRECISION": "fp32"})
        out["c0_text"]["catalogue_bytes"] = os.path.getsize(df0)
    line = {"metric": "capow CLI wall time per run (process start to exit)", "unit": "s", "higher_is_better": False,
            "value": out["c1_binary"]["wall_s"], "n_gpus": 1, "runs": reps, **out,
            "data": "synthetic (seeded Zel'dovich lattice; uniform particles for the text run)",
            "config": {"workload": f"{WORKLOAD}, binary float32 columns, CAPOW_SPECTRA=dd,dp,pp; and 2,097,152 "
                                   "uniform particles, CIC 128^3, LOS=z, text catalogue (%.9g)"}}
    print(json.dumps(line), flush=True)


SURVEY_PARAMS = dict(NX=512, NY=512, NZ=512, XMIN=-1000.0, XMAX=1000.0, YMIN=-1000.0, YMAX=1000.0, ZMIN=-1000.0,
                     ZMAX=1000.0, InterpOrder=3, DoInterlacing=1, NK=100, NMU=1, Output2D=0, OutputLog=0, Mink=0.0,
                     Maxk=0.5, Omega_m=0.3089, Redshift=0.1, LOS=0, Momentum=0, Odd_Multipoles=0)


def survey_catalogues(n_side: int, L: float, radius: float, ratio: int, seed: int):
    """A full-sky survey around an observer at the box centre: data = a Zel'dovich lattice of n_side^3 in
    [-L/2, L/2)^3 kept within `radius`; randoms = `ratio` times as many uniform points in the same ball;
    w = 1, nbar = N_data / V_ball. float32 host arrays (the reference's object fields)."""
    from capow_gb300 import synth

    x, y, z, vx, vy, vz = synth.zeldovich(n_side, L=L, mesh=512, rms_cells=1.5, seed=seed)
    pos = np.stack([x, y, z], 1).astype(np.float64) - L / 2
    d = pos[(pos ** 2).sum(1) < radius ** 2]
    rng = np.random.default_rng(seed + 1)
    nr = ratio * len(d)
    u = rng.normal(size=(nr, 3))
    r = u / np.linalg.norm(u, axis=1)[:, None] * (radius * rng.uniform(size=(nr, 1)) ** (1.0 / 3.0))
    nbar = len(d) / (4.0 / 3.0 * np.pi * radius ** 3)

    def cat(a):
        n = len(a)
        return {"x": a[:, 0].astype(np.float32), "y": a[:, 1].astype(np.float32), "z": a[:, 2].astype(np.float32),
                "w": np.ones(n, np.float32), "nbar": np.full(n, nbar, np.float32)}
    return cat(d), cat(r)


def survey_bench(args):
    """The survey estimator (Periodic 0, Survey 1): a full-sky survey around an observer at the centre of a
    2000 Mpc/h box, 192^3-lattice Zel'dovich data inside radius 950 (3.1M objects) and 10x as many uniform
    randoms, TSC on a 512^3 grid with interlacing, FKP weights (P_FKP = 10^4), P0/P2/P4 to k = 0.5
    (15 FFT sets of two grids). Times FP32 and FP64 evaluations with the catalogues resident in HBM (CUDA
    events on the context stream) and through the C ABI with host arrays (e2e), and the oracle (the
    reference's survey algorithm in C, one core) beside the GPU on a bounded sample: a 128^3 grid with
    1/16 of the objects, timed on both. Prints one JSON line."""
    import torch

    import capow_gb300 as cg
    import oracle as orc

    dev = torch.device("cuda", 0)
    data, rand = survey_catalogues(192, 2000.0, 950.0, 10, SEED)
    p = cg.Params(**SURVEY_PARAMS)
    sv = cg.SurveyParams(X_Origin=0.0, Y_Origin=0.0, Z_Origin=0.0, FKP_Column=-1, FKP_Pk=1e4, NBAR_Column=5)
    dd = {k: torch.from_numpy(v).to(dev) for k, v in data.items()}
    rr = {k: torch.from_numpy(v).to(dev) for k, v in rand.items()}
    ts = torch.cuda.Stream(device=dev)
    out = {}
    for prec, reps in (("fp32", max(args.steps, 3)), ("fp64", 3)):
        with cg.SurveySpectrum(p, sv, precision=prec, stream=ts.cuda_stream) as ss:
            for _ in range(2):
                ss.power(dd, rr)
            times, walls = [], []
            for _ in range(reps):
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(ts)
                res = ss.power(dd, rr)
                e1.record(ts)
                torch.cuda.synchronize()
                times.append(e0.elapsed_time(e1))
                stage = ss.stage_ms()
            for _ in range(reps):  # end to end: host float32 arrays copied in by the call
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                ss.power(data, rand)
                walls.append((time.perf_counter() - t0) * 1e3)
            out[prec] = {"ms": statistics.median(times), "e2e_ms": statistics.median(walls), "res": res,
                         "stage": stage, "launches": ss.kernel_launches()}
    r32, r64 = out["fp32"]["res"], out["fp64"]["res"]
    m = np.asarray(r64["Nmodes"]) > 0
    acc = {f"l{l}": float(np.max((2 * l + 1) * np.abs(r32[f"Pk{l}"][m] - r64[f"Pk{l}"][m]) / np.abs(r64["Pk0"][m])))
           for l in (0, 2, 4)}
    # bounded sample for the CPU: 128^3 grid, 1/16 of the objects, through the oracle and the GPU
    ps = cg.Params(**dict(SURVEY_PARAMS, NX=128, NY=128, NZ=128, NK=25))
    sub = {k: v[::16] for k, v in data.items()}, {k: v[::16] for k, v in rand.items()}
    import tempfile
    with tempfile.TemporaryDirectory() as tmp:
        po = orc.Params(**{**SURVEY_PARAMS, "NX": 128, "NY": 128, "NZ": 128, "NK": 25, "Periodic": 0,
                           "X_Origin": 0.0, "Y_Origin": 0.0, "Z_Origin": 0.0, "REDMININ": 0.0, "REDMAXIN": 10.0,
                           "NOBJ_Max": 1 << 30, "NBAR_Column": 5, "FKP_Column": -1, "FKP_Pk": 1e4})
        files = []
        for nm, c, cols in (("d", sub[0], 12), ("r", sub[1], 8)):
            a = np.zeros((len(c["x"]), cols))
            for j, k in enumerate(("x", "y", "z", "w", "nbar")):
                a[:, j] = c[k]
            f = os.path.join(tmp, nm + ".txt")
            np.savetxt(f, a, fmt="%.9g")
            files.append(f)
        t0 = time.perf_counter()
        orc.survey_run(po, files[0], files[1])
        cpu_s = time.perf_counter() - t0
    with cg.SurveySpectrum(ps, sv, precision="fp64", stream=ts.cuda_stream) as ss:
        ss.power(sub[0], sub[1])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ss.power(sub[0], sub[1])
        gpu_sample_ms = (time.perf_counter() - t0) * 1e3
    nd, nr = len(data["x"]), len(rand["x"])
    line = {"metric": "ms per survey P0/2/4(k), 512^3 TSC interlaced, 3.1M data + 31M randoms", "unit": "ms",
            "higher_is_better": False, "value": round(out["fp32"]["ms"], 3), "n_gpus": 1, "dtype": "f32",
            "fp64_ms": round(out["fp64"]["ms"], 2),
            "e2e": {"value": round(out["fp32"]["e2e_ms"], 3), "unit": "ms",
                    "h2d_bytes_per_step": 4 * 5 * (nd + nr), "d2h_bytes_per_step": 8 * 5 * p.NK},
            "fp64_e2e_ms": round(out["fp64"]["e2e_ms"], 2),
            "stages_ms": {prec: {"paint": round(out[prec]["stage"][0], 3),
                                 "multipoles": round(out[prec]["stage"][1], 3), "fft_sets": out[prec]["stage"][2]}
                          for prec in ("fp32", "fp64")},
            "gpu_launches": int(out["fp32"]["launches"]), "accuracy_fp32_vs_fp64": acc,
            "cpu_baseline": {"value": round(cpu_s * 1e3, 1), "unit": "ms", "cores": 1, "kind": "port",
                             "sample": f"128^3 grid, {len(sub[0]['x'])} data + {len(sub[1]['x'])} randoms (1/16), "
                                       "the oracle's survey path (Cartesian products: 22 FFT sets)",
                             "gpu_fp64_ms_same_sample": round(gpu_sample_ms, 2), "cpu_model": cpu_model()},
            "data": "synthetic (seeded Zel'dovich lattice within a ball; uniform randoms)",
            "config": {"workload": f"survey: {nd} data, {nr} randoms, observer at the centre of a 2000 Mpc/h box, "
                                   "TSC 512^3 interlaced, FKP P=1e4, NK=100 to k=0.5, even multipoles"}}
    print(json.dumps(line), flush=True)


def gpu_bench(args, world, rank, local):
    import torch

    import capow_gb300 as cg

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    parts = make_particles()
    x, y, z, vx, vy, vz = parts
    n = len(x)
    params = cg.Params(**PARAMS)
    d = [torch.from_numpy(a).to(dev) for a in (x, y, z, vz)]
    host = [torch.from_numpy(a).pin_memory() for a in (x, y, z, vz)]
    torch.cuda.synchronize()
    # every context runs on this stream, and every CUDA event below is recorded on it
    ts = torch.cuda.Stream(device=dev)
    sh = ts.cuda_stream
    ps = cg.PowerSpectrum(params, precision="fp32", spectra=["dd", "dp", "pp"], device=local, stream=sh,
                          fft_path=args.fft_path)

    def step_device():
        ps.paint(*d)
        return ps.power()

    def step_host():
        ps.paint(*[h.numpy() for h in host])
        return ps.power()

    for _ in range(args.warmup):
        res = step_device()
    stage = ps.stage_ms()
    # ---- value: device-resident inputs
    barrier(world)
    torch.cuda.synchronize()
    launches0 = ps.kernel_launches()
    with ClockSampler(local) as clk, torch.cuda.stream(ts):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        ev0.record(ts)
        for _ in range(args.steps):
            res = step_device()
        ev1.record(ts)
        torch.cuda.synchronize()
        wall = (time.perf_counter() - t0) * 1e3
    launches = ps.kernel_launches() - launches0
    # stage times and the tile-deposit kernel's time, from the library's CUDA events on the same
    # stream, in a separate pass (each read synchronises)
    stage_acc, tile_acc, nsamp = np.zeros(3), 0.0, max(3, min(args.steps, 10))
    for _ in range(nsamp):
        step_device()
        stage_acc += np.array(ps.stage_ms())
        tile_acc += ps.tile_kernel_ms()[0]
    tile_records = ps.tile_kernel_ms()[1]
    dev_ms = ev0.elapsed_time(ev1)
    total_ms = max(dev_ms, 0.0)
    total_ms = max_over_ranks(world, total_ms, dev)
    barrier(world)
    ms_per = total_ms / (args.steps * world)
    stage_ms = stage_acc / nsamp
    tile_ms = tile_acc / nsamp
    # ---- e2e: host buffers through the public API, every step copying its catalogue from pinned host
    # memory and reading its sums back. A stream of K evaluations: power_enqueue, the next catalogue's
    # paint (its copy runs while this power stage does), power_result. e2e_sequential: paint + power
    # one after the other (each copy waits for the previous evaluation's result).
    def stream_host(k):
        hs = [h.numpy() for h in host]
        ps.paint(*hs)
        out = None
        for i in range(k):
            ps.power_enqueue()
            if i + 1 < k:
                ps.paint(*hs)
            out = ps.power_result()
        return out

    def timed_host(run):
        barrier(world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        run()
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) * 1e3
        return max_over_ranks(world, ms, dev) / (args.steps * world)

    for _ in range(2):
        step_host()
    stream_host(2)
    e2e_seq_ms = timed_host(lambda: [step_host() for _ in range(args.steps)])
    e2e_ms = timed_host(lambda: stream_host(args.steps))
    h2d = sum(int(h.numel() * h.element_size()) for h in host)
    d2h = 3 * 5 * PARAMS["NK"] * 8
    # ---- adjoint (C3 workload): the same particles, density multipoles on a 256^3 TSC grid
    try:
        adj = adjoint_timing(d, ts, local, steps=3, warmup=1)
    except cg.CapowError as e:  # pragma: no cover
        adj = {"error": str(e)}
    # ---- FP64 GPU path on the same workload (fewer steps: it is the slow baseline)
    ps.close()
    fp64_ms = None
    acc = None
    r64 = None
    try:
        p64 = cg.PowerSpectrum(params, precision="fp64", spectra=["dd", "dp", "pp"], device=local, stream=sh)
        p64.paint(*d)
        r64 = p64.power()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        k64 = max(1, min(3, args.steps))
        e0.record(ts)
        for _ in range(k64):
            p64.paint(*d)
            r64 = p64.power()
        e1.record(ts)
        torch.cuda.synchronize()
        fp64_ms = e0.elapsed_time(e1) / k64
        p64.close()
        # accuracy of the FP32-mixed bins against the FP64 GPU path (itself checked against the oracle)
        acc = {}
        m = np.asarray(r64[0]["Nmodes"]) > 0
        for q, name in enumerate(("dd", "dp", "pp")):
            n0 = np.abs(r64[q]["Pk0"]) if name != "dp" else np.sqrt(np.abs(r64[0]["Pk0"] * r64[2]["Pk0"]))
            acc[name] = {f"l{l}": float(np.max((2 * l + 1) * np.abs(res[q][f"Pk{l}"][m] - r64[q][f"Pk{l}"][m])
                                               / n0[m])) for l in (0, 2, 4)}
            acc[name]["nmodes_equal"] = bool(np.array_equal(res[q]["Nmodes"], r64[q]["Nmodes"]))
    except cg.CapowError as e:  # pragma: no cover
        fp64_ms = None
        acc = {"error": str(e)}
    ng = 512 ** 3
    nc = 512 * 512 * 257
    B32 = algorithmic_bytes(n, ng, nc, 4, 16, 4, 8)
    B64 = algorithmic_bytes(n, ng, nc, 4, 32, 8, 16)
    pk = peaks()
    return {
        "ms_per": ms_per, "wall_ms": wall, "stage_ms": stage_ms, "launches": launches, "e2e_ms": e2e_ms,
        "e2e_seq_ms": e2e_seq_ms, "h2d": h2d,
        "d2h": d2h, "fp64_ms": fp64_ms, "acc": acc, "B32": B32, "B64": B64, "peaks": pk, "clocks": clk.summary(),
        "n": n, "parts": parts, "adjoint": adj, "tile_ms": tile_ms, "tile_records": tile_records,
        "res": res, "r64": r64,
    }


ADJOINT_WORKLOAD = "same 16,777,216 particles, TSC 256^3, interlaced, LOS=z, loss sum_l (P_l)^2, l=0,2"


def adjoint_timing(d, ts, local, steps, warmup):
    """The adjoint workload (C3): the headline particles d (device tensors x, y, z, v_los) painted on a 256^3
    TSC grid, density multipoles, loss sum over l = 0, 2 of (P_l)^2. Forward (paint + power) and
    capow_backward are timed separately with CUDA events on the context's stream ts; medians in ms."""
    import torch

    import capow_gb300 as cg

    p3 = cg.Params(**dict(PARAMS, NX=256, NY=256, NZ=256, NK=80, Maxk=0.8))
    with cg.PowerSpectrum(p3, precision="fp32", device=local, stream=ts.cuda_stream) as pa:
        gbuf = {k: torch.empty_like(d[0]) for k in ("dx", "dy", "dz", "dvlos", "dw")}
        torch.cuda.synchronize()
        fw, bw = [], []
        for it in range(warmup + steps):
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(ts)
            pa.paint(*d)
            r3 = pa.normalise(pa.power()[0])
            e1.record(ts)
            pa.backward({"Pk0": 2 * r3["Pk0"], "Pk2": 2 * r3["Pk2"]}, out=gbuf)
            e2.record(ts)
            torch.cuda.synchronize()
            if it >= warmup:
                fw.append(e0.elapsed_time(e1))
                bw.append(e1.elapsed_time(e2))
    return {"workload": ADJOINT_WORKLOAD, "forward_ms": round(statistics.median(fw), 3),
            "backward_ms": round(statistics.median(bw), 3)}


def adjoint_bench(args):
    """The adjoint workload alone, for timing and profiler captures of capow_backward: one JSON line."""
    import torch

    dev = torch.device("cuda", 0)
    x, y, z, vx, vy, vz = make_particles()
    d = [torch.from_numpy(a).to(dev) for a in (x, y, z, vz)]
    ts = torch.cuda.Stream(device=dev)
    adj = adjoint_timing(d, ts, 0, args.steps, args.warmup)
    line = {"metric": "ms per capow_backward (adjoint of paint + power + normalise)", "value": adj["backward_ms"],
            "unit": "ms", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": False,
            "dtype": "f32", "data": "synthetic (seeded Zel'dovich lattice, float32 positions/velocities)",
            "config": {"workload": ADJOINT_WORKLOAD}, "forward_ms": adj["forward_ms"]}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=1)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--fft-path", default="auto", choices=["auto", "3d", "one_launch"],
                    help="FFT path of the FP32 context (capow_options.fft_path)")
    ap.add_argument("--batch", action="store_true", help="run the batched-mocks workload instead (mocks/s)")
    ap.add_argument("--mocks", type=int, default=256)
    ap.add_argument("--scale", action="store_true", help="run the 1024^3 / 134M-particle workload instead")
    ap.add_argument("--survey", action="store_true", help="run the survey-estimator workload instead")
    ap.add_argument("--cli", action="store_true", help="time the capow driver end to end instead")
    ap.add_argument("--adjoint", action="store_true", help="time capow_backward on the adjoint workload instead")
    ap.add_argument("--profile-case", action="store_true",
                    help="run the 8x smaller workload for profiler captures (prints stage times only)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.profile_case:
        profile_case(args)
        return
    if args.batch:
        batch_bench(args)
        return
    if args.scale:
        scale_bench(args)
        return
    if args.survey:
        survey_bench(args)
        return
    if args.cli:
        cli_bench(args)
        return
    if args.adjoint:
        adjoint_bench(args)
        return
    world, rank, local = dist_init()
    log = (lambda *a: print(*a, file=sys.stderr, flush=True))

    if args.impl == "reference":
        if rank != 0:
            return
        parts = make_particles()
        cpu = cpu_reference(args.steps, args.warmup, parts, log)
        line = {"metric": METRIC, "value": round(cpu["value"], 1), "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(cpu["value"], 1),
                "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded Zel'dovich lattice, float32 positions/velocities)",
                "config": config_dict(len(parts[0])), "impl": "reference",
                "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample", "nproc", "cpu_model")},
                "e2e": {"value": round(cpu["value"], 1), "unit": UNIT, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0},
                "runs_ms": cpu["runs_ms"], "wall_ms": cpu["wall_ms"]}
        print(json.dumps(line), flush=True)
        return

    r = gpu_bench(args, world, rank, local)
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu:
        cpu = cpu_reference(args.cpu_steps, 0, r["parts"], log)
    pk = r["peaks"]
    eval_gbs = r["B32"] / (r["ms_per"] * world * 1e-3) / 1e9
    paint_ms, fft_ms, bin_ms = [float(v) for v in r["stage_ms"]]
    line = {
        "metric": METRIC, "value": round(r["ms_per"], 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(r["ms_per"] * world, 4), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Zel'dovich lattice, float32 positions/velocities)",
        "config": config_dict(r["n"]),
        "precision": PRECISION,
        "e2e": {"value": round(r["e2e_ms"], 4), "unit": UNIT, "h2d_bytes_per_step": r["h2d"],
                "d2h_bytes_per_step": r["d2h"],
                "mode": "stream of host catalogues: capow_power_enqueue, next capow_paint, capow_power_result"},
        "e2e_sequential": {"value": round(r["e2e_seq_ms"], 4), "unit": UNIT,
                           "mode": "capow_paint then capow_power per catalogue"},
        "gpu_launches": int(r["launches"]),
        "stages_ms": {"paint": round(paint_ms, 4), "fft": round(fft_ms, 4), "bin": round(bin_ms, 4)},
        "roofline": None,
        "roofline_eval": {"bound": "hbm", "achieved": round(eval_gbs, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
                          "frac": round(eval_gbs / pk["hbm_gbs"], 4), "algorithmic_bytes": r["B32"],
                          "peak_source": pk["source"]},
        "fp64_gpu": {"ms": round(r["fp64_ms"], 3) if r["fp64_ms"] else None, "algorithmic_bytes": r["B64"]},
        "accuracy_fp32_vs_fp64_gpu": r["acc"],
        "adjoint_c3": r["adjoint"],
        "clocks": r["clocks"],
        "cpu_baseline": ({k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample", "nproc", "cpu_model")}
                         if cpu else None),
    }
    if cpu:  # the same particles through the oracle: the headline's error against the reference's algorithm
        line["accuracy_vs_oracle"] = {"fp32": accuracy_vs_oracle(r["res"], cpu["raw"])}
        if r["r64"]:
            line["accuracy_vs_oracle"]["fp64"] = accuracy_vs_oracle(r["r64"], cpu["raw"])
    # the two largest kernels, each timed by the library's CUDA events on the context stream:
    # k_tile_rec (the FP32 tile deposit; events around its one launch) and k_xfft_bin (x-axis FFT
    # fused with the binning: the whole "bin" stage). "roofline" is the one that took longer.
    # k_tile_rec algorithmic bytes per launch: the four grids written once (NX NY NZ cells, 4 bytes)
    # plus one read of its particle records (16 bytes each; one record per particle and tile its
    # stencils reach). k_xfft_bin: one read of the four (y,z)-transformed grids. Traffic: DRAM read
    # + write of one ncu capture of each at this workload.
    alg_t = 4 * 512 ** 3 * 4 + 16 * int(r["tile_records"])
    alg_x = 4 * 512 * 512 * 257 * 8
    rl = {}
    for name, alg, ms, traffic in (("k_tile_rec", alg_t, r["tile_ms"], TRAFFIC_TILE_REC),
                                   ("k_xfft_bin", alg_x, bin_ms, TRAFFIC_XFFT_BIN)):
        ach = alg / (ms * 1e-3) / 1e9
        rl[name] = {"bound": "hbm", "kernel": name, "achieved": round(ach, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
                    "frac": round(ach / pk["hbm_gbs"], 4), "traffic": traffic, "algorithmic_bytes": alg,
                    "ms_per_launch": round(ms, 4), "peak_source": pk["source"]}
    rl["k_tile_rec"]["records"] = int(r["tile_records"])
    line["roofline"] = max(rl.values(), key=lambda v: v["ms_per_launch"])
    line["roofline_by_kernel"] = rl
    # the paint stage (five kernels; k_tile_rec dominates) against the same peak
    pbytes = r["n"] * 16 + 4 * 512 * 512 * 514 * 4
    line["roofline_paint"] = {"achieved": round(pbytes / (paint_ms * 1e-3) / 1e9, 1), "unit": "GB/s",
                              "frac": round(pbytes / (paint_ms * 1e-3) / 1e9 / pk["hbm_gbs"], 4),
                              "algorithmic_bytes": pbytes}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
