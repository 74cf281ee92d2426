"""CPU oracle for the CAPOW periodic power-spectrum path (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl
reference`` legs of ``bench.py`` import this package, always as the oracle the results are
compared with or the timed CPU baseline, never as part of the product. The product
(``capow_gb300``) never imports it.

Two oracles live here:

* ``liborc`` -- ``capow_oracle.c``, a plain-C restatement of the reference's periodic
  path (src/read_data.c:32-179, 514-745; src/main.c:106-148, 211-225, 266-271,
  302-468, 1019-1056). It builds on any host, the GPU machine included.
* ``oracle/_ref/capow_ref`` -- the UNMODIFIED reference sources compiled against the
  single-rank MPI / FFTW / GSL stand-ins in ``shims/`` (``Makefile.ref``). It can only
  be built where the reference sources are mounted; it pins the restatement and
  generates the committed golden fixtures.
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
import os
import subprocess
import sys
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liborc.so")
REF_BIN = os.path.join(HERE, "_ref", "capow_ref")
# Where the CAPOW sources are mounted (only where the reference binary is to be built); no default.
REF_SRC_ENV = "CAPOW_REFERENCE_SRC"

_CFLAGS = ["-O2", "-std=gnu99", "-ffp-contract=off", "-fPIC", "-shared", "-Wall", "-Wno-unused-function"]


def build(force: bool = False, ref_src: Optional[str] = None) -> str:
    """Compile liborc.so, and oracle/_ref/capow_ref when the reference sources are given (``ref_src``
    or the CAPOW_REFERENCE_SRC environment variable) and present."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, f) for f in ("capow_oracle.c", "orc_fft.c", "orc_gsl.c")]
    hdrs = [os.path.join(HERE, f) for f in ("capow_oracle.h", "orc_fft.h", "shims/gsl/gsl_spline.h",
                                            "shims/gsl/gsl_integration.h")]
    newest = max(os.path.getmtime(f) for f in srcs + hdrs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        subprocess.check_call(["gcc", *_CFLAGS, "-I", HERE, "-o", LIB, *srcs, "-lm"])
    ref_src = ref_src or os.environ.get(REF_SRC_ENV)
    if ref_src and os.path.isdir(os.path.join(ref_src, "src")):
        subprocess.check_call(
            ["make", "-s", "-f", os.path.join("oracle", "Makefile.ref"), f"REF={ref_src}"],
            cwd=os.path.dirname(HERE),
        )
    return LIB


class OrcParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("xmin", ctypes.c_double), ("xmax", ctypes.c_double),
        ("ymin", ctypes.c_double), ("ymax", ctypes.c_double),
        ("zmin", ctypes.c_double), ("zmax", ctypes.c_double),
        ("interp_order", ctypes.c_int), ("do_interlacing", ctypes.c_int), ("los", ctypes.c_int),
        ("omega_m", ctypes.c_double), ("redshift", ctypes.c_double),
        ("nk", ctypes.c_int), ("nmu", ctypes.c_int), ("output_2d", ctypes.c_int),
        ("output_log", ctypes.c_int), ("odd_multipoles", ctypes.c_int),
        ("mink", ctypes.c_double), ("maxk", ctypes.c_double),
    ]


class OrcStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("nread", "nout", "ngrid", "npv", "nsq", "vr_ave", "vr2_ave", "vr3_ave", "vr4_ave")] + [
        ("fatal", ctypes.c_int)]


@dataclasses.dataclass
class Params:
    """The periodic-path subset of the reference's run_parameters.dat tags (src/read_params.c:65-227)."""
    NX: int = 32
    NY: int = 32
    NZ: int = 32
    XMIN: float = 0.0
    XMAX: float = 1000.0
    YMIN: float = 0.0
    YMAX: float = 1000.0
    ZMIN: float = 0.0
    ZMAX: float = 1000.0
    InterpOrder: int = 2
    DoInterlacing: int = 1
    NK: int = 20
    NMU: int = 4
    Mink: float = 0.0
    Maxk: float = 0.2
    Output2D: int = 0
    OutputLog: int = 0
    Omega_m: float = 0.3089
    Redshift: float = 0.1
    LOS: int = 0
    Momentum: int = 0
    Odd_Multipoles: int = 0
    # survey-mode tags (src/read_params.c:65-227); the periodic path ignores them
    Periodic: int = 1
    Coord_Type: int = 0
    X_Origin: float = 0.0
    Y_Origin: float = 0.0
    Z_Origin: float = 0.0
    REDMININ: float = 0.0
    REDMAXIN: float = 1.0
    NOBJ_Max: int = 1
    NBAR_Column: int = -1
    SkyArea: float = 1.0
    FKP_Column: int = -1
    FKP_Pk: float = 0.0
    FKP_Pk_mom: float = 0.0
    FKP_Pk_cross: float = 0.0

    def to_c(self) -> OrcParams:
        return OrcParams(self.NX, self.NY, self.NZ, self.XMIN, self.XMAX, self.YMIN, self.YMAX, self.ZMIN,
                         self.ZMAX, self.InterpOrder, self.DoInterlacing, self.LOS, self.Omega_m, self.Redshift,
                         self.NK, self.NMU, self.Output2D, self.OutputLog, self.Odd_Multipoles, self.Mink, self.Maxk)

    def write_file(self, path: str) -> None:
        """Write a complete run_parameters.dat (all 41 tags the reference parser requires)."""
        tags = dict(
            NumFilesInParallel=1, NX=self.NX, NY=self.NY, NZ=self.NZ,
            XMIN=repr(float(self.XMIN)), XMAX=repr(float(self.XMAX)), YMIN=repr(float(self.YMIN)),
            YMAX=repr(float(self.YMAX)), ZMIN=repr(float(self.ZMIN)), ZMAX=repr(float(self.ZMAX)),
            DoInterlacing=self.DoInterlacing, InterpOrder=self.InterpOrder, NK=self.NK, NMU=self.NMU,
            Output2D=self.Output2D, OutputLog=self.OutputLog, Mink=repr(float(self.Mink)),
            Maxk=repr(float(self.Maxk)), Omega_m=repr(float(self.Omega_m)), Redshift=repr(float(self.Redshift)),
            Periodic=self.Periodic, LOS=self.LOS, Survey=0 if self.Periodic else 1, Momentum=self.Momentum,
            X_Origin=repr(float(self.X_Origin)), Y_Origin=repr(float(self.Y_Origin)),
            Z_Origin=repr(float(self.Z_Origin)), REDMININ=repr(float(self.REDMININ)),
            REDMAXIN=repr(float(self.REDMAXIN)), NOBJ_Max=self.NOBJ_Max, Coord_Type=self.Coord_Type, x_Column=1,
            y_Column=2, z_Column=3, NBAR_Column=self.NBAR_Column, SkyArea=repr(float(self.SkyArea)),
            FKP_Column=self.FKP_Column, FKP_Pk=repr(float(self.FKP_Pk)),
            FKP_Pk_mom=repr(float(self.FKP_Pk_mom)), FKP_Pk_cross=repr(float(self.FKP_Pk_cross)),
            Odd_Multipoles=self.Odd_Multipoles,
        )
        with open(path, "w") as f:
            f.write("% CAPOW run parameters\n")
            for k, v in tags.items():
                f.write(f"{k:<20s} {v}\n")


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        P = ctypes.POINTER(OrcParams)
        L.orc_grid_doubles.restype = ctypes.c_int64
        L.orc_grid_doubles.argtypes = [P]
        L.orc_slice_doubles.restype = ctypes.c_int64
        L.orc_slice_doubles.argtypes = [P]
        L.orc_paint.restype = ctypes.c_int
        L.orc_paint.argtypes = [P, ctypes.c_int, ctypes.c_int64] + [dp] * 11 + [ctypes.POINTER(OrcStats)]
        L.orc_shot_norm.argtypes = [P, ctypes.c_int, ctypes.POINTER(OrcStats), dp, dp, dp]
        L.orc_subtract_mean.argtypes = [P, ctypes.c_int, ctypes.c_double, dp, dp]
        L.orc_fft_grids.argtypes = [P, ctypes.c_int, dp, dp, dp, dp]
        L.orc_compute_power.argtypes = [P, ctypes.c_int, dp, dp, dp, dp, dp, dp, dp, dp, dp, ip, dp, ip]
        L.orc_normalise.restype = ctypes.c_int
        L.orc_normalise.argtypes = [P, ctypes.c_double, ctypes.c_double, dp, dp, dp, dp, dp, ip, dp, ip]
        L.orc_kbin.restype = ctypes.c_int
        L.orc_kbin.argtypes = [P, ctypes.c_double]
        L.orc_fft_r2c_3d_inplace.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
        L.orc_fft_c2c_1d.argtypes = [ctypes.c_int, dp, dp]
        L.orc_fft_c2r_3d_inplace.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
        _lib = L
    return _lib


def _dp(a: Optional[np.ndarray]):
    if a is None:
        return ctypes.cast(None, ctypes.POINTER(ctypes.c_double))
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a: Optional[np.ndarray]):
    if a is None:
        return ctypes.cast(None, ctypes.POINTER(ctypes.c_int))
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def has_mom_grid(momentum: int) -> bool:
    return momentum not in (0, 2, 5)


def paint(p: Params, x, y, z, vx, vy, vz, w=None, momentum: Optional[int] = None):
    """Paint particles as the reference's periodic reader does. Returns (grids dict, stats dict).

    Grids are the padded [NX+InterpOrder][NY][2(NZ/2+1)] float64 arrays after the halo fold.
    """
    L = lib()
    m = p.Momentum if momentum is None else momentum
    pc = p.to_c()
    nd = L.orc_grid_doubles(ctypes.byref(pc))
    g = {"ddg": np.zeros(nd)}
    if p.DoInterlacing:
        g["ddg_interlace"] = np.zeros(nd)
    if has_mom_grid(m):
        g["ddg_mom"] = np.zeros(nd)
        if p.DoInterlacing:
            g["ddg_mom_interlace"] = np.zeros(nd)
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z, vx, vy, vz)]
    wa = None if w is None else np.ascontiguousarray(w, dtype=np.float64)
    st = OrcStats()
    rc = L.orc_paint(ctypes.byref(pc), m, len(arrs[0]), *[_dp(a) for a in arrs], _dp(wa), _dp(g.get("ddg")),
                     _dp(g.get("ddg_interlace")), _dp(g.get("ddg_mom")), _dp(g.get("ddg_mom_interlace")),
                     ctypes.byref(st))
    stats = {f: getattr(st, f) for f, _ in OrcStats._fields_}
    if rc != 0:
        raise ValueError("particle out of grid bounds with LOS == 0 (the reference aborts here)")
    return g, stats


def shot_norm(p: Params, stats: dict, momentum: Optional[int] = None):
    m = p.Momentum if momentum is None else momentum
    st = OrcStats(**{k: v for k, v in stats.items()})
    a, s, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    lib().orc_shot_norm(ctypes.byref(p.to_c()), m, ctypes.byref(st), ctypes.byref(a), ctypes.byref(s),
                        ctypes.byref(n))
    return a.value, s.value, n.value


def compute_power(p: Params, g: dict, momentum: Optional[int] = None):
    """Raw bin sums of src/main.c:302-468 from FFT'd grids."""
    m = p.Momentum if momentum is None else momentum
    NK, NMU = p.NK, p.NMU
    pk = [np.zeros(NK) for _ in range(5)]
    nm = np.zeros(NK, np.int32)
    pk2d = np.zeros(NK * NMU) if p.Output2D else None
    nm2d = np.zeros(NK * NMU, np.int32) if p.Output2D else None
    lib().orc_compute_power(ctypes.byref(p.to_c()), m, _dp(g.get("ddg")), _dp(g.get("ddg_interlace")),
                            _dp(g.get("ddg_mom")), _dp(g.get("ddg_mom_interlace")), *[_dp(a) for a in pk],
                            _ip(nm), _dp(pk2d), _ip(nm2d))
    out = {"Pk0": pk[0], "Pk1": pk[1], "Pk2": pk[2], "Pk3": pk[3], "Pk4": pk[4], "Nmodes": nm}
    if p.Output2D:
        out["Pk_2D"] = pk2d
        out["Nmodes_2D"] = nm2d
    return out


def normalise(p: Params, raw: dict, shot: float, norm: float):
    """src/main.c:1019-1056 on copies of the raw sums; returns (dict, last_zeroed_bin)."""
    o = {k: np.array(v, copy=True) for k, v in raw.items()}
    pk2d = o.get("Pk_2D")
    nm2d = o.get("Nmodes_2D")
    last = lib().orc_normalise(ctypes.byref(p.to_c()), shot, norm, _dp(o["Pk0"]), _dp(o["Pk1"]), _dp(o["Pk2"]),
                               _dp(o["Pk3"]), _dp(o["Pk4"]), _ip(o["Nmodes"]), _dp(pk2d), _ip(nm2d))
    return o, last


def run(p: Params, x, y, z, vx, vy, vz, w=None, momentum: Optional[int] = None, fft=None):
    """The whole periodic branch of main() (src/main.c:75-288) for one Momentum value.

    ``fft`` (optional) replaces the oracle FFT: a callable taking (grid, p) and transforming
    the padded grid in place (e.g. a scipy-backed one for CPU baseline timing)."""
    m = p.Momentum if momentum is None else momentum
    g, st = paint(p, x, y, z, vx, vy, vz, w, momentum=m)
    alpha, shot, norm = shot_norm(p, st, m)
    L = lib()
    pc = p.to_c()
    L.orc_subtract_mean(ctypes.byref(pc), m, alpha, _dp(g["ddg"]), _dp(g.get("ddg_interlace")))
    if fft is None:
        L.orc_fft_grids(ctypes.byref(pc), m, _dp(g.get("ddg")), _dp(g.get("ddg_interlace")), _dp(g.get("ddg_mom")),
                        _dp(g.get("ddg_mom_interlace")))
    else:
        for k in g:
            fft(g[k], p)
    raw = compute_power(p, g, m)
    normed, last = normalise(p, raw, shot, norm)
    return {"raw": raw, "norm": normed, "last": last, "stats": st, "alpha": alpha, "shot": shot, "normf": norm,
            "grids": g}


def fft_r2c_inplace(grid: np.ndarray, nx: int, ny: int, nz: int) -> None:
    lib().orc_fft_r2c_3d_inplace(nx, ny, nz, _dp(grid))


def fft_scipy(grid: np.ndarray, p: Params) -> None:
    """In-place forward r2c of a padded grid with scipy's pocketfft (one thread): the same transform as
    the oracle FFT (sign -1, unnormalised, src/main.c:266-271), several times faster at 512^3."""
    import scipy.fft as sfft

    row = 2 * (p.NZ // 2 + 1)
    a = grid[: p.NX * p.NY * row].reshape(p.NX, p.NY, row)
    c = sfft.rfftn(a[:, :, : p.NZ], workers=1)
    a[:] = c.view(np.float64).reshape(p.NX, p.NY, row)


def _summary(res: dict) -> dict:
    """What a parity check or a timing needs from run(): everything but the grids."""
    return {k: v for k, v in res.items() if k != "grids"}


def _load_particles(path: str):
    d = np.load(path)
    return tuple(np.asarray(d[k], dtype=np.float64) for k in ("x", "y", "z", "vx", "vy", "vz"))


def _run_from_file(args):
    import time

    pdict, path, momentum, use_scipy = args
    parts = _load_particles(path)
    t0 = time.perf_counter()
    res = run(Params(**pdict), *parts, momentum=momentum, fft=fft_scipy if use_scipy else None)
    return _summary(res), time.perf_counter() - t0


def save_particles(path: str, x, y, z, vx, vy, vz) -> None:
    """Write a catalogue for run_parallel (one .npz of the six columns)."""
    np.savez(path, x=x, y=y, z=z, vx=vx, vy=vy, vz=vz)


class ParallelRuns:
    """Single-threaded oracle runs of one catalogue for several Momentum values, one process each, as
    the reference is run once per spectrum (src/main.c:28-298). Processes are started with `spawn`
    (never forked from a process that has used the GPU); a worker that dies raises instead of being
    restarted. Each run() call returns, per Momentum, the run() results without the grids and that
    run's seconds."""

    def __init__(self, nproc: int):
        import concurrent.futures as cf
        import multiprocessing as mp

        build()
        self.pool = cf.ProcessPoolExecutor(max_workers=nproc, mp_context=mp.get_context("spawn"))

    def run(self, p: Params, path: str, momenta, use_scipy: bool = True, timeout: Optional[float] = None):
        pdict = dataclasses.asdict(p)
        return list(self.pool.map(_run_from_file, [(pdict, path, m, use_scipy) for m in momenta], timeout=timeout))

    def close(self):
        self.pool.shutdown(wait=True, cancel_futures=True)

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def real_view(p: Params, grid: np.ndarray) -> np.ndarray:
    """[NX][NY][NZ] view of the FFT region of a padded grid (halo and padding excluded)."""
    row = 2 * (p.NZ // 2 + 1)
    return grid[: p.NX * p.NY * row].reshape(p.NX, p.NY, row)[:, :, : p.NZ]


def complex_view(p: Params, grid: np.ndarray) -> np.ndarray:
    nzc = p.NZ // 2 + 1
    return grid[: p.NX * p.NY * 2 * nzc].view(np.complex128).reshape(p.NX, p.NY, nzc)


# --------------------------------------------------------------------------- reference binary
def ref_available() -> bool:
    return os.path.exists(REF_BIN)


def write_catalogue(path: str, x, y, z, vx, vy, vz) -> None:
    """ASCII catalogue in the reference's `x y z vx vy vz` format with exact round-trip precision."""
    data = np.stack([np.asarray(a, dtype=np.float64) for a in (x, y, z, vx, vy, vz)], axis=1)
    np.savetxt(path, data, fmt="%.17g")


def parse_dump(path: str) -> dict:
    out = {}
    with open(path) as f:
        for line in f:
            parts = line.split()
            if not parts:
                continue
            k, vals = parts[0], parts[1:]
            if k in ("NK", "NMU"):
                out[k] = int(vals[0])
            elif k in ("Nmodes", "Nmodes_2D"):
                out[k] = np.array([int(v) for v in vals], dtype=np.int64)
            else:
                out[k] = np.array([float(v) for v in vals])
    return out


def run_ref_binary(p: Params, workdir: str, x, y, z, vx, vy, vz, grids: bool = False):
    """Run the unmodified reference (oracle/_ref/capow_ref) on one catalogue.

    Returns dict with stdout, output-file text, the raw-sum dump and (optionally) the painted grids."""
    os.makedirs(workdir, exist_ok=True)
    pf, df, of, dump = (os.path.join(workdir, n) for n in ("params.dat", "data.txt", "out.txt", "dump.txt"))
    p.write_file(pf)
    write_catalogue(df, x, y, z, vx, vy, vz)
    for name in ("ddg", "ddg_interlace", "ddg_mom", "ddg_mom_interlace"):
        stale = os.path.join(workdir, f"g.{name}.bin")
        if os.path.exists(stale):
            os.remove(stale)
    for stale in (of, dump, of + "_2D"):
        if os.path.exists(stale):
            os.remove(stale)
    env = dict(os.environ, CAPOW_REF_DUMP=dump)
    if grids:
        env["CAPOW_REF_GRIDS"] = os.path.join(workdir, "g")
    r = subprocess.run([REF_BIN, pf, df, "none", of], capture_output=True, text=True, env=env)
    res = {"returncode": r.returncode, "stdout": r.stdout}
    if os.path.exists(of):
        with open(of) as f:
            res["output"] = f.read()
    if os.path.exists(dump):
        res["dump"] = parse_dump(dump)
    if grids:
        for name in ("ddg", "ddg_interlace", "ddg_mom", "ddg_mom_interlace"):
            fp = os.path.join(workdir, f"g.{name}.bin")
            if os.path.exists(fp):
                res.setdefault("grids", {})[name] = np.fromfile(fp, dtype=np.float64)
    return res


if __name__ == "__main__":  # pragma: no cover
    build(force="--force" in sys.argv)
    print(LIB)


# --------------------------------------------------------------------------- survey mode
class OrcSurvey(ctypes.Structure):
    _fields_ = [("x_origin", ctypes.c_double), ("y_origin", ctypes.c_double), ("z_origin", ctypes.c_double)]


def _survey_lib():
    L = lib()
    if not getattr(L, "_survey_bound", False):
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        P = ctypes.POINTER(OrcParams)
        L.orc_survey_assign.restype = ctypes.c_double
        L.orc_survey_assign.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int64, dp, dp, dp, dp, dp, dp,
                                        ctypes.c_double, dp, dp, dp, dp]
        L.orc_survey_power.argtypes = [P, ctypes.POINTER(OrcSurvey), ctypes.c_int, dp, dp, dp, dp, dp, dp, dp, dp,
                                       dp, ip]
        L.orc_survey_redshift.restype = ctypes.c_double
        L.orc_survey_redshift.argtypes = [ctypes.c_double, ctypes.c_double]
        L.orc_survey_distance.restype = ctypes.c_double
        L.orc_survey_distance.argtypes = [ctypes.c_double, ctypes.c_double]
        L.orc_cspline_eval.restype = ctypes.c_double
        L.orc_cspline_eval.argtypes = [ctypes.c_int, dp, dp, ctypes.c_double]
        L._survey_bound = True
    return L


def _seqsum(a) -> float:
    """Left-to-right double sum, as the reference's loops add (numpy's sum is pairwise)."""
    a = np.asarray(a, dtype=np.float64)
    return float(np.cumsum(a)[-1]) if a.size else 0.0


def survey_read(p: Params, path: str, randoms: bool) -> dict:
    """read_survey_serial_ascii (src/read_data.c:184-361) with the number density from its column
    (NBAR_Column > 0): data lines hold 12 numbers, randoms 8; the weight is the 4th, the number density the
    5th (the reader copies that column into nbar, :244-250). Cartesian input (Coord_Type 0) takes the
    redshift from the distance table's inverse at |x| (:259-266); angular input (Coord_Type 1: RA and Dec in
    degrees, 2: in radians) reads the redshift as the third number, skips objects of zero weight and places
    the rest at the table's distance r(z) along the direction (:267-291). Objects whose redshift lies outside
    [REDMININ, REDMAXIN] are dropped; an object outside the grid less the interpolation margin is the
    reference's fatal error (:293-299)."""
    L = _survey_lib()
    a = np.loadtxt(path, comments="#", ndmin=2)
    need = 8 if randoms else 12
    if a.shape[1] < need:
        raise ValueError(f"survey catalogue {path} has {a.shape[1]} columns, the reference reads {need}")
    dx, dy, dz = (p.XMAX - p.XMIN) / p.NX, (p.YMAX - p.YMIN) / p.NY, (p.ZMAX - p.ZMIN) / p.NZ
    xlo, xhi = p.XMIN + (p.InterpOrder - 1) * dx, p.XMAX - (p.InterpOrder - 1) * dx
    ylo, yhi = p.YMIN + (p.InterpOrder - 1) * dy, p.YMAX - (p.InterpOrder - 1) * dy
    zlo, zhi = p.ZMIN + (p.InterpOrder - 1) * dz, p.ZMAX - (p.InterpOrder - 1) * dz
    if p.DoInterlacing:
        xhi -= 0.5 * dx
        yhi -= 0.5 * dy
        zhi -= 0.5 * dz
    keep = []
    red = []
    pos = []
    for i in range(a.shape[0]):
        tx, ty, tz = float(a[i, 0]), float(a[i, 1]), float(a[i, 2])
        if p.Coord_Type == 0:
            tred = L.orc_survey_redshift(p.Omega_m, math.sqrt(tx * tx + ty * ty + tz * tz))
            if tred < p.REDMININ or tred > p.REDMAXIN:
                continue
        else:
            tred = tz
            if tred < p.REDMININ or tred > p.REDMAXIN or a[i, 3] == 0.0:
                continue
            tdist = L.orc_survey_distance(p.Omega_m, tred)
            ra, dec = (tx * (math.pi / 180.0), ty * (math.pi / 180.0)) if p.Coord_Type == 1 else (tx, ty)
            tx = tdist * math.cos(dec) * math.cos(ra)
            ty = tdist * math.cos(dec) * math.sin(ra)
            tz = tdist * math.sin(dec)
        if tx < xlo or tx >= xhi or ty < ylo or ty >= yhi or tz < zlo or tz >= zhi:
            raise ValueError(f"object out of grid bounds for chosen InterpOrder: x={tx}, y={ty}, z={tz}")
        keep.append(i)
        red.append(tred)
        pos.append((tx, ty, tz))
    # the reference keeps each object in float fields (struct survey_data, src/vars.h:136-142)
    k = np.array(keep, dtype=np.int64)
    f32 = np.float32
    xyz = np.array(pos, dtype=np.float64).reshape(-1, 3)
    out = {"x": xyz[:, 0].astype(f32), "y": xyz[:, 1].astype(f32), "z": xyz[:, 2].astype(f32),
           "weight": a[k, 3].astype(f32), "redshift": np.array(red).astype(f32), "nread": a.shape[0],
           "redmin": min(red, default=1.0e30), "redmax": max(red, default=-1.0e30)}  # REDMIN/REDMAX, :327-328
    out["nbar"] = a[k, 4].astype(f32) if p.NBAR_Column > 0 else np.zeros(len(k), f32)
    if p.Momentum:  # :308-316; a random line carries no log-distance (its pv is never used), only the error
        q = 3.0 / 2.0 * p.Omega_m - 1.0
        tr = np.array(red, dtype=np.float64)
        zmod = tr * (1.0 + 0.5 * (1.0 - q) * tr - 1.0 / 6.0 * (2.0 - q - 3.0 * q * q) * tr * tr)
        logdist = np.zeros(len(k)) if randoms else a[k, 6]
        logdist_err = a[k, 6] if randoms else a[k, 7]
        out["pv"] = (299792.458 * zmod * np.log(10.0) * logdist / (1.0 + zmod)).astype(f32)
        out["pverr"] = (299792.458 * zmod * np.log(10.0) * logdist_err / (1.0 + zmod)).astype(f32)
    else:
        out["pv"] = out["pverr"] = np.zeros(len(k), f32)
    out["weight_pv"] = np.zeros(len(k), f32)
    return out


def survey_nbar(p: Params, data: dict, rand: dict) -> list:
    """compute_nbar (src/read_data.c:385-446, one rank) in place on both catalogues' float nbar: counts of
    the first NDATA randoms' redshifts (the reference indexes the randoms with the data's count, :401-405)
    in ceil((REDMAXIN - REDMININ) / 0.002) bins over [REDMIN, REDMAX] of both catalogues, over each bin's
    shell volume (SkyArea square degrees, distances from the table's r(z) spline), then a natural cubic
    spline through the bin centres with the raw end values half a bin outside. Returns the printed lines."""
    L = _survey_lib()
    nbins = int(np.ceil((p.REDMAXIN - p.REDMININ) / 0.002))
    redmin = min(data["redmin"], rand["redmin"])
    redmax = max(data["redmax"], rand["redmax"])
    rbw = (redmax - redmin) / float(np.float32(nbins))
    znbar = np.zeros(nbins + 2)
    nbar = np.zeros(nbins + 2)
    lines = ["Calculating Number Density..."]
    for i in range(len(data["x"])):
        nb = int(np.floor((float(rand["redshift"][i]) - redmin) / rbw)) + 1
        if nb == nbins + 1:
            nb -= 1
        nbar[nb] += 1.0
    for i in range(nbins):
        outer = L.orc_survey_distance(p.Omega_m, (i + 1) * rbw + redmin)
        inner = L.orc_survey_distance(p.Omega_m, i * rbw + redmin)
        volume = p.SkyArea / (180.0 * 180.0) * np.pi * np.pi * (outer * outer * outer - inner * inner * inner) / 3.0
        znbar[i + 1] = (i + 0.5) * rbw + redmin
        nbar[i + 1] /= volume
        lines.append("%12.6f, %12.6f" % (znbar[i + 1], nbar[i + 1]))
    znbar[0] = redmin - 0.5 * rbw
    znbar[nbins + 1] = redmax + 0.5 * rbw
    for c in (data, rand):
        c["nbar"] = np.array([L.orc_cspline_eval(nbins + 2, _dp(znbar), _dp(nbar), float(z)) for z in c["redshift"]],
                             dtype=np.float64).astype(np.float32)
    return lines


def survey_fkp(p: Params, cat: dict) -> None:
    """compute_fkp (src/read_data.c:450-466) in place, products in double and results stored back in the float
    fields. Momentum 0: w *= 1/(1 + nbar FKP_Pk). Momentum 1: w *= 1/((pverr^2 + 300^2) + nbar FKP_Pk_mom), with
    pverr^2 a float product. Momentum 2, 3: the density and velocity weights, both times the cross factor
    1/sqrt(1 + w_d w_v nbar^2 FKP_Pk_cross^2), into weight and weight_pv."""
    f32 = np.float32
    w = cat["weight"].astype(np.float64)
    nb = cat["nbar"].astype(np.float64)
    pe2 = (cat["pverr"] * cat["pverr"]).astype(np.float64)  # float * float
    if p.Momentum == 0:
        cat["weight"] = (w * (1.0 / (1.0 + nb * p.FKP_Pk))).astype(f32)
    elif p.Momentum == 1:
        cat["weight"] = (w * (1.0 / ((pe2 + 300.0 * 300.0) + nb * p.FKP_Pk_mom))).astype(f32)
    else:
        tw = 1.0 / (1.0 + nb * p.FKP_Pk)
        twpv = 1.0 / ((pe2 + 300.0 * 300.0) + nb * p.FKP_Pk_mom)
        twc = 1.0 / np.sqrt(1.0 + tw * twpv * nb * nb * p.FKP_Pk_cross * p.FKP_Pk_cross)
        cat["weight_pv"] = (w * twpv * twc).astype(f32)
        cat["weight"] = (w * (tw * twc)).astype(f32)


def survey_run(p: Params, data_path: str, rand_path: str, grids: bool = False) -> dict:
    """The survey branch of main (src/main.c:77-95, 149-204, 226-258, 279-288) for Momentum 0-3: read data and
    randoms, n(z) when NBAR_Column < 0, FKP weights, the sums, alpha, shot and norm of the Momentum, the
    painted grids (data minus alpha randoms; Momentum 1 paints the data's w pv only; Momentum 2, 3 add the
    data's w_pv pv momentum grid), the Yamamoto multipoles, output_power's normalisation."""
    L = _survey_lib()
    m = p.Momentum
    data = survey_read(p, data_path, False)
    rand = survey_read(p, rand_path, True)
    nbar_lines = survey_nbar(p, data, rand) if p.NBAR_Column < 0 else []
    if p.FKP_Column < 0:
        survey_fkp(p, data)
        survey_fkp(p, rand)
    elif m >= 2:
        raise ValueError("Momentum 2, 3 need the FKP weights: the reference leaves weight_pv unset otherwise")
    # float32 fields: the products below are float products, summed in double, as in C (:151-163)
    wd, wr, nd_, nr_ = data["weight"], rand["weight"], data["nbar"], rand["nbar"]
    data_nbw, data_nbwsq, data_nbsqwsq = _seqsum(wd), _seqsum(wd * wd), _seqsum(wd * wd * nd_)
    data_vr = data_vrsq = data_nbsqwsq_pv = 0.0
    if m:
        wpv, pv = data["weight_pv"], data["pv"]
        data_vr, data_vrsq = _seqsum(wd * wpv * pv), _seqsum(wd * wd * pv * pv)
        data_nbsqwsq_pv = _seqsum(wpv * wpv * nd_)
    rand_nbw, rand_nbwsq, rand_nbsqwsq = _seqsum(wr), _seqsum(wr * wr), _seqsum(wr * wr * nr_)
    rand_nbsqwsq_pv = _seqsum(rand["weight_pv"] * rand["weight_pv"] * nr_) if m == 2 else 0.0
    alpha = data_nbw / rand_nbw
    rand_nbwsq *= alpha * alpha
    rand_nbsqwsq *= alpha
    if m == 0:
        shot, norm = data_nbwsq + rand_nbwsq, rand_nbsqwsq
    elif m == 1:
        shot, norm = data_vrsq, rand_nbsqwsq
    elif m == 2:
        shot, norm = data_vr, float(np.sqrt(rand_nbsqwsq * rand_nbsqwsq_pv))
    else:
        shot, norm = data_vrsq, float(np.sqrt(rand_nbsqwsq * rand_nbsqwsq_pv))
    d64 = {c: {a: v.astype(np.float64) for a, v in cat.items() if isinstance(v, np.ndarray)}
           for c, cat in (("d", data), ("r", rand))}
    pc = p.to_c()
    nd = lib().orc_grid_doubles(ctypes.byref(pc))
    ddg = np.zeros(nd)
    ddgi = np.zeros(nd) if p.DoInterlacing else None
    ddgm = np.zeros(nd) if m >= 2 else None
    ddgmi = np.zeros(nd) if m >= 2 and p.DoInterlacing else None

    def assign(c, is_data, pref):
        a = d64[c]
        return L.orc_survey_assign(ctypes.byref(pc), m, is_data, len(a["x"]), _dp(a["x"]), _dp(a["y"]), _dp(a["z"]),
                                   _dp(a["weight"]), _dp(a["weight_pv"]), _dp(a["pv"]), pref, _dp(ddg), _dp(ddgi),
                                   _dp(ddgm) if is_data else None, _dp(ddgmi) if is_data else None)

    ngrid_d = assign("d", 1, 1.0)
    ngrid_r = assign("r", 0, -alpha) if m != 1 else None  # src/main.c:229
    painted = ({"ddg": ddg.copy(), "ddg_interlace": None if ddgi is None else ddgi.copy(),
                "ddg_mom": None if ddgm is None else ddgm.copy(),
                "ddg_mom_interlace": None if ddgmi is None else ddgmi.copy()} if grids else None)
    NK = p.NK
    pk = [np.zeros(NK) for _ in range(5)]
    nm = np.zeros(NK, np.int32)
    sp = OrcSurvey(p.X_Origin, p.Y_Origin, p.Z_Origin)
    L.orc_survey_power(ctypes.byref(pc), ctypes.byref(sp), m, _dp(ddg), _dp(ddgi), _dp(ddgm), _dp(ddgmi),
                       *[_dp(a) for a in pk], _ip(nm))
    raw = {"Pk0": pk[0], "Pk1": pk[1], "Pk2": pk[2], "Pk3": pk[3], "Pk4": pk[4], "Nmodes": nm}
    with np.errstate(divide="ignore", invalid="ignore"):
        normed, last = normalise(p, raw, shot, norm)
    return {"raw": raw, "norm": normed, "last": last, "alpha": alpha, "shot": shot, "normf": norm,
            "ndata": len(wd), "nrand": len(wr), "ngrid_data": ngrid_d,
            "ngrid_rand": None if ngrid_r is None else ngrid_r / -alpha,
            "sums": {"data_nbw": data_nbw, "data_nbwsq": data_nbwsq, "data_nbsqwsq": data_nbsqwsq,
                     "rand_nbwsq": rand_nbwsq, "rand_nbsqwsq": rand_nbsqwsq, "data_vr": data_vr,
                     "data_vrsq": data_vrsq, "data_nbsqwsq_pv": data_nbsqwsq_pv, "rand_nbsqwsq_pv": rand_nbsqwsq_pv},
            "data": data, "rand": rand, "painted": painted, "nbar_lines": nbar_lines}
