"""Shared helpers for parity tests: run the GPU path and the CPU oracle on the same inputs and
compare with the tolerances the path is held to.

Tolerances (raw bin sums, per k bin with modes):
  * l = 0 : |dP0| / (P0_ref + shot/norm) <= tol0   -- equals the relative error of the raw sum
  * l = 2,4 (and 1, 3): (2l+1) |dRaw_l| / Raw0_ref <= tol2
  * cross spectra are normalised by sqrt(Raw0_dd * Raw0_pp) of the same bin
  * mode counts: bit-exact
FP32-mixed: tol0 = 1e-4, tol2 = 1e-3 (the benchmark spec's bound). FP64: 1e-10 for both.
"""
from __future__ import annotations

import numpy as np

import capow_gb300 as cg
import oracle as orc

TOL = {"fp64": (1e-10, 1e-10), "fp32": (1e-4, 1e-3), "det": (1e-4, 1e-3)}


def params_pair(**kw):
    return orc.Params(**kw), cg.Params(**kw)


def vlos_of(los, vx, vy, vz):
    return vx if los == 1 else (vy if los == 2 else vz)


def particles(p, n, seed, edges=True, dtype=np.float64):
    """Uniform particles plus planted edge cases (nodes, half cells, box faces)."""
    rng = np.random.default_rng(seed)
    lo = np.array([p.XMIN, p.YMIN, p.ZMIN])
    hi = np.array([p.XMAX, p.YMAX, p.ZMAX])
    N = np.array([p.NX, p.NY, p.NZ])
    d = (hi - lo) / N
    pos = rng.uniform(lo[:, None], hi[:, None], size=(3, n))
    if edges and n >= 64:
        m = n // 16
        for a in range(3):
            pos[a, a * m:(a + 1) * m] = lo[a] + d[a] * rng.integers(0, N[a], m)               # nodes
            pos[a, (a + 3) * m:(a + 4) * m] = lo[a] + d[a] * (rng.integers(0, N[a], m) + 0.5)  # half cells
        pos[0, 6 * m:6 * m + 4] = lo[0]
        pos[1, 6 * m + 4:6 * m + 8] = np.nextafter(hi[1], lo[1])
        pos[2, 6 * m + 8:6 * m + 12] = lo[2] + 0.5 * d[2]
        pos[0, 6 * m + 12:6 * m + 16] = lo[0] + d[0]
        if p.LOS == 0:
            pos[0, 6 * m + 16:6 * m + 18] = hi[0]
    vel = rng.normal(0.0, 300.0, size=(3, n))
    if dtype == np.float32:
        pos = pos.astype(np.float32)
        # keep float32 positions inside the box for LOS == 0 (the reference aborts otherwise)
        for a in range(3):
            pos[a] = np.minimum(pos[a], np.float32(hi[a]) if np.float32(hi[a]) <= hi[a] else np.nextafter(
                np.float32(hi[a]), np.float32(0)))
            pos[a] = np.maximum(pos[a], np.float32(lo[a]) if np.float32(lo[a]) >= lo[a] else np.nextafter(
                np.float32(lo[a]), np.float32(hi[a])))
        vel = vel.astype(np.float32)
    return pos[0], pos[1], pos[2], vel[0], vel[1], vel[2]


def oracle_run(po, parts, momentum):
    """Full oracle pipeline; ``painted`` holds the grids after the halo fold, before the mean
    subtraction and the FFT (the run's own ``grids`` are transformed in place)."""
    x, y, z, vx, vy, vz = [np.asarray(a, dtype=np.float64) for a in parts]
    out = orc.run(po, x, y, z, vx, vy, vz, momentum=momentum)
    out["painted"] = orc.paint(po, x, y, z, vx, vy, vz, momentum=momentum)[0]
    return out


def gpu_run(pc, parts, precision, spectra=None, grids=False, fft_path="auto"):
    x, y, z, vx, vy, vz = parts
    v = vlos_of(pc.LOS, vx, vy, vz)
    with cg.PowerSpectrum(pc, precision=precision, spectra=spectra, fft_path=fft_path) as ps:
        ps.paint(x, y, z, v)
        st = ps.stats()
        g = None
        if grids:
            g = {}
            names = ["ddg", "ddg_interlace", "ddg_mom", "ddg_mom_interlace"]
            for which in range(4):
                try:
                    g[names[which]] = ps.grid(which)
                except cg.CapowError:
                    pass
        res = ps.power()
        launches = ps.kernel_launches()
    return res, st, g, launches


def bin_errors(gpu: dict, ref: dict, norm0: np.ndarray, odd: bool):
    """max normalised error per multipole over bins with modes."""
    m = (ref["Nmodes"] > 0) & (norm0 > 0)
    out = {}
    for l in (0, 1, 2, 3, 4):
        if l in (1, 3) and not odd:
            continue
        k = f"Pk{l}"
        e = (2 * l + 1) * np.abs(gpu[k][m] - ref[k][m]) / norm0[m]
        out[l] = float(e.max()) if e.size else 0.0
    return out


def assert_spectrum(gpu, ref, norm0, precision, odd, label=""):
    assert np.array_equal(np.asarray(gpu["Nmodes"], np.int64), np.asarray(ref["Nmodes"], np.int64)), (
        f"{label}: mode counts differ")
    t0, t2 = TOL[precision]
    err = bin_errors(gpu, ref, norm0, odd)
    assert err[0] <= t0, f"{label}: l=0 error {err[0]:.3e} > {t0}"
    for l, e in err.items():
        if l:
            assert e <= t2, f"{label}: l={l} error {e:.3e} > {t2}"
    return err


def assert_shot(gpu: dict, ref: dict, norm0: np.ndarray, precision: str, label=""):
    """Shot noise enters P0 as -Nmodes*shot/(Nmodes*norm): bound its effect on the normalised P0.
    FP64: 1e-12 relative. FP32 paths sum the velocity moments in FP32 per thread (FP64 across
    threads), so the bound is on the l=0 error it causes, a tenth of the l=0 tolerance."""
    ds = abs(gpu["shot"] - ref["shot"])
    if precision == "fp64":
        assert ds <= 1e-12 * abs(ref["shot"]) + 1e-9, f"{label}: shot {gpu['shot']} vs {ref['shot']}"
        return
    m = (np.asarray(ref["raw"]["Nmodes"]) > 0) & (norm0 > 0)
    worst = float(np.max(ds * np.asarray(ref["raw"]["Nmodes"])[m] / norm0[m])) if m.any() else 0.0
    assert worst <= TOL[precision][0] / 10, f"{label}: shot error moves P0 by {worst:.2e}"


def grid_close(g_gpu, g_ref, p, precision, label=""):
    row = 2 * (p.NZ // 2 + 1)
    a = g_gpu.reshape(p.NX, p.NY, row)[:, :, :p.NZ]
    b = g_ref[: p.NX * p.NY * row].reshape(p.NX, p.NY, row)[:, :, :p.NZ]
    scale = max(np.abs(b).max(), 1e-30)
    err = np.abs(a - b).max() / scale
    tol = 1e-12 if precision == "fp64" else 1e-5  # FP32 cells hold cancelling sums of +-w*v*W
    assert err <= tol, f"{label}: grid max error {err:.3e} > {tol}"
    return err
