"""GPU parity against the CPU oracle (the reference's algorithm restated in C and pinned to the
unmodified reference): painted grids cell by cell, mode counts bit-exact, P_l within tolerance."""
import itertools

import numpy as np
import pytest

import capow_gb300 as cg
from parity_util import (assert_shot, assert_spectrum, gpu_run, grid_close, oracle_run, params_pair,
                         particles)

pytestmark = pytest.mark.gpu

BASE = dict(XMIN=-3.0, XMAX=997.0, YMIN=0.0, YMAX=1000.0, ZMIN=10.0, ZMAX=510.0, NK=24, Maxk=0.55, NMU=5,
            Odd_Multipoles=1)

CASES = list(itertools.product([1, 2, 3], [0, 3], [0, 1], [0, 1, 2]))


@pytest.mark.parametrize("precision", ["fp64", "fp32", "det"])
@pytest.mark.parametrize("order,los,il,mom", CASES)
def test_reference_run_parity(gpu, precision, order, los, il, mom):
    """One reference run (Momentum 0/1/2) on a 24x20x16 grid: grids and raw sums."""
    po, pc = params_pair(NX=24, NY=20, NZ=16, InterpOrder=order, LOS=los, DoInterlacing=il, Momentum=mom, **BASE)
    parts = particles(po, 3000, seed=100 + order * 10 + los + il * 100 + mom * 1000)
    ref = oracle_run(po, parts, mom)
    res, st, grids, _ = gpu_run(pc, parts, precision, grids=True)
    label = f"{precision} order={order} los={los} il={il} mom={mom}"
    assert st["ngrid"] == ref["stats"]["ngrid"], label
    assert st["nread"] == ref["stats"]["nread"], label
    assert st["nout"] == ref["stats"]["nout"], label
    for k, g in grids.items():
        grid_close(g, ref["painted"][k], po, precision, f"{label} {k}")
    r = res[0]
    assert abs(r["norm"] - ref["normf"]) <= 1e-12 * abs(ref["normf"]), label
    raw = ref["raw"]
    if mom == 1:  # cross spectrum: normalise by sqrt(P_dd P_pp) of the same bin
        dd = oracle_run(po, parts, 0)["raw"]["Pk0"]
        pp = oracle_run(po, parts, 2)["raw"]["Pk0"]
        norm0 = np.sqrt(np.abs(dd * pp))
    else:
        norm0 = np.abs(raw["Pk0"])
    assert_shot(r, ref, norm0, precision, label)
    assert_spectrum(r, raw, norm0, precision, odd=True, label=label)


# Momentum 3-8: the v^2, v^3, v^4 fields (src/read_data.c:103-130), their shot moments (src/main.c:141-148)
# and mean-subtraction rule (src/main.c:211-225); orders and LOS rotate over the runs
MOMENTS = [(m, 1 + (m + k) % 3, los) for m in range(3, 9) for k, los in enumerate((0, 3))]


@pytest.mark.parametrize("precision", ["fp64", "fp32", "det"])
@pytest.mark.parametrize("mom,order,los", MOMENTS)
def test_velocity_moment_runs_parity(gpu, precision, mom, order, los):
    """One reference run for Momentum 3..8 on a 24x20x16 grid: painted grids cell by cell, counters,
    shot noise and raw sums. Several of these spectra have no auto-spectrum run to normalise by, so
    every bin is held to the tolerance relative to the spectrum's largest |P0| sum."""
    po, pc = params_pair(NX=24, NY=20, NZ=16, InterpOrder=order, LOS=los, DoInterlacing=1, Momentum=mom, **BASE)
    parts = particles(po, 3000, seed=900 + mom * 10 + los)
    ref = oracle_run(po, parts, mom)
    res, st, grids, _ = gpu_run(pc, parts, precision, grids=True)
    label = f"{precision} mom={mom} order={order} los={los}"
    for key in ("ngrid", "nread", "nout"):
        assert st[key] == ref["stats"][key], label
    for k, g in grids.items():
        grid_close(g, ref["painted"][k], po, precision, f"{label} {k}")
    r = res[0]
    raw = ref["raw"]
    norm0 = np.full(po.NK, np.abs(raw["Pk0"]).max())
    assert abs(r["norm"] - ref["normf"]) <= 1e-12 * abs(ref["normf"]), label
    assert_shot(r, ref, norm0, precision, label)
    assert_spectrum(r, raw, norm0, precision, odd=True, label=label)


FUSED = [(3, 3, 1, 1, 1, 64, 48, 40), (3, 0, 1, 0, 0, 128, 24, 30), (2, 3, 0, 2, 1, 64, 40, 48),
         (1, 0, 0, 1, 0, 16, 20, 18), (3, 1, 1, 1, 1, 256, 16, 12), (2, 2, 1, 0, 1, 2048, 8, 6),
         # power-of-two NZ: the z axis by k_zr2c into the transposed layout, the y axis by cuFFT C2C
         (3, 3, 1, 1, 1, 64, 48, 32), (2, 0, 1, 2, 0, 32, 20, 64), (1, 1, 0, 0, 1, 16, 12, 128),
         (3, 2, 1, 1, 0, 128, 36, 32), (2, 3, 1, 0, 0, 64, 8, 2048),
         # power-of-two NY and NZ: the z and y axes in one launch (k_zy), NY from 16 to 1024
         (3, 3, 1, 1, 1, 32, 16, 32), (2, 0, 1, 2, 0, 16, 64, 128), (1, 1, 1, 0, 1, 64, 32, 64),
         (3, 2, 1, 1, 0, 16, 1024, 32), (2, 3, 0, 1, 1, 32, 128, 256)]


@pytest.mark.parametrize("precision", ["fp32", "det"])
@pytest.mark.parametrize("order,los,il,mom,odd,nx,ny,nz", FUSED)
def test_fused_x_fft_bin_parity(gpu, precision, order, los, il, mom, odd, nx, ny, nz):
    """Power-of-two NX: the (y, z) axes (cuFFT 2-D, or k_zr2c + cuFFT C2C along y for a power-of-two
    NZ, or with fft_path one_launch and power-of-two NY both in one k_zy launch) + the fused x-axis FFT
    and binning, against the oracle and against the 3-D cuFFT + binning kernel path on the same paint."""
    kw = dict(BASE, Odd_Multipoles=odd)
    po, pc = params_pair(NX=nx, NY=ny, NZ=nz, InterpOrder=order, LOS=los, DoInterlacing=il, Momentum=mom, **kw)
    parts = particles(po, 4000, seed=300 + nx + order * 7 + mom)
    ref = oracle_run(po, parts, mom)
    res, _, _, _ = gpu_run(pc, parts, precision)
    res3, _, _, _ = gpu_run(pc, parts, precision, fft_path="3d")
    res1, _, _, _ = gpu_run(pc, parts, precision, fft_path="one_launch")
    label = f"fused {precision} nx={nx} order={order} los={los} il={il} mom={mom} odd={odd}"
    raw = ref["raw"]
    if mom == 1:
        norm0 = np.sqrt(np.abs(oracle_run(po, parts, 0)["raw"]["Pk0"] * oracle_run(po, parts, 2)["raw"]["Pk0"]))
    else:
        norm0 = np.abs(raw["Pk0"])
    assert_spectrum(res[0], raw, norm0, precision, odd=bool(odd), label=label)
    assert_spectrum(res[0], res3[0], norm0, precision, odd=bool(odd), label=label + " vs 3d")
    assert_spectrum(res1[0], raw, norm0, precision, odd=bool(odd), label=label + " one launch")


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_combined_spectra_equal_three_reference_runs(gpu, precision):
    """dd, dp, pp from one paint equal Momentum 0, 1, 2 reference runs."""
    po, pc = params_pair(NX=32, NY=32, NZ=32, InterpOrder=3, LOS=3, DoInterlacing=1, Momentum=0, **BASE)
    parts = particles(po, 20000, seed=7)
    refs = {m: oracle_run(po, parts, m) for m in (0, 1, 2)}
    res, st, _, _ = gpu_run(pc, parts, precision, spectra=["dd", "dp", "pp"])
    assert [r["kind"] for r in res] == ["dd", "dp", "pp"]
    dd, pp = refs[0]["raw"]["Pk0"], refs[2]["raw"]["Pk0"]
    for r, m, n0 in zip(res, (0, 1, 2), (np.abs(dd), np.sqrt(np.abs(dd * pp)), np.abs(pp))):
        assert_shot(r, refs[m], n0, precision, f"{precision} spec {r['kind']}")
        assert_spectrum(r, refs[m]["raw"], n0, precision, odd=True, label=f"{precision} spec {r['kind']}")


@pytest.mark.parametrize("precision", ["fp64", "fp32", "det"])
def test_float32_input(gpu, precision):
    po, pc = params_pair(NX=32, NY=24, NZ=40, InterpOrder=3, LOS=0, DoInterlacing=1, Momentum=1, **BASE)
    parts = particles(po, 10000, seed=11, dtype=np.float32)
    ref = oracle_run(po, parts, 1)
    res, st, grids, _ = gpu_run(pc, parts, precision, grids=True)
    for k, g in grids.items():
        grid_close(g, ref["painted"][k], po, precision, f"f32 {k}")
    dd = oracle_run(po, parts, 0)["raw"]["Pk0"]
    pp = oracle_run(po, parts, 2)["raw"]["Pk0"]
    assert_spectrum(res[0], ref["raw"], np.sqrt(np.abs(dd * pp)), precision, odd=True, label="f32 input")


def test_output2d_and_log_bins(gpu):
    for log in (0, 1):
        kw = dict(BASE)
        kw.update(Output2D=1, NMU=7, OutputLog=log)
        if log:
            kw.update(Mink=-2.5, Maxk=-0.3)
        po, pc = params_pair(NX=32, NY=32, NZ=32, InterpOrder=2, LOS=1, DoInterlacing=1, Momentum=0, **kw)
        parts = particles(po, 8000, seed=21 + log)
        ref = oracle_run(po, parts, 0)
        for prec in ("fp64", "fp32"):
            res, _, _, _ = gpu_run(pc, parts, prec)
            r = res[0]
            assert np.array_equal(r["Nmodes"], ref["raw"]["Nmodes"])
            assert np.array_equal(r["Nmodes_2D"], ref["raw"]["Nmodes_2D"])
            assert_spectrum(r, ref["raw"], np.abs(ref["raw"]["Pk0"]), prec, odd=True, label=f"log={log} {prec}")
            m = ref["raw"]["Nmodes_2D"] > 0
            e = np.abs(r["Pk_2D"][m] - ref["raw"]["Pk_2D"][m]) / np.abs(ref["raw"]["Pk_2D"][m])
            assert e.max() <= (1e-10 if prec == "fp64" else 1e-3)


def test_deterministic_mode_is_bit_reproducible(gpu):
    po, pc = params_pair(NX=48, NY=48, NZ=48, InterpOrder=3, LOS=3, DoInterlacing=1, Momentum=1, **BASE)
    parts = particles(po, 50000, seed=5)
    a = gpu_run(pc, parts, "det", grids=True)
    b = gpu_run(pc, parts, "det", grids=True)
    for k in a[2]:
        assert np.array_equal(a[2][k], b[2][k]), k


def test_deterministic_dense_tiles(gpu):
    """A clump of 60,000 particles inside two cells: its tiles hold far more than the 8192 records of the
    deterministic kernel's two-limb cells, so they take its uint64 cells at the run's global scale, beside
    ordinary tiles. The grids against the oracle and bit-reproducible."""
    po, pc = params_pair(NX=32, NY=32, NZ=32, InterpOrder=3, LOS=3, DoInterlacing=1, Momentum=1, **BASE)
    x, y, z, vx, vy, vz = particles(po, 20000, seed=9)
    rng = np.random.default_rng(10)
    d = np.array([(po.XMAX - po.XMIN) / po.NX, (po.YMAX - po.YMIN) / po.NY, (po.ZMAX - po.ZMIN) / po.NZ])
    c = np.array([po.XMIN, po.YMIN, po.ZMIN]) + d * np.array([10.3, 17.6, 20.2])
    clump = c[:, None] + rng.uniform(-1.0, 1.0, size=(3, 60000)) * d[:, None]
    parts = (np.r_[x, clump[0]], np.r_[y, clump[1]], np.r_[z, clump[2]], np.r_[vx, rng.normal(0, 300, 60000)],
             np.r_[vy, rng.normal(0, 300, 60000)], np.r_[vz, rng.normal(0, 300, 60000)])
    ref = oracle_run(po, parts, 1)
    a = gpu_run(pc, parts, "det", grids=True)
    b = gpu_run(pc, parts, "det", grids=True)
    for k in a[2]:
        assert np.array_equal(a[2][k], b[2][k]), k
        grid_close(a[2][k], ref["painted"][k], po, "det", f"dense det {k}")


def test_out_of_box_los0_is_an_error(gpu):
    po, pc = params_pair(NX=16, NY=16, NZ=16, InterpOrder=2, LOS=0, DoInterlacing=0, Momentum=0, **BASE)
    x, y, z, vx, vy, vz = particles(po, 100, seed=1, edges=False)
    x = x.copy()
    x[5] = po.XMAX + 1.0
    for prec in ("fp64", "fp32"):
        with cg.PowerSpectrum(pc, precision=prec) as ps:
            ps.paint(x, y, z, vz)
            with pytest.raises(cg.CapowError) as e:
                ps.power()
            assert e.value.status == cg.EBOUNDS


def test_nonfinite_is_an_error(gpu):
    po, pc = params_pair(NX=16, NY=16, NZ=16, InterpOrder=3, LOS=3, DoInterlacing=1, Momentum=1, **BASE)
    x, y, z, vx, vy, vz = particles(po, 100, seed=1, edges=False)
    vz = vz.copy()
    vz[3] = np.nan
    for prec in ("fp64", "fp32"):
        with cg.PowerSpectrum(pc, precision=prec) as ps:
            ps.paint(x, y, z, vz)
            with pytest.raises(cg.CapowError) as e:
                ps.power()
            assert e.value.status == cg.EINVAL


def _clumped(po, n, frac, seed, width):
    """Uniform particles with a fraction packed into a small cube (a few cells wide)."""
    x, y, z, vx, vy, vz = particles(po, n, seed=seed, edges=False)
    rng = np.random.default_rng(seed + 1)
    m = int(n * frac)
    d = (po.XMAX - po.XMIN) / po.NX
    c = np.array([po.XMIN + 0.37 * (po.XMAX - po.XMIN), po.YMIN + 0.41 * (po.YMAX - po.YMIN),
                  po.ZMIN + 0.43 * (po.ZMAX - po.ZMIN)])
    for a, arr in enumerate((x, y, z)):
        arr[:m] = c[a] + rng.uniform(-width / 2, width / 2, m) * d
    return x, y, z, vx, vy, vz


@pytest.mark.parametrize("frac,n", [(0.3, 40000), (0.95, 300000)])
def test_fp32_bucket_overflow_parity(gpu, frac, n):
    """A clump overflows its tiles' buckets: the overflow list (first case) or, when that fills too,
    the fall-back to the two-pass paint (second case) must paint exactly what the oracle paints."""
    po, pc = params_pair(NX=64, NY=64, NZ=64, InterpOrder=3, LOS=3, DoInterlacing=1, Momentum=1, **BASE)
    parts = _clumped(po, n, frac, seed=61 + n, width=3.0)
    ref = oracle_run(po, parts, 1)
    res, st, grids, _ = gpu_run(pc, parts, "fp32", grids=True)
    assert st["ngrid"] == ref["stats"]["ngrid"]
    # an FP32 cell of the clump sums ~n*frac deposits, each rounded at about 2^-24 of the cell (the
    # int32 tile quantum is of the same order): the error grows as sqrt(deposits)
    tol = max(1e-5, 4.0 * 2.0 ** -24 * np.sqrt(n * frac) * 2.0)
    row = 2 * (po.NZ // 2 + 1)
    for k, g in grids.items():
        a = g.reshape(po.NX, po.NY, row)[:, :, :po.NZ]
        b = ref["painted"][k][: po.NX * po.NY * row].reshape(po.NX, po.NY, row)[:, :, :po.NZ]
        err = np.abs(a - b).max() / np.abs(b).max()
        assert err <= tol, f"clump {frac} {k}: {err:.3e} > {tol:.3e}"
    dd = oracle_run(po, parts, 0)["raw"]["Pk0"]
    pp = oracle_run(po, parts, 2)["raw"]["Pk0"]
    assert_spectrum(res[0], ref["raw"], np.sqrt(np.abs(dd * pp)), "fp32", odd=True, label=f"clump {frac}")


def test_tile_kernel_timing(gpu):
    """capow_tile_kernel_ms: the tile-deposit kernel's event time and record count of the last FP32
    paint (every particle has at least one record, at most one per tile its two stencils reach);
    FP64 contexts have no tile kernel."""
    p = cg.Params(NX=64, NY=64, NZ=64, NK=20, Maxk=0.3, XMIN=0.0, XMAX=1000.0, YMIN=0.0, YMAX=1000.0,
                  ZMIN=0.0, ZMAX=1000.0, InterpOrder=3, DoInterlacing=1, LOS=3, Momentum=0)
    rng = np.random.default_rng(5)
    n = 50000
    x, y, z = (rng.uniform(1.0, 999.0, n) for _ in range(3))
    v = rng.normal(0.0, 10.0, n)
    with cg.PowerSpectrum(p, precision="fp32") as ps:
        with pytest.raises(cg.CapowError):
            ps.tile_kernel_ms()
        ps.paint(x, y, z, v)
        ms, rec = ps.tile_kernel_ms()
        assert ms > 0.0
        assert n <= rec <= 8 * n
    with cg.PowerSpectrum(p, precision="fp64") as ps:
        ps.paint(x, y, z, v)
        with pytest.raises(cg.CapowError):
            ps.tile_kernel_ms()


def test_fp32_tile_scale_heavy_weights(gpu):
    """Weights over six decades plus a few dominant particles: FP32 tiles whose scale is set by the
    largest deposit (each deposit below 2^22, rounded by the FFMA magic-number add) as well as by the
    tile sum. Grids and spectra against the FP64 path (weights are a library extension; the FP64
    path is pinned to the oracle elsewhere)."""
    p = cg.Params(NX=64, NY=64, NZ=64, NK=20, Maxk=0.3, XMIN=0.0, XMAX=1000.0, YMIN=0.0, YMAX=1000.0,
                  ZMIN=0.0, ZMAX=1000.0, InterpOrder=3, DoInterlacing=1, LOS=3, Momentum=0)
    rng = np.random.default_rng(17)
    n = 200000
    x, y, z = (rng.uniform(20.0, 980.0, n) for _ in range(3))
    v = rng.normal(0.0, 300.0, n)
    w = 10.0 ** rng.uniform(-3.0, 3.0, n)
    w[:5] = 1.0e6
    out = {}
    for prec in ("fp64", "fp32"):
        with cg.PowerSpectrum(p, precision=prec, spectra=["dd", "dp", "pp"]) as ps:
            ps.paint(x, y, z, v, w)
            g = [ps.grid(k) for k in range(4)]
            out[prec] = (g, ps.power())
    for k in range(4):
        grid_close(out["fp32"][0][k], out["fp64"][0][k], p, "fp32", label=f"slot {k}")
    r32, r64 = out["fp32"][1], out["fp64"][1]
    for q, name in ((0, "dd"), (2, "pp")):
        assert_spectrum(r32[q], r64[q], np.abs(np.asarray(r64[q]["Pk0"])), "fp32", odd=False, label=name)


def test_transposed_path_falls_back_when_memory_is_short(gpu):
    """A power-of-two NZ takes the transposed (y,z) pass, which needs a second grid-sized buffer.
    With the device nearly full (a bounded filler allocation leaves room for the grids but not for
    that buffer), capow_create keeps the in-place 2-D cuFFT layout: one library kernel fewer per
    capow_power (no k_zr2c), same spectra."""
    torch = pytest.importorskip("torch")
    p = cg.Params(NX=256, NY=256, NZ=256, NK=40, Maxk=0.6, XMIN=0.0, XMAX=1000.0, YMIN=0.0, YMAX=1000.0,
                  ZMIN=0.0, ZMAX=1000.0, InterpOrder=3, DoInterlacing=1, LOS=3, Momentum=0)
    rng = np.random.default_rng(23)
    n = 300000
    x, y, z = (rng.uniform(1.0, 999.0, n) for _ in range(3))
    v = rng.normal(0.0, 100.0, n)

    def run():
        with cg.PowerSpectrum(p, precision="fp32", spectra=["dd", "dp", "pp"]) as ps:
            ps.paint(x, y, z, v)
            l0 = ps.kernel_launches()
            r = ps.power()
            return r, ps.kernel_launches() - l0

    r_normal, k_normal = run()
    grids = 4 * 256 * 256 * 258 * 4  # the painted slots; the transposed buffer is as large
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    free, _ = torch.cuda.mem_get_info()
    # leave room for the grids and 0.9 of them (plans, tables, records), not for a second copy
    filler = torch.empty(max(0, free - int(1.9 * grids)), dtype=torch.uint8, device=gpu)
    try:
        r_short, k_short = run()
    finally:
        del filler
        torch.cuda.empty_cache()
    assert k_short == k_normal - 1, (k_short, k_normal)
    pdd, ppp = (np.abs(np.asarray(r_normal[q]["Pk0"])) for q in (0, 2))
    for q, norm0 in ((0, pdd), (1, np.sqrt(pdd * ppp)), (2, ppp)):
        assert_spectrum(r_short[q], r_normal[q], norm0, "fp32", odd=False, label=f"spectrum {q}")


def test_host_catalogue_in_chunks_matches_device_input(gpu):
    """A host catalogue of >= 4M particles is copied in chunks that the bucket pass consumes as they
    land. Against the same catalogue passed on the device (one bucket launch): equal grids, counters
    and spectra, with edge particles in every chunk (their indices go through the chunk's base) and,
    for LOS = 0, the first out-of-box particle planted in the last chunk reported by its index."""
    torch = pytest.importorskip("torch")
    p = cg.Params(NX=64, NY=64, NZ=64, NK=20, Maxk=0.3, XMIN=0.0, XMAX=1000.0, YMIN=0.0, YMAX=1000.0,
                  ZMIN=0.0, ZMAX=1000.0, InterpOrder=3, DoInterlacing=1, LOS=3, Momentum=1)
    rng = np.random.default_rng(31)
    n = 5_000_000
    d = 1000.0 / 64
    x, y, z = (rng.uniform(2.0, 998.0, n).astype(np.float32) for _ in range(3))
    v = rng.normal(0.0, 100.0, n).astype(np.float32)
    picks = rng.choice(n, 400, replace=False)  # on cell edges (the exact-rules path), all chunks
    x[picks] = (np.floor(x[picks] / d) * d).astype(np.float32)
    out = {}
    for where in ("host", "device"):
        arrs = [x, y, z, v] if where == "host" else [torch.from_numpy(a).to(gpu) for a in (x, y, z, v)]
        with cg.PowerSpectrum(p, precision="fp32", spectra=["dd", "dp", "pp"]) as ps:
            ps.paint(*arrs)
            g = [ps.grid(k) for k in range(4)]
            st = ps.stats()
            out[where] = (g, st, ps.power())
    gh, sh, rh = out["host"]
    gd, sd, rd = out["device"]
    for k in range(4):
        scale = np.abs(gd[k]).max()
        assert np.abs(gh[k] - gd[k]).max() <= 1e-6 * scale, k
    for key in ("nread", "nout", "ngrid", "nsq"):
        assert sh[key] == sd[key], key
    pdd, ppp = (np.abs(np.asarray(rd[q]["Pk0"])) for q in (0, 2))
    for q, norm0 in ((0, pdd), (1, np.sqrt(pdd * ppp)), (2, ppp)):
        assert_spectrum(rh[q], rd[q], norm0, "fp32", odd=False, label=f"spectrum {q}")
    # LOS = 0: a particle outside the box in the last chunk is the reference's fatal error
    p0 = cg.Params(NX=64, NY=64, NZ=64, NK=20, Maxk=0.3, XMIN=0.0, XMAX=1000.0, YMIN=0.0, YMAX=1000.0,
                   ZMIN=0.0, ZMAX=1000.0, InterpOrder=3, DoInterlacing=1, LOS=0, Momentum=0)
    bad = n - 1234
    xb = x.copy()
    xb[bad] = np.float32(1003.0)
    with cg.PowerSpectrum(p0, precision="fp32") as ps:
        ps.paint(xb, y, z)
        with pytest.raises(cg.CapowError) as e:
            ps.power()
        assert e.value.status == cg.EBOUNDS
        assert ps.stats()["first_out_of_box"] == bad


def test_zy_wait_that_runs_out_reports_timeout(gpu, monkeypatch):
    """The one-launch z + y transform (fft_path one_launch) waits, per x-plane, for that plane's z transforms. Each wait is
    bounded: with the test switch CAPOW_TEST_STALL_ZY=1 every y item waits for one z item more than
    exists, its wait runs out (about a second), the launch stops, and capow_power returns
    CAPOW_ETIMEOUT. The device stays usable: a context created without the switch gives the spectra
    of the 3-D transform path."""
    p = cg.Params(NX=32, NY=32, NZ=32, NK=12, Maxk=0.3, XMIN=0.0, XMAX=1000.0, YMIN=0.0, YMAX=1000.0,
                  ZMIN=0.0, ZMAX=1000.0, InterpOrder=3, DoInterlacing=1, LOS=3, Momentum=0)
    rng = np.random.default_rng(41)
    x, y, z = (rng.uniform(1.0, 999.0, 20000) for _ in range(3))
    v = rng.normal(0.0, 100.0, 20000)
    monkeypatch.setenv("CAPOW_TEST_STALL_ZY", "1")
    with cg.PowerSpectrum(p, precision="fp32", fft_path="one_launch") as ps:
        ps.paint(x, y, z, v)
        with pytest.raises(cg.CapowError) as e:
            ps.power()
        assert e.value.status == cg.ETIMEOUT
    monkeypatch.delenv("CAPOW_TEST_STALL_ZY")
    with cg.PowerSpectrum(p, precision="fp32", fft_path="one_launch") as ps:
        ps.paint(x, y, z, v)
        r = ps.power()[0]
    with cg.PowerSpectrum(p, precision="fp32", fft_path="3d") as ps:
        ps.paint(x, y, z, v)
        r3 = ps.power()[0]
    assert_spectrum(r, r3, np.abs(np.asarray(r3["Pk0"])), "fp32", odd=False, label="after timeout")
