"""GPU parity of the survey estimator (capow_survey_*) against the oracle's restatement of the reference's
survey path (pinned bit for bit to the unmodified reference on the golden survey cases): the unmodified
reference's raw bin sums for the golden catalogues, the oracle on seeded catalogues (every order, with and
without interlacing, odd multipoles, an observer inside the grid on a cell corner, the velocity spectra of
Momentum 1 to 3), painted grids, the weight sums, and the edge cases of the reader's float storage."""
import os

import numpy as np
import pytest

import capow_gb300 as cg
import oracle as orc
from parity_util import TOL
from test_oracle_golden import SURVEY, write_survey_inputs

pytestmark = pytest.mark.gpu


def assert_survey(res, ref, p, precision, label=""):
    """Raw sums against the reference's (or the oracle's): Nmodes bit-exact; per bin with modes
    (2l+1) |dP_l| <= tol |P0_ref|, the tolerances of the periodic parity tests (FP64 1e-10; FP32 1e-4 for
    l = 0, 1e-3 above). The k = 0 mode carries the grid's total, data minus alpha randoms, which is zero
    up to rounding in both computations: its bin is also allowed (2l+1) (1e-12 W)^2 (FP32: (1e-5 W)^2) with
    W = sum w_data + alpha sum w_rand the total painted weight. The cross spectra of Momentum 2 and 3 change
    sign from bin to bin: their |P0| scale is the largest within two bins, so that a bin whose P0 crosses
    zero (or holds only the k = 0 mode, where the cross form vanishes) keeps the spectrum's own scale."""
    assert np.array_equal(np.asarray(res["Nmodes"], np.int64), np.asarray(ref["Nmodes"], np.int64)), label
    t0, t2 = TOL[precision]
    allow = np.zeros(p.NK)
    bw = (p.Maxk - p.Mink) / p.NK
    kb0 = int(np.float32(0.0 - p.Mink) / bw) if not p.OutputLog else -1
    if 0 <= kb0 < p.NK:
        W = 2.0 * res["stats"]["data_nbw"]
        allow[kb0] = ((1e-12 if precision == "fp64" else 1e-5) * W) ** 2
    m = np.asarray(ref["Nmodes"]) > 0
    norm0 = np.abs(np.asarray(ref["Pk0"]))
    if p.Momentum >= 2:
        a = np.where(m, norm0, 0.0)
        norm0 = np.array([a[max(0, b - 2):b + 3].max() for b in range(p.NK)])
    for l in range(5):
        if l in (1, 3) and not p.Odd_Multipoles:
            continue
        err = (2 * l + 1) * np.abs(np.asarray(res[f"Pk{l}"]) - np.asarray(ref[f"Pk{l}"]))
        lim = (t0 if l == 0 else t2) * norm0 + (2 * l + 1) * allow
        bad = m & (err > lim)
        assert not bad.any(), f"{label}: l={l} bins {np.nonzero(bad)[0]} err {err[bad]} > {lim[bad]}"


def _catalogues(tmp_path, p, nd, nr, seed, origin_inside=False):
    """Seeded data (12 columns) and random (8 columns) catalogues inside the reader's bounds. With a
    Momentum, the data's 7th and 8th numbers are a log-distance ratio that follows the position (so the
    velocity field correlates with the density) and its error, the randoms' 7th an error."""
    rng = np.random.default_rng(seed)
    dx, dy, dz = (p.XMAX - p.XMIN) / p.NX, (p.YMAX - p.YMIN) / p.NY, (p.ZMAX - p.ZMIN) / p.NZ
    m = p.InterpOrder - 1
    lo = np.array([p.XMIN + m * dx, p.YMIN + m * dy, p.ZMIN + m * dz])
    hi = np.array([p.XMAX - m * dx, p.YMAX - m * dy, p.ZMAX - m * dz]) - (0.5 * np.array([dx, dy, dz])
                                                                          if p.DoInterlacing else 0.0)
    span = hi - lo

    def cat(n, cols, clustered):
        a = np.zeros((n, cols))
        if clustered:  # a few clumps on top of a uniform part, so the multipoles are not pure noise
            c = lo + span * rng.uniform(0.2, 0.8, size=(8, 3))
            k = rng.integers(0, 8, n)
            pos = c[k] + rng.normal(scale=0.08, size=(n, 3)) * span
            u = rng.uniform(size=n) < 0.4
            pos[u] = lo + span * rng.uniform(size=(int(u.sum()), 3))
            pos = np.clip(pos, lo, hi - 1e-9 * span)
        else:
            pos = lo + span * rng.uniform(size=(n, 3)) * (1 - 1e-12)
        a[:, :3] = pos
        a[:, 3] = rng.uniform(0.5, 1.5, n)
        a[:, 4] = rng.uniform(1e-4, 3e-4, n)
        return a

    d, r = cat(nd, 12, True), cat(nr, 8, False)
    if p.Momentum:
        d[:, 6] = 0.04 * np.sin(d[:, 0] / 150.0 + d[:, 1] / 230.0) + rng.normal(0.0, 0.02, nd)
        d[:, 7] = rng.uniform(0.03, 0.08, nd)
        r[:, 6] = rng.uniform(0.03, 0.08, nr)
    df, rf = str(tmp_path / "data.txt"), str(tmp_path / "rand.txt")
    np.savetxt(df, d, fmt="%.17g")
    np.savetxt(rf, r, fmt="%.17g")
    return df, rf


def _write_params(tmp_path, **kw):
    p = orc.Params(**kw)
    pf = str(tmp_path / "p.dat")
    p.write_file(pf)
    prm, sv = cg.read_survey_params(pf)
    return p, prm, sv


def _gpu(prm, sv, df, rf, precision, grids=False, device_inputs=False):
    data, rand, _ = cg.read_survey_pair(df, rf, prm, sv)
    keys = ("x", "y", "z", "w", "nbar") + (("pv", "pverr") if prm.Momentum else ())
    if device_inputs:
        import torch
        dd = {k: torch.from_numpy(data[k]).cuda() for k in keys}
        rr = {k: torch.from_numpy(rand[k]).cuda() for k in keys}
    else:
        dd, rr = {k: data[k] for k in keys}, {k: rand[k] for k in keys}
    with cg.SurveySpectrum(prm, sv, precision=precision) as ss:
        res = ss.power(dd, rr)
        nslot = (1 + prm.DoInterlacing) * (2 if prm.Momentum >= 2 else 1)
        g = [ss.grid(w) for w in range(nslot)] if grids else None
        res["launches"] = ss.kernel_launches()
        res["stage"] = ss.stage_ms()
    return res, g


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", sorted(SURVEY))
def test_survey_golden_reference_sums(gpu, tmp_path, name, precision):
    """The unmodified reference's raw sums for the golden survey catalogues, read by the product's reader."""
    p, pf, df, rf, d = write_survey_inputs(tmp_path, name)
    prm, sv = cg.read_survey_params(pf)
    res, _ = _gpu(prm, sv, df, rf, precision)
    ref = {k: d[k] for k in ("Pk0", "Pk1", "Pk2", "Pk3", "Pk4", "Nmodes")}
    assert_survey(res, ref, p, precision, label=f"{name} {precision}")
    r = orc.survey_run(p, df, rf)
    for k, v in (("alpha", r["alpha"]), ("shot", r["shot"]), ("norm", r["normf"])):
        assert abs(res[k] - v) <= 1e-13 * abs(v), (k, res[k], v)
    assert res["stage"][2] == (25 if p.Odd_Multipoles else 15)
    assert res["launches"] > 0


CASES = [(1, 0, 0), (2, 0, 1), (2, 1, 0), (3, 1, 1), (3, 0, 0), (1, 1, 1)]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("order,il,odd", CASES)
def test_survey_matches_oracle(gpu, tmp_path, precision, order, il, odd):
    """Seeded clustered data and uniform randoms on a 40x36x32 grid off the observer: raw sums, Nmodes,
    alpha, shot, norm and the gridded counters against the oracle."""
    p, prm, sv = _write_params(tmp_path, NX=40, NY=36, NZ=32, XMIN=300.0, XMAX=1100.0, YMIN=-400.0, YMAX=320.0,
                               ZMIN=-300.0, ZMAX=340.0, InterpOrder=order, DoInterlacing=il, NK=20, Maxk=0.15,
                               Odd_Multipoles=odd, Periodic=0, X_Origin=-50.0, Y_Origin=20.0, Z_Origin=5.0,
                               REDMININ=0.0, REDMAXIN=5.0, NOBJ_Max=100000, NBAR_Column=5, FKP_Column=-1,
                               FKP_Pk=4000.0)
    df, rf = _catalogues(tmp_path, p, 4000, 30000, seed=order * 10 + il + 2 * odd)
    r = orc.survey_run(p, df, rf, grids=True)
    res, g = _gpu(prm, sv, df, rf, precision, grids=True)
    label = f"{precision} order={order} il={il} odd={odd}"
    assert_survey(res, r["raw"], p, precision, label=label)
    for k, v in (("alpha", r["alpha"]), ("shot", r["shot"]), ("norm", r["normf"])):
        assert abs(res[k] - v) <= 1e-13 * abs(v), (label, k)
    assert abs(res["stats"]["ngrid_data"] - r["ngrid_data"]) <= 1e-9 * r["ngrid_data"]
    assert abs(res["stats"]["ngrid_rand"] - r["ngrid_rand"]) <= 1e-9 * r["ngrid_rand"]
    row = 2 * (p.NZ // 2 + 1)
    for which, key in enumerate(("ddg", "ddg_interlace")[: 1 + il]):
        a = g[which].reshape(p.NX, p.NY, row)[:, :, :p.NZ]
        b = r["painted"][key][: p.NX * p.NY * row].reshape(p.NX, p.NY, row)[:, :, :p.NZ]
        scale = np.abs(b).max()
        err = np.abs(a - b).max() / scale
        # FP32: the tile kernels accumulate int32 fixed point with a quantum of 2^-30 of the tile's sum of
        # |w|, data and randoms together, while a cell holds their difference
        assert err <= (1e-12 if precision == "fp64" else 5e-5), (label, key, err)


def test_survey_long_z_axis(gpu, tmp_path):
    """A 16 x 16 x 1024 grid: the FP32 path's z pass takes its eight-row blocks there (its weighted variant
    included), with odd multipoles; against the oracle."""
    p, prm, sv = _write_params(tmp_path, NX=16, NY=16, NZ=1024, XMIN=300.0, XMAX=700.0, YMIN=-200.0, YMAX=200.0,
                               ZMIN=-2000.0, ZMAX=2000.0, InterpOrder=3, DoInterlacing=1, NK=12, Maxk=0.06,
                               Odd_Multipoles=1, Periodic=0, X_Origin=-40.0, Y_Origin=10.0, Z_Origin=5.0,
                               REDMININ=0.0, REDMAXIN=5.0, NOBJ_Max=100000, NBAR_Column=5, FKP_Column=-1,
                               FKP_Pk=4000.0)
    df, rf = _catalogues(tmp_path, p, 3000, 20000, seed=57)
    r = orc.survey_run(p, df, rf)
    for precision in ("fp32", "fp64"):
        res, _ = _gpu(prm, sv, df, rf, precision)
        assert_survey(res, r["raw"], p, precision, label=f"long z {precision}")


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("order,momentum", [(2, 0), (3, 0), (3, 1), (2, 2)])
def test_survey_observer_on_a_cell_corner(gpu, tmp_path, precision, order, momentum):
    """The observer inside the grid exactly on a cell corner (r2 == 0 there: the reference zeroes every
    r^ product of that cell). The solid-harmonic multipoles add that cell's L_l(0) term in closed form: for
    the density and the velocity auto spectrum against F0, for the cross spectrum (Momentum 2) the
    symmetric form of the cell's density against F0_mom and its momentum against F0."""
    p, prm, sv = _write_params(tmp_path, NX=32, NY=32, NZ=32, XMIN=-400.0, XMAX=400.0, YMIN=-400.0, YMAX=400.0,
                               ZMIN=-400.0, ZMAX=400.0, InterpOrder=order, DoInterlacing=1, NK=16, Maxk=0.12,
                               Odd_Multipoles=1, Periodic=0, X_Origin=0.0, Y_Origin=0.0, Z_Origin=0.0,
                               REDMININ=0.0, REDMAXIN=5.0, NOBJ_Max=100000, NBAR_Column=5, FKP_Column=-1,
                               FKP_Pk=4000.0, FKP_Pk_mom=5e9, FKP_Pk_cross=5e5, Momentum=momentum)
    df, rf = _catalogues(tmp_path, p, 5000, 25000, seed=70 + order + 10 * momentum)
    # a heavy object next to the observer, so the corner cell carries weight (and velocity)
    with open(df, "a") as f:
        f.write("1.0 2.0 -1.5 40 0.0002 0 0.5 0.07 0 0 0 0\n")
    r = orc.survey_run(p, df, rf, grids=True)
    oc = r["painted"]["ddg"].reshape(-1)[(16 * 32 + 16) * 34 + 16]
    assert oc != 0.0
    if momentum >= 2:
        assert r["painted"]["ddg_mom"].reshape(-1)[(16 * 32 + 16) * 34 + 16] != 0.0
    res, _ = _gpu(prm, sv, df, rf, precision)
    assert_survey(res, r["raw"], p, precision, label=f"origin {precision} Momentum {momentum}")


def test_survey_float_storage_edges_and_device_inputs(gpu, tmp_path):
    """Objects the reader accepts in double whose float copy lands on the grid edge (the Survey clamps
    pull the stencil back), an object on the TSC x limit, and host vs device inputs giving the same sums."""
    p, prm, sv = _write_params(tmp_path, NX=20, NY=24, NZ=16, XMIN=-500.0, XMAX=500.0, YMIN=-600.0, YMAX=600.0,
                               ZMIN=-400.0, ZMAX=400.0, InterpOrder=2, DoInterlacing=0, NK=12, Maxk=0.09,
                               Odd_Multipoles=1, Periodic=0, X_Origin=900.0, Y_Origin=900.0, Z_Origin=900.0,
                               REDMININ=0.0, REDMAXIN=5.0, NOBJ_Max=100000, NBAR_Column=5, FKP_Column=-1,
                               FKP_Pk=3000.0)
    df, rf = _catalogues(tmp_path, p, 2000, 9000, seed=5)
    dy = 1200.0 / 24
    edge = 600.0 - dy  # YMAX_Interp for CIC; just below it in double, on it in float
    below = float(np.nextafter(edge, -np.inf))
    assert below < edge and np.float32(below) == np.float32(edge)
    with open(df, "a") as f:
        for x in (-100.0, 0.0, 250.0):
            f.write(f"{x!r} {below!r} 10.0 1.2 0.0002 0 0 0 0 0 0 0\n")
    r = orc.survey_run(p, df, rf)
    for precision in ("fp64", "fp32"):
        host, _ = _gpu(prm, sv, df, rf, precision)
        dev, _ = _gpu(prm, sv, df, rf, precision, device_inputs=True)
        assert_survey(host, r["raw"], p, precision, label=f"edges {precision}")
        scale = np.abs(host["Pk0"])
        for k in ("Pk0", "Pk2", "Pk4"):
            diff = np.abs(host[k] - dev[k])
            assert np.all(diff <= (1e-12 if precision == "fp64" else 1e-5) * scale), k


def test_survey_rejects_non_finite_and_bad_arguments(gpu, tmp_path):
    p, prm, sv = _write_params(tmp_path, NX=16, NY=16, NZ=16, XMIN=0.0, XMAX=800.0, YMIN=0.0, YMAX=800.0,
                               ZMIN=0.0, ZMAX=800.0, InterpOrder=2, DoInterlacing=0, NK=8, Maxk=0.1, Periodic=0,
                               X_Origin=-10.0, REDMININ=0.0, REDMAXIN=5.0, NOBJ_Max=1000, NBAR_Column=5,
                               FKP_Column=-1, FKP_Pk=1000.0)
    rng = np.random.default_rng(1)
    cat = {k: rng.uniform(100, 700, 100).astype(np.float32) for k in ("x", "y", "z")}
    cat["w"] = np.ones(100, np.float32)
    cat["nbar"] = np.full(100, 1e-4, np.float32)
    bad = dict(cat)
    bad["x"] = cat["x"].copy()
    bad["x"][7] = np.nan
    with cg.SurveySpectrum(prm, sv, precision="fp64") as ss:
        with pytest.raises(cg.CapowError) as e:
            ss.power(bad, cat)
        assert e.value.status == cg.EINVAL
        ok = ss.power(cat, cat)  # the context stays usable
        assert np.isfinite(ok["Pk0"]).all()
        mixed = dict(cat)
        mixed["w"] = np.ones(100)
        with pytest.raises(ValueError):
            ss.power(mixed, cat)
    p2 = cg.Params(**{**prm.__dict__, "Momentum": 4})
    with pytest.raises(cg.CapowError) as e:
        cg.SurveySpectrum(p2, sv)
    assert e.value.status == cg.ENOTSUP
    # Momentum 2, 3 take the velocity weights from the FKP weighting only
    p3 = cg.Params(**{**prm.__dict__, "Momentum": 3})
    sv3 = cg.SurveyParams(**{**sv.__dict__, "FKP_Column": 6})
    with pytest.raises(cg.CapowError) as e:
        cg.SurveySpectrum(p3, sv3)
    assert e.value.status == cg.EINVAL
    # Momentum 1 needs the data's pv and pverr: the C ABI refuses a catalogue without them
    p1 = cg.Params(**{**prm.__dict__, "Momentum": 1})
    with cg.SurveySpectrum(p1, sv, precision="fp64") as ss:
        with pytest.raises(cg.CapowError) as e:
            ss.power(dict(cat, pverr=cat["w"]), dict(cat, pverr=cat["w"]))  # the data without pv
        assert e.value.status == cg.EINVAL
        v = dict(cat, pv=np.full(100, 250.0, np.float32), pverr=np.full(100, 40.0, np.float32))
        ok = ss.power(v, dict(cat, pverr=v["pverr"]))
        assert np.isfinite(ok["Pk0"]).all() and ok["stats"]["ngrid_rand"] == 0.0


VCASES = [(1, 3, 1, 1), (1, 2, 0, 0), (2, 2, 1, 1), (2, 3, 0, 0), (3, 3, 1, 0), (3, 1, 0, 1)]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("momentum,order,il,odd", VCASES)
def test_survey_velocity_spectra_match_oracle(gpu, tmp_path, precision, momentum, order, il, odd):
    """The survey velocity spectra on seeded catalogues with a position-dependent log-distance ratio:
    Momentum 1 (the data's w pv field against itself, no randoms), 2 and 3 (the density of data minus alpha
    randoms crossed with the data's w_pv pv momentum field; the reference's Momentum 2 stops in its own
    allocation, so the oracle pins it; Momentum 3's reference norm is zero, so its raw sums are compared).
    Raw sums, Nmodes, shot, norm, the velocity sums and the gridded counters against the oracle."""
    p, prm, sv = _write_params(tmp_path, NX=40, NY=36, NZ=32, XMIN=300.0, XMAX=1100.0, YMIN=-400.0, YMAX=320.0,
                               ZMIN=-300.0, ZMAX=340.0, InterpOrder=order, DoInterlacing=il, NK=20, Maxk=0.15,
                               Odd_Multipoles=odd, Periodic=0, X_Origin=-50.0, Y_Origin=20.0, Z_Origin=5.0,
                               REDMININ=0.0, REDMAXIN=5.0, NOBJ_Max=100000, NBAR_Column=5, FKP_Column=-1,
                               FKP_Pk=4000.0, FKP_Pk_mom=5e9, FKP_Pk_cross=5e5, Momentum=momentum)
    df, rf = _catalogues(tmp_path, p, 4000, 30000, seed=100 + 10 * momentum + order)
    r = orc.survey_run(p, df, rf, grids=True)
    res, g = _gpu(prm, sv, df, rf, precision, grids=True)
    label = f"{precision} Momentum {momentum} order={order} il={il} odd={odd}"
    assert_survey(res, r["raw"], p, precision, label=label)
    for k, v in (("shot", r["shot"]), ("norm", r["normf"])):
        assert abs(res[k] - v) <= 1e-13 * abs(v), (label, k, res[k], v)
    st, sums = res["stats"], r["sums"]
    for k in ("data_vr", "data_vrsq", "data_nbsqwsq_pv", "rand_nbsqwsq_pv", "data_nbw", "rand_nbsqwsq"):
        assert abs(st[k] - sums[k]) <= 1e-12 * abs(sums[k]), (label, k, st[k], sums[k])
    assert abs(st["ngrid_data"] - r["ngrid_data"]) <= 1e-9 * abs(r["ngrid_data"]) + 1e-12, label
    if momentum != 1:
        assert abs(st["ngrid_rand"] - r["ngrid_rand"]) <= 1e-9 * r["ngrid_rand"], label
    row = 2 * (p.NZ // 2 + 1)
    nf = 2 if momentum >= 2 else 1
    # grid slots: stencil * fields + field (density 0, momentum 1)
    keys = [("ddg", 0), ("ddg_interlace", nf), ("ddg_mom", 1), ("ddg_mom_interlace", 3)]
    keys = [(k, s) for k, s in keys if r["painted"][k] is not None]
    assert len(keys) == len(g), label
    for key, slot in keys:
        a = g[slot].reshape(p.NX, p.NY, row)[:, :, :p.NZ]
        b = r["painted"][key][: p.NX * p.NY * row].reshape(p.NX, p.NY, row)[:, :, :p.NZ]
        err = np.abs(a - b).max() / np.abs(b).max()
        assert err <= (1e-12 if precision == "fp64" else 5e-5), (label, key, err)
