"""The CPU oracle against the reference's own outputs.

* Committed golden fixtures (tests/golden, generated from the unmodified reference by
  make_golden.py): raw bin sums, mode counts, Allreduce scalars and painted grids must be
  bit-identical, and the oracle's normalised output must print exactly as the reference's file.
* Where the reference binary can be built (its sources mounted), fresh random cases as well.
"""
import glob
import json
import os

import numpy as np
import pytest

import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
MANIFEST = json.load(open(os.path.join(GOLD, "manifest.json")))
CASES = sorted(n for n in (os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLD, "*.npz"))) if n in MANIFEST)


@pytest.fixture(scope="module", autouse=True)
def _built():
    orc.build()


def load(name):
    d = dict(np.load(os.path.join(GOLD, f"{name}.npz")))
    p = orc.Params(**{k: v for k, v in MANIFEST[name]["params"].items()})
    return p, d


@pytest.mark.parametrize("name", CASES)
def test_raw_sums_bit_exact(name):
    p, d = load(name)
    r = orc.run(p, d["x"], d["y"], d["z"], d["vx"], d["vy"], d["vz"])
    for k in ("Pk0", "Pk2", "Pk4") + (("Pk1", "Pk3") if p.Odd_Multipoles else ()):
        assert np.array_equal(r["raw"][k], d[k]), k
    assert np.array_equal(r["raw"]["Nmodes"], d["Nmodes"])
    if p.Output2D:
        assert np.array_equal(r["raw"]["Pk_2D"], d["Pk_2D"])
        assert np.array_equal(r["raw"]["Nmodes_2D"], d["Nmodes_2D"])
    # NPERIODIC then (Momentum != 0) nsq, vr_ave..vr4_ave, as the reference's Allreduce calls saw them
    st = r["stats"]
    ar = d["allreduce"]
    assert ar[0] == st["ngrid"]
    if p.Momentum:
        assert list(ar[1:6]) == [st["nsq"], st["vr_ave"], st["vr2_ave"], st["vr3_ave"], st["vr4_ave"]]


@pytest.mark.parametrize("name", [c for c in CASES if "grid_ddg" in np.load(os.path.join(GOLD, f"{c}.npz"))])
def test_painted_grids_bit_exact(name):
    p, d = load(name)
    g, _ = orc.paint(p, d["x"], d["y"], d["z"], d["vx"], d["vy"], d["vz"])
    n = p.NX * 2 * p.NY * (p.NZ // 2 + 1)
    for k in ("ddg", "ddg_interlace", "ddg_mom", "ddg_mom_interlace"):
        if "grid_" + k in d:
            assert np.array_equal(g[k][:n], d["grid_" + k]), k


def format_output(p, normed):
    """the reference's output_power text (src/main.c:1058-1081) from normalised sums"""
    binwidth = (p.Maxk - p.Mink) / p.NK
    lines = [f"# shot = {normed['shot'] / normed['norm']:g}", f"# norm = {normed['norm']:g}"]
    lines.append("# k  pk0  pk1  pk2  pk3  pk4  Nmodes" if p.Odd_Multipoles else "# k  pk0  pk2  pk4  Nmodes")
    for i in range(p.NK):
        kp = p.Mink + (float(np.float32(i)) + 0.5) * binwidth
        if p.OutputLog:
            kp = 10.0 ** kp
        vals = [normed["Pk0"][i]] + ([normed["Pk1"][i]] if p.Odd_Multipoles else []) + [normed["Pk2"][i]] + (
            [normed["Pk3"][i]] if p.Odd_Multipoles else []) + [normed["Pk4"][i]]
        lines.append(" ".join(f"{v:g}" for v in [kp] + vals) + f" {int(normed['Nmodes'][i])}")
    return "\n".join(lines) + "\n"


@pytest.mark.parametrize("name", CASES)
def test_normalised_output_matches_reference_file(name):
    p, d = load(name)
    r = orc.run(p, d["x"], d["y"], d["z"], d["vx"], d["vy"], d["vz"])
    nm = dict(r["norm"], shot=r["shot"], norm=r["normf"])
    with open(os.path.join(GOLD, f"{name}.out")) as f:
        ref = f.read()
    if p.OutputLog:  # pow(10, x) vs 10.0 ** x may differ in the last ulp; compare numerically
        a = np.loadtxt(ref.splitlines()[3:])
        b = np.loadtxt(format_output(p, nm).splitlines()[3:])
        assert np.allclose(a, b, rtol=1e-5)
    else:
        assert format_output(p, nm) == ref


def test_fft_matches_numpy():
    rng = np.random.default_rng(0)
    for n3 in [(8, 8, 8), (6, 10, 7), (12, 9, 15), (16, 32, 30)]:
        nx, ny, nz = n3
        a = rng.normal(size=n3)
        row = 2 * (nz // 2 + 1)
        g = np.zeros(nx * ny * row)
        g.reshape(nx, ny, row)[:, :, :nz] = a
        orc.fft_r2c_inplace(g, nx, ny, nz)
        ref = np.fft.rfftn(a)
        got = g.view(np.complex128).reshape(nx, ny, nz // 2 + 1)
        assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


def test_fft_plane_wave_kat():
    """known answer: a single cosine mode lands on exactly two r2c coefficients"""
    nx, ny, nz = 8, 6, 10
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    a = np.cos(2 * np.pi * (2 * i / nx + 1 * j / ny + 3 * k / nz))
    row = 2 * (nz // 2 + 1)
    g = np.zeros(nx * ny * row)
    g.reshape(nx, ny, row)[:, :, :nz] = a
    orc.fft_r2c_inplace(g, nx, ny, nz)
    F = g.view(np.complex128).reshape(nx, ny, nz // 2 + 1)
    expect = np.zeros_like(F)
    expect[2, 1, 3] = nx * ny * nz / 2
    assert np.abs(F - expect).max() < 1e-10


@pytest.mark.skipif(not orc.ref_available(), reason="reference binary only buildable where its sources are mounted")
@pytest.mark.parametrize("seed", [11, 12, 13])
def test_fresh_random_cases_against_reference_binary(tmp_path, seed):
    rng = np.random.default_rng(seed)
    for _ in range(6):
        kw = dict(NX=int(rng.integers(5, 14)), NY=int(rng.integers(5, 14)), NZ=int(rng.integers(5, 14)),
                  InterpOrder=int(rng.integers(1, 4)), LOS=int(rng.choice([0, 1, 2, 3])),
                  DoInterlacing=int(rng.integers(0, 2)), Momentum=int(rng.integers(0, 9)), NK=9, Maxk=0.08,
                  Odd_Multipoles=1, XMIN=-50.0, XMAX=450.0, YMIN=0.0, YMAX=300.0, ZMIN=1.0, ZMAX=601.0)
        p = orc.Params(**kw)
        n = 300
        pos = np.stack([rng.uniform(p.XMIN, p.XMAX, n), rng.uniform(p.YMIN, p.YMAX, n),
                        rng.uniform(p.ZMIN, p.ZMAX, n)])
        vel = rng.normal(0, 300, (3, n))
        r = orc.run_ref_binary(p, str(tmp_path / "c"), *pos, *vel, grids=True)
        assert r["returncode"] == 0, r["stdout"][-400:]
        mine = orc.run(p, *pos, *vel)
        g, _ = orc.paint(p, *pos, *vel)
        slab = p.NX * 2 * p.NY * (p.NZ // 2 + 1)
        for k, v in r["grids"].items():
            assert np.array_equal(v, g[k][:slab]), (kw, k)
        for k in ("Pk0", "Pk1", "Pk2", "Pk3", "Pk4", "Nmodes"):
            assert np.array_equal(r["dump"][k], mine["raw"][k]), (kw, k)


SURVEY = json.load(open(os.path.join(GOLD, "survey_manifest.json")))


def write_survey_inputs(tmp_path, name):
    """The golden survey case's parameter file and catalogues, written as the reference read them."""
    m = SURVEY[name]
    d = np.load(os.path.join(GOLD, f"{name}.npz"))
    p = orc.Params(**m["params"])
    pf, df, rf = (str(tmp_path / f) for f in ("p.dat", "data.txt", "rand.txt"))
    p.write_file(pf)
    np.savetxt(df, d["data"], fmt="%.17g")
    np.savetxt(rf, d["rand"], fmt="%.17g")
    return p, pf, df, rf, d


@pytest.mark.parametrize("name", sorted(SURVEY))
def test_oracle_survey_matches_reference_bit_for_bit(tmp_path, name):
    """The oracle's survey-mode restatement (reader with the redshift cut and float object fields, FKP
    weights, data minus alpha randoms, the Yamamoto multipoles of compute_survey_power) against the
    unmodified reference's raw bin sums for the same catalogues."""
    p, pf, df, rf, d = write_survey_inputs(tmp_path, name)
    r = orc.survey_run(p, df, rf)
    assert np.array_equal(r["raw"]["Nmodes"], d["Nmodes"])
    for k in ("Pk0", "Pk1", "Pk2", "Pk3", "Pk4"):
        if k in ("Pk1", "Pk3") and not p.Odd_Multipoles:
            continue
        assert np.array_equal(r["raw"][k], d[k]), (name, k)
    # the normalised first data row of the reference's output file
    row = [float(t) for t in open(os.path.join(GOLD, f"{name}.out")).read().splitlines()[3].split()]
    got = r["norm"]["Pk0"][0]
    if np.isfinite(row[1]):
        assert abs(row[1] - got) <= 1e-5 * abs(row[1]) + 1e-9
    else:  # Momentum 3: the reference's norm is zero
        assert got == row[1]
    # the scalars the reference printed (src/main.c:189-203)
    txt = open(os.path.join(GOLD, f"{name}.stdout")).read()
    if p.Momentum == 0:
        assert f"alpha = {r['alpha']:g}" in txt
    elif p.Momentum == 1:
        assert f"shot-noise [data]    = {r['sums']['data_vrsq']:g} " in txt
    else:
        assert f"shot-noise    = {r['sums']['data_vr']:g}" in txt and f"normalisation = {r['normf']:g}" in txt
