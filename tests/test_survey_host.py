"""Host side of the survey estimator (no GPU): the parameter reader's survey tags and the product's
survey catalogue reader (read_survey_serial_ascii, src/read_data.c:184-361) against the oracle's reader on
the golden survey catalogues, plus its edge cases."""
import os

import numpy as np
import pytest

import capow_gb300 as cg
import oracle as orc
from test_oracle_golden import SURVEY, write_survey_inputs


def _read_params(pf):
    return cg.read_survey_params(pf)


@pytest.mark.parametrize("name", sorted(SURVEY))
def test_survey_params_reader_returns_the_survey_tags(tmp_path, name):
    p, pf, df, rf, d = write_survey_inputs(tmp_path, name)
    prm, sv = _read_params(pf)
    assert (sv.Periodic, sv.Survey) == (0, 1)
    assert (prm.NX, prm.NY, prm.NZ, prm.InterpOrder) == (p.NX, p.NY, p.NZ, p.InterpOrder)
    assert (sv.X_Origin, sv.Y_Origin, sv.Z_Origin) == (p.X_Origin, p.Y_Origin, p.Z_Origin)
    assert (sv.REDMININ, sv.REDMAXIN, sv.FKP_Pk, sv.NBAR_Column, sv.FKP_Column) == (
        p.REDMININ, p.REDMAXIN, p.FKP_Pk, p.NBAR_Column, p.FKP_Column)
    with pytest.raises(cg.CapowError) as e:
        cg.read_params(pf)
    assert e.value.status == cg.ENOTSUP


@pytest.mark.parametrize("name", sorted(SURVEY))
@pytest.mark.parametrize("randoms", [False, True])
def test_survey_reader_matches_the_oracle(tmp_path, name, randoms):
    """Kept objects, their float fields, NREAD and the printed ranges: identical to the oracle's reader
    (which is pinned to the reference's output through the golden spectra)."""
    p, pf, df, rf, d = write_survey_inputs(tmp_path, name)
    prm, sv = _read_params(pf)
    path = rf if randoms else df
    got = cg.read_survey(path, prm, sv, randoms)
    ref = orc.survey_read(p, path, randoms)
    assert got["n"] == len(ref["x"]) and got["nread"] == ref["nread"]
    for k in ("x", "y", "z", "weight", "nbar", "redshift", "pv", "pverr"):
        mine = got["w" if k == "weight" else k]
        assert mine.dtype == np.float32
        assert np.array_equal(mine, ref[k]), k
    if p.Momentum:  # the velocity cases carry log-distance ratios: pv and its error are not all zero
        assert np.any(got["pverr"] != 0) and (randoms or np.any(got["pv"] != 0))
    # "Have N objects" and the ranges, as the unmodified reference printed them for this catalogue
    txt = open(os.path.join(os.path.dirname(__file__), "golden", f"{name}.stdout")).read().splitlines()
    at = [i for i, t in enumerate(txt) if t.startswith("Have ")][1 if randoms else 0]
    assert txt[at] == f"Have {got['n']} objects"
    for ax, lab in enumerate("XYZ"):
        assert txt[at + 1 + ax] == "%12.6f <   %s  < %12.6f" % (got["lo"][ax], lab, got["hi"][ax])


def _params_file(tmp_path, **kw):
    base = dict(NX=16, NY=16, NZ=16, XMIN=-500.0, XMAX=500.0, YMIN=-500.0, YMAX=500.0, ZMIN=-500.0, ZMAX=500.0,
                InterpOrder=2, DoInterlacing=0, Periodic=0, Coord_Type=0, REDMININ=0.0, REDMAXIN=5.0,
                NOBJ_Max=1000, NBAR_Column=5, FKP_Column=-1, FKP_Pk=1000.0)
    base.update(kw)
    p = orc.Params(**base)
    pf = str(tmp_path / "p.dat")
    p.write_file(pf)
    return p, pf


def test_survey_reader_errors_and_quirks(tmp_path):
    p, pf = _params_file(tmp_path)
    prm, sv = _read_params(pf)
    row = "10 20 30 1.5 0.001 0 0 0 0 0 0 0"
    f = tmp_path / "d.txt"
    # leading comments skipped; blank lines skipped; a last line without a newline is not read
    f.write_text("# a\n# b\n" + row + "\n" + row + "\n" + row.replace("10 ", "11 "))
    got = cg.read_survey(str(f), prm, sv, False)
    assert got["n"] == 2 and got["nread"] == 2
    # ... unless blank lines before it leave room in the reference's byte count
    f.write_text(row + "\n\n" + row.replace("10 ", "11 "))
    assert cg.read_survey(str(f), prm, sv, False)["n"] == 2
    # too few numbers: the reference's message with the offending line
    f.write_text(row + "\n1 2 3\n")
    with pytest.raises(cg.CapowError) as e:
        cg.read_survey(str(f), prm, sv, False)
    assert "Task 0 has error reading file: 1 2 3" in str(e.value) and "line 102 in routine read_data" in str(e.value)
    # an object outside the grid less the interpolation margin
    f.write_text("499.5 0 0 1 0.001 0 0 0 0 0 0 0\n")
    with pytest.raises(cg.CapowError) as e:
        cg.read_survey(str(f), prm, sv, False)
    assert "object out of grid bounds for chosen InterpOrder: x=499.500000" in str(e.value)
    assert "line 155 in routine read_data" in str(e.value)
    # randoms take 8 numbers
    f.write_text("10 20 30 1.5 0.002 0 0 0\n")
    r = cg.read_survey(str(f), prm, sv, True)
    assert r["n"] == 1 and r["nbar"][0] == np.float32(0.002)
    # a missing file
    with pytest.raises(cg.CapowError) as e:
        cg.read_survey(str(tmp_path / "none.txt"), prm, sv, False)
    assert "cannot open input file" in str(e.value)
    # NOBJ_Max: the reference overruns its array; here it is an error
    p2, pf2 = _params_file(tmp_path, NOBJ_Max=1)
    prm2, sv2 = _read_params(pf2)
    f.write_text(row + "\n" + row + "\n")
    with pytest.raises(cg.CapowError):
        cg.read_survey(str(f), prm2, sv2, False)


@pytest.mark.parametrize("coord", [1, 2])
def test_survey_reader_angular_input(tmp_path, coord):
    """Coord_Type 1 (RA, Dec in degrees) and 2 (radians), redshift third: positions at the table's distance
    r(z) along each direction against the oracle's reader, bit for bit in float; objects of zero weight
    skipped with the reference's printed line; the redshift cut applied to the third number."""
    p, pf = _params_file(tmp_path, Coord_Type=coord, REDMININ=0.02, REDMAXIN=0.15, NOBJ_Max=10000, XMIN=-1000.0,
                         XMAX=1000.0, YMIN=-1000.0, YMAX=1000.0, ZMIN=-1000.0, ZMAX=1000.0)
    prm, sv = _read_params(pf)
    rng = np.random.default_rng(11 + coord)
    n = 3000
    scale = 180.0 / np.pi if coord == 1 else 1.0
    a = np.zeros((n, 12))
    a[:, 0] = rng.uniform(0.0, 2.0 * np.pi, n) * scale
    a[:, 1] = np.arcsin(rng.uniform(-1.0, 1.0, n)) * scale
    a[:, 2] = rng.uniform(0.0, 0.16, n)  # ~6% above REDMAXIN or below REDMININ
    a[:, 3] = rng.uniform(0.5, 1.5, n)
    a[:, 4] = 1e-4
    a[7, 2], a[7, 3] = 0.05, 0.0  # zero weight inside the redshift range: skipped and printed
    a[9, 2], a[9, 3] = 0.5, 0.0  # zero weight outside it: dropped by the cut first, silently
    f = str(tmp_path / "ang.txt")
    np.savetxt(f, a, fmt="%.17g")
    got = cg.read_survey(f, prm, sv, False)
    ref = orc.survey_read(p, f, False)
    assert got["nread"] == n and got["n"] == len(ref["x"])
    assert 0 < got["n"] < n - 100
    for k in ("x", "y", "z", "weight", "redshift"):
        assert np.array_equal(got["w" if k == "weight" else k], ref[k]), k
    r = np.sqrt(got["x"].astype(np.float64) ** 2 + got["y"] ** 2 + got["z"] ** 2)
    d = np.array([orc._survey_lib().orc_survey_distance(p.Omega_m, float(z)) for z in ref["redshift"]])
    assert np.allclose(r, d, rtol=1e-5)
    assert got["log"].splitlines() == ["%lf, %lf, %lf, %lf, %lf".replace("%lf", "%f") % tuple(a[7, :5])]


def test_survey_reader_redshift_cut_and_progress_lines(tmp_path):
    """The redshift of each object from its distance (the redshift-distance table) against the oracle's
    table, and the 'Read N objects, kept K' line every million lines."""
    p, pf = _params_file(tmp_path, REDMININ=0.05, REDMAXIN=0.1, NOBJ_Max=2_000_000, XMIN=-1000.0, XMAX=1000.0,
                         YMIN=-1000.0, YMAX=1000.0, ZMIN=-1000.0, ZMAX=1000.0)
    prm, sv = _read_params(pf)
    rng = np.random.default_rng(3)
    n = 1_000_500
    pos = rng.uniform(-900, 900, size=(n, 3))
    a = np.zeros((n, 8))
    a[:, :3] = pos
    a[:, 3] = 1.0
    a[:, 4] = 1e-4
    f = str(tmp_path / "r.txt")
    np.savetxt(f, a, fmt="%.9g")
    got = cg.read_survey(f, prm, sv, True)
    r = np.sqrt((np.loadtxt(f, max_rows=5000) ** 2)[:, :3].sum(1))
    z_orc = np.array([orc._survey_lib().orc_survey_redshift(p.Omega_m, float(v)) for v in r])
    inside = (z_orc >= 0.05) & (z_orc <= 0.1)
    assert got["nread"] == n
    kept_first = int(inside.sum())
    assert np.allclose(got["redshift"][:kept_first],
                       z_orc[inside].astype(np.float32), rtol=1e-6)
    lines = got["log"].splitlines()
    assert len(lines) == 1 and lines[0].startswith("Read 1000000 objects, kept ")


def test_survey_nbar_matches_the_oracle_and_the_reference_table(tmp_path):
    """compute_nbar (NBAR_Column < 0) on the golden catalogue that uses it: the lines the reference printed
    (the per-bin number density table), and every object's nbar against the oracle's restatement (the
    distance tables differ in the last digits, so float nbar may differ in the last bit)."""
    name = "sv_cic_nbar"
    p, pf, df, rf, d = write_survey_inputs(tmp_path, name)
    prm, sv = _read_params(pf)
    assert sv.NBAR_Column < 0
    data, rand, log = cg.read_survey_pair(df, rf, prm, sv)
    txt = open(os.path.join(os.path.dirname(__file__), "golden", f"{name}.stdout")).read().splitlines()
    at = txt.index("Calculating Number Density...")
    lines = log.splitlines()
    assert lines == txt[at: at + len(lines)]
    assert txt[at + len(lines)] == "Computing FKP Weights..."
    od, orr = orc.survey_read(p, df, False), orc.survey_read(p, rf, True)
    assert orc.survey_nbar(p, od, orr) == lines
    for mine, ref in ((data, od), (rand, orr)):
        assert np.allclose(mine["nbar"], ref["nbar"], rtol=1e-6, atol=0)
        assert np.mean(mine["nbar"] == ref["nbar"]) > 0.99


def test_survey_nbar_rejects_more_data_than_randoms(tmp_path):
    p, pf = _params_file(tmp_path, NBAR_Column=-1, REDMAXIN=0.3)
    prm, sv = _read_params(pf)
    row = "10 20 30 1.5 0.001 0 0 0 0 0 0 0\n"
    f, g = tmp_path / "d.txt", tmp_path / "r.txt"
    f.write_text(row * 3)
    g.write_text("10 20 30 1 0 0 0 0\n" * 2)
    with pytest.raises(cg.CapowError) as e:
        cg.read_survey_pair(str(f), str(g), prm, sv)
    assert e.value.status == cg.EINVAL and "randoms" in str(e.value)
