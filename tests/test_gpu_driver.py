"""The drop-in command-line driver end to end on the GPU: `capow <ParameterFile> <DataFile> <RandomFile>
<OutputFile>` on each golden catalogue (written as the reference read it: `x y z vx vy vz`, %.17g),
against the unmodified reference's own stdout and output file for that catalogue.

The path under test is the whole periodic branch of main (src/main.c:28-298): parameter file,
catalogue reader, paint from pageable float64 host arrays, FFT, binning, output_power's arithmetic
and file format. FP64: stdout byte for byte, the output file token for token (but for roundoff-level
entries of cancelling sums, which depend on the summation order). FP32: the same lines, every number within
the FP32 path's tolerance, Nmodes and counts exact. The cases cover NN/CIC/TSC, LOS 0-3, interlacing,
odd multipoles, the 2-D output, log bins and Momentum 0, 1, 2, 4 and 8."""
import json
import os
import re
import subprocess

import numpy as np
import pytest

import capow_gb300 as cg
import oracle as orc

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MANIFEST = json.load(open(os.path.join(GOLD, "manifest.json")))
NUM = re.compile(r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?")


def _run_driver(tmp_path, name, precision):
    m = MANIFEST[name]
    d = np.load(os.path.join(GOLD, f"{name}.npz"))
    po = orc.Params(**m["params"])
    pf, df, of = (str(tmp_path / f) for f in ("params.dat", "data.txt", "out.txt"))
    po.write_file(pf)
    orc.write_catalogue(df, d["x"], d["y"], d["z"], d["vx"], d["vy"], d["vz"])
    env = dict(os.environ, CAPOW_PRECISION=precision)
    r = subprocess.run([cg.DRIVER_PATH, pf, df, "none", of], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    gold_stdout = open(os.path.join(GOLD, f"{name}.stdout")).read().replace("{DATAFILE}", df).replace("{OUTFILE}", of)
    gold_out = open(os.path.join(GOLD, f"{name}.out")).read()
    return r.stdout, gold_stdout, open(of).read(), gold_out


def _same_text_close_numbers(got: str, want: str, rtol: float, label: str):
    """Line for line equal once the numbers are taken out; every number within rtol of the reference's."""
    gl, wl = got.splitlines(), want.splitlines()
    assert len(gl) == len(wl), label
    for a, b in zip(gl, wl):
        assert NUM.sub("#", a) == NUM.sub("#", b), (label, a, b)
        for x, y in zip(NUM.findall(a), NUM.findall(b)):
            fx, fy = float(x), float(y)
            assert abs(fx - fy) <= rtol * abs(fy) + 1e-300, (label, a, b)


def _output_close(got: str, want: str, odd: bool, label: str):
    """The output file: header lines equal to 5 significant digits; per row k and Nmodes exact, each
    multipole within 1e-4 (l = 0) / 1e-3 (l > 0) of the row's scale (its largest |P| plus shot/norm),
    plus the %g rounding of the printed value."""
    gl, wl = got.splitlines(), want.splitlines()
    assert len(gl) == len(wl), label
    shot = float(wl[0].split("=")[1])
    _same_text_close_numbers("\n".join(gl[:3]), "\n".join(wl[:3]), 1e-5, label)
    cols = [0, 1, 2, 3, 4] if odd else [0, 2, 4]
    for a, b in zip(gl[3:], wl[3:]):
        va, vb = [float(t) for t in a.split()], [float(t) for t in b.split()]
        assert len(va) == len(vb) == len(cols) + 2, (label, a)
        assert va[0] == vb[0] and va[-1] == vb[-1], (label, a, b)  # k centre, Nmodes
        scale = max(abs(v) for v in vb[1:-1]) + abs(shot)
        for j, l in enumerate(cols):
            tol = (1e-4 if l == 0 else 1e-3) * scale + 1e-5 * abs(vb[1 + j])
            assert abs(va[1 + j] - vb[1 + j]) <= tol, (label, l, a, b)


def _output_equal_but_roundoff(got: str, want: str, label: str):
    """The output file printed the same, token for token, except entries that are FP64 roundoff of a
    sum that cancels (odd multipoles of a symmetric bin): there both values are below 1e-9 of the row's
    largest |P| and are printed from different summation orders."""
    gl, wl = got.splitlines(), want.splitlines()
    assert gl[:3] == wl[:3] and len(gl) == len(wl), label
    for a, b in zip(gl[3:], wl[3:]):
        ta, tb = a.split(), b.split()
        assert len(ta) == len(tb), (label, a, b)
        scale = max(abs(float(t)) for t in tb[1:-1])
        for x, y in zip(ta, tb):
            if x != y:
                assert max(abs(float(x)), abs(float(y))) <= 1e-9 * scale, (label, a, b)


@pytest.mark.parametrize("name", sorted(MANIFEST))
def test_driver_fp64_reproduces_reference_stdout_and_file(gpu, tmp_path, name):
    out, gold_out_text, outfile, gold_file = _run_driver(tmp_path, name, "fp64")
    assert out == gold_out_text, name
    _output_equal_but_roundoff(outfile, gold_file, name)


@pytest.mark.parametrize("precision", ["fp32", "det"])
@pytest.mark.parametrize("name", sorted(MANIFEST))
def test_driver_fp32_matches_reference_within_tolerance(gpu, tmp_path, name, precision):
    out, gold_out_text, outfile, gold_file = _run_driver(tmp_path, name, precision)
    _same_text_close_numbers(out, gold_out_text, 1e-5, f"{name} {precision} stdout")
    _output_close(outfile, gold_file, bool(MANIFEST[name]["params"]["Odd_Multipoles"]), f"{name} {precision} file")


SURVEY = json.load(open(os.path.join(GOLD, "survey_manifest.json")))


def _run_survey_driver(tmp_path, name, precision):
    m = SURVEY[name]
    d = np.load(os.path.join(GOLD, f"{name}.npz"))
    po = orc.Params(**m["params"])
    pf, df, rf, of = (str(tmp_path / f) for f in ("params.dat", "data.txt", "rand.txt", "out.txt"))
    po.write_file(pf)
    np.savetxt(df, d["data"], fmt="%.17g")
    np.savetxt(rf, d["rand"], fmt="%.17g")
    env = dict(os.environ, CAPOW_PRECISION=precision)
    r = subprocess.run([cg.DRIVER_PATH, pf, df, rf, of], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    gold = open(os.path.join(GOLD, f"{name}.stdout")).read()
    gold = gold.replace("{DATAFILE}", df).replace("{RANDFILE}", rf).replace("{OUTFILE}", of)
    return r.stdout, gold, open(of).read(), open(os.path.join(GOLD, f"{name}.out")).read(), po, d


def _output_nonfinite(got: str, want: str, raw, odd: bool, rel: float, label: str):
    """An output file with norm = 0 (survey Momentum 3, as the reference computes it): every multipole of
    a bin with modes prints as inf, -inf or nan. Header lines equal; per row the k centre and Nmodes equal;
    each entry prints the same where the reference's raw sum for it is clearly signed (above rel of the
    largest raw |P| within two bins); a nan matches a nan of either sign (0/0 gives -nan on x86-64 and nan
    on AArch64); an entry whose raw sum is a rounding-level zero only has to be non-finite."""
    gl, wl = got.splitlines(), want.splitlines()
    assert gl[:3] == wl[:3] and len(gl) == len(wl), label
    cols = [0, 1, 2, 3, 4] if odd else [0, 2, 4]
    allp = np.abs(np.array([raw[f"Pk{l}"] for l in cols]))
    for b, (a, c) in enumerate(zip(gl[3:], wl[3:])):
        ta, tc = a.split(), c.split()
        assert len(ta) == len(tc) == len(cols) + 2 and ta[0] == tc[0] and ta[-1] == tc[-1], (label, a, c)
        r = np.array([raw[f"Pk{l}"][b] for l in cols])
        scale = allp[:, max(0, b - 2):b + 3].max()
        for j in range(len(cols)):
            if ta[1 + j] == tc[1 + j]:
                continue
            x, y = float(ta[1 + j]), float(tc[1 + j])
            assert not np.isfinite(x) and not np.isfinite(y), (label, a, c)
            if np.isnan(x) and np.isnan(y):
                continue
            if abs(r[j]) > rel * scale:
                assert x == y, (label, cols[j], a, c)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", sorted(SURVEY))
def test_driver_survey_reproduces_reference_stdout_and_file(gpu, tmp_path, name, precision):
    """The survey branch of main (Periodic 0, Survey 1) on the golden survey catalogues: the reader's
    counts and ranges, the FKP line, the gridded counters, alpha, shot noise and normalisation, the
    multipole banners with the reference's index lines, and the output file. stdout is byte for byte in
    both precisions (the weight sums are FP64 in both); the file token for token (FP64) or within the FP32
    path's tolerance."""
    out, gold, outfile, gold_file, po, d = _run_survey_driver(tmp_path, name, precision)
    assert out == gold, name
    if not np.isfinite(float(gold_file.splitlines()[0].split("=")[1])):
        _output_nonfinite(outfile, gold_file, d, bool(po.Odd_Multipoles), 1e-9 if precision == "fp64" else 1e-3,
                          name)
    elif precision == "fp64":
        _output_equal_but_roundoff(outfile, gold_file, name)
    else:
        _output_close(outfile, gold_file, bool(po.Odd_Multipoles), name)
