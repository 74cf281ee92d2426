"""The drop-in boundary on CPU: the C-ABI library loads and exports every entry point of
include/capow.h; the parameter-file reader, catalogue reader and output writer behave like the
reference (messages and bytes compared with the reference's own stdout and output files)."""
import ctypes
import json
import os
import re
import subprocess

import numpy as np
import pytest

import capow_gb300 as cg
import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLD = os.path.join(HERE, "golden")
ERRS = json.load(open(os.path.join(GOLD, "param_errors.json")))
MANIFEST = json.load(open(os.path.join(GOLD, "manifest.json")))


@pytest.fixture(scope="module", autouse=True)
def _built(built):
    return built


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "capow.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(capow_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_header_symbol():
    L = cg.lib()
    syms = header_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(L, s), f"{s} declared in include/capow.h but not exported"
    out = subprocess.run(["nm", "-D", "--defined-only", cg.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (capow_\w+)", out))
    assert set(syms) <= exported
    assert set(cg.EXPORTS) == set(syms)


def test_strerror_and_status_codes():
    L = cg.lib()
    assert L.capow_strerror(0) == b"ok"
    assert b"bounds" in L.capow_strerror(cg.EBOUNDS)
    assert L.capow_strerror(99) == b"unknown status"


def test_create_without_device_reports_status_not_crash():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(cg.CapowError) as e:
        cg.PowerSpectrum(cg.Params(NX=8, NY=8, NZ=8), precision="fp32")
    assert e.value.status == cg.ECUDA


def test_create_rejects_bad_params_before_touching_the_device():
    for bad in (dict(LOS=7), dict(InterpOrder=4), dict(NK=0), dict(XMAX=-1.0), dict(Maxk=-1.0), dict(Momentum=9),
                dict(Output2D=1, NMU=0)):
        kw = dict(NX=8, NY=8, NZ=8)
        kw.update(bad)
        with pytest.raises(cg.CapowError) as e:
            cg.PowerSpectrum(cg.Params(**kw))
        assert e.value.status == cg.EINVAL, bad


@pytest.mark.parametrize("case", [k for k in ERRS if k not in ("usage", "catalogue_bad_line",
                                                                 "catalogue_out_of_box", "comments_and_short_lines")])
def test_param_errors_match_reference_messages(tmp_path, case):
    e = ERRS[case]
    pf = tmp_path / "p.dat"
    pf.write_text("\n".join(e["lines"]) + "\n")
    with pytest.raises(cg.CapowError) as err:
        cg.read_params(str(pf))
    ref = e["stdout"].replace("{PARAMFILE}", str(pf))
    banner = "\nReading Input Parameters and setting up CAPOW\n=============================================\n"
    assert ref.startswith(banner)
    assert str(err.value) == ref[len(banner):], case


def test_params_comments_short_lines_and_values(tmp_path):
    e = ERRS["comments_and_short_lines"]
    pf = tmp_path / "p.dat"
    pf.write_text("\n".join(e["lines"]) + "\n")
    p = cg.read_params(str(pf))
    assert (p.NX, p.NY, p.NZ) == (8, 8, 8) and p.XMIN == -3.0 and p.ZMAX == 510.0
    for name, m in MANIFEST.items():  # every golden case's file parses to the same values
        po = orc.Params(**m["params"])
        f = tmp_path / f"{name}.dat"
        po.write_file(str(f))
        q = cg.read_params(str(f))
        for k, v in m["params"].items():
            assert getattr(q, k) == v, (name, k)


def test_params_missing_file():
    with pytest.raises(cg.CapowError) as e:
        cg.read_params("/nonexistent/run_parameters.dat")
    assert "not found" in str(e.value) and "Fatal Error at line 330" in str(e.value)


def test_catalogue_reader_matches_numpy(tmp_path):
    rng = np.random.default_rng(3)
    a = rng.normal(0, 300, (5000, 6))
    f = tmp_path / "cat.txt"
    with open(f, "w") as fh:
        fh.write("# header line\n")
        np.savetxt(fh, a, fmt="%.17g")
        fh.write("# trailing comment\n")
    for los, col in ((0, 5), (1, 3), (2, 4), (3, 5)):
        x, y, z, v = cg.read_catalogue(str(f), los)
        assert np.array_equal(x, a[:, 0]) and np.array_equal(y, a[:, 1]) and np.array_equal(z, a[:, 2])
        assert np.array_equal(v, a[:, col])


def test_catalogue_reader_large_parallel(tmp_path):
    rng = np.random.default_rng(4)
    a = rng.uniform(0, 1000, (200000, 6))
    f = tmp_path / "big.txt"
    np.savetxt(f, a, fmt="%.9g")
    x, y, z, v = cg.read_catalogue(str(f), 3)
    ref = np.loadtxt(f)
    assert np.array_equal(x, ref[:, 0]) and np.array_equal(v, ref[:, 5])


def test_catalogue_number_parsing_is_correctly_rounded(tmp_path):
    """The reader's fast path (exact mantissa and power of ten) and its strtod fallback both give the
    correctly rounded double of every token, as the reference's sscanf("%lf") does: against Python's
    float() over many formats, signs, exponent ranges, long mantissas, subnormals, hex and inf/nan."""
    rng = np.random.default_rng(11)
    vals = np.concatenate([rng.normal(0, 300, 4000), rng.uniform(-1e-3, 1e-3, 2000),
                           10.0 ** rng.uniform(-310, 308, 2000) * rng.choice([-1.0, 1.0], 2000),
                           rng.integers(-(1 << 60), 1 << 60, 1000).astype(np.float64)])
    toks = []
    fmts = ["%.9g", "%.17g", "%.6f", "%.3e", "%.15e", "%g", "%.20g", "%.25f", "%+.8f"]
    for i, v in enumerate(vals):
        toks.append(fmts[i % len(fmts)] % v)
    toks += ["0", "-0", "-0.0", "+0.5", ".5", "5.", "-.25", "1e5", "1.E-5", "1e+22", "1e23", "9007199254740993",
             "9007199254740992", "123456789012345678901234", "0.1", "0.3", "2.2250738585072011e-308",
             "4.9e-324", "1e-400", "1.7976931348623157e308", "0x1.8p3", "-0X10", "inf", "-Infinity", "nan",
             "00000000000000000000000123.5", "0.000000000000000000000000000123", "7e-22", "7e22", "3.0e-23"]
    while len(toks) % 6:
        toks.append("1")
    f = tmp_path / "nums.txt"
    with open(f, "w") as fh:
        for k in range(0, len(toks), 6):
            fh.write(" ".join(toks[k:k + 6]) + "\n")
    x, y, z, v = cg.read_catalogue(str(f), 1)  # LOS 1: the fourth column
    got = np.stack([x, y, z, v], axis=1).ravel()
    ref = np.array([float.fromhex(t) if "x" in t.lower() else float(t) for t in toks]).reshape(-1, 6)[:, :4].ravel()
    same = (got.view(np.uint64) == ref.view(np.uint64)) | (np.isnan(got) & np.isnan(ref))
    assert same.all(), [(toks[6 * (i // 4) + i % 4], got[i], ref[i]) for i in np.nonzero(~same)[0][:5]]


def test_catalogue_long_mantissas_and_near_ties(tmp_path):
    """Up to 19 significant digits over the whole exponent range (the Eisel-Lemire path), decimals
    cut from the exact midpoints between adjacent doubles (and one unit either side), and exact ties
    that fit in 19 digits: bit-identical to correctly rounded parsing (Python's float())."""
    import random
    import struct
    from decimal import Decimal, getcontext
    getcontext().prec = 1200
    rnd = random.Random(7)
    toks = []
    for _ in range(60000):
        nd = rnd.randint(15, 19)
        toks.append(f"{rnd.randint(10 ** (nd - 1), 10 ** nd - 1)}e{rnd.randint(-345, 310)}")
    for _ in range(8000):
        d = struct.unpack("<d", struct.pack("<Q", rnd.getrandbits(63)))[0]
        if not 2.3e-308 < abs(d) < 1.7e308:
            continue
        mid = (Decimal(d) + Decimal(float(np.nextafter(d, np.inf)))) / 2
        for nd in (17, 18, 19):
            t = f"{mid:.{nd - 1}e}"
            mant, ex = t.split("e")
            k = int(mant.replace(".", ""))
            toks += [t, f"{k - 1}e{int(ex) - (nd - 1)}", f"{k + 1}e{int(ex) - (nd - 1)}"]
    toks += [str((2 ** 53 + o) * 2 ** k) for k in range(0, 10) for o in range(1, 400, 2)]
    while len(toks) % 6:
        toks.append("1")
    f = tmp_path / "long.txt"
    with open(f, "w") as fh:
        for k in range(0, len(toks), 6):
            fh.write(" ".join(toks[k:k + 6]) + "\n")
    x, y, z, v = cg.read_catalogue(str(f), 1)
    got = np.stack([x, y, z, v], axis=1).ravel()
    ref = np.array([float(t) for t in toks]).reshape(-1, 6)[:, :4].ravel()
    bad = np.nonzero(got.view(np.uint64) != ref.view(np.uint64))[0]
    assert bad.size == 0, [(toks[6 * (i // 4) + i % 4], got[i], ref[i]) for i in bad[:5]]


def test_catalogue_bad_line_message(tmp_path):
    e = ERRS["catalogue_bad_line"]
    f = tmp_path / "bad.txt"
    f.write_text(e["catalogue"])
    with pytest.raises(cg.CapowError) as err:
        cg.read_catalogue(str(f), 0)
    ref_tail = e["stdout"].split("Reading: {DATAFILE}\n", 1)[1]
    assert str(err.value) == ref_tail


def test_catalogue_blank_line_is_an_error(tmp_path):
    f = tmp_path / "blank.txt"
    f.write_text("1 2 3 4 5 6\n\n1 2 3 4 5 6\n")
    with pytest.raises(cg.CapowError):
        cg.read_catalogue(str(f), 0)


@pytest.mark.parametrize("name", sorted(MANIFEST))
def test_normalise_and_writer_reproduce_reference_file(tmp_path, name):
    """capow_normalise + capow_write_output on the reference's raw sums print its file byte for byte."""
    d = dict(np.load(os.path.join(GOLD, f"{name}.npz")))
    po = orc.Params(**MANIFEST[name]["params"])
    pc = cg.Params(**MANIFEST[name]["params"])
    st = orc.run(po, d["x"], d["y"], d["z"], d["vx"], d["vy"], d["vz"])
    s = cg._Spectrum()
    arrs = {k: np.array(d[k], dtype=np.float64) for k in ("Pk0", "Pk1", "Pk2", "Pk3", "Pk4")}
    nm = np.array(d["Nmodes"], dtype=np.int64)
    for l in range(5):
        s.pk[l] = arrs[f"Pk{l}"].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    s.nmodes = nm.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    if pc.Output2D:
        p2 = np.array(d["Pk_2D"], dtype=np.float64)
        n2 = np.array(d["Nmodes_2D"], dtype=np.int64)
        s.pk2d = p2.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        s.nmodes2d = n2.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    s.shot, s.norm = st["shot"], st["normf"]
    pcc = pc.to_c()
    assert cg.lib().capow_normalise(ctypes.byref(pcc), ctypes.byref(s)) == 0
    assert s.last_bin == st["last"]
    out = tmp_path / "out.txt"
    assert cg.lib().capow_write_output(str(out).encode(), ctypes.byref(pcc), ctypes.byref(s)) == 0
    assert out.read_text() == open(os.path.join(GOLD, f"{name}.out")).read()


def test_driver_usage_message():
    r = subprocess.run([cg.DRIVER_PATH, "only-one-arg"], capture_output=True, text=True)
    assert r.returncode == 1
    assert r.stdout == ERRS["usage"]["stdout"]


@pytest.mark.parametrize("case", ["bad_los", "missing_tag", "duplicate_tag", "nmu_2d"])
def test_driver_param_errors_print_reference_stdout(tmp_path, case):
    e = ERRS[case]
    pf = tmp_path / "p.dat"
    pf.write_text("\n".join(e["lines"]) + "\n")
    r = subprocess.run([cg.DRIVER_PATH, str(pf), "data.txt", "none", str(tmp_path / "o.txt")], capture_output=True,
                       text=True)
    assert r.returncode == 1
    assert r.stdout == e["stdout"].replace("{PARAMFILE}", str(pf))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("los", [0, 1, 2, 3])
def test_soa_catalogue_round_trip(tmp_path, dtype, los):
    """The binary column catalogue the driver reads instead of text: x, y, z and the LOS column, bit for
    bit, in the file's dtype; a text file is not taken for one; a truncated file is an error."""
    rng = np.random.default_rng(los)
    cols = [rng.uniform(0, 1000, 1001).astype(dtype) for _ in range(6)]
    f = str(tmp_path / "c.bin")
    cg.write_soa_catalogue(f, *cols, dtype=dtype)
    assert cg.lib().capow_is_soa_catalogue(f.encode()) == 1
    x, y, z, v = cg.read_catalogue_soa(f, los)
    assert x.dtype == dtype
    for a, b in zip((x, y, z, v), cols[:3] + [cols[3 if los == 1 else (4 if los == 2 else 5)]]):
        assert np.array_equal(a, b)
    t = tmp_path / "c.txt"
    t.write_text("1 2 3 4 5 6\n")
    assert cg.lib().capow_is_soa_catalogue(str(t).encode()) == 0
    raw = open(f, "rb").read()
    open(f, "wb").write(raw[:-8])
    with pytest.raises(cg.CapowError) as e:
        cg.read_catalogue_soa(f, los)
    assert "truncated" in str(e.value)
