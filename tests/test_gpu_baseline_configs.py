"""GPU parity against the CPU oracle at the two benchmark configurations, full size:

* the plain run: 2,097,152 uniform float64 particles in L = 1000 Mpc/h, CIC on a 128^3 grid, interlaced,
  LOS = z (RSD shift), density P0/P2/P4 in bins of 0.01 h/Mpc to k = 0.41 (one reference run,
  Momentum 0);
* the headline workload: a 256^3 Zel'dovich lattice (16,777,216 float32 particles), TSC on a 512^3
  grid, interlaced, LOS = z, dd / dp / pp from one paint against the three reference runs
  Momentum 0, 1 and 2 (each a single-threaded oracle process, run side by side).

Mode counts bit-exact, NGRID / NOUT / NREAD equal, P_l within the tolerances of parity_util (FP32:
1e-4 for l = 0, 1e-3 for l = 2, 4; FP64: 1e-10), dp normalised by sqrt(P_dd P_pp) of the bin.
"""
import os

import numpy as np
import pytest

import capow_gb300 as cg
import oracle as orc
from capow_gb300 import synth
from parity_util import assert_spectrum

pytestmark = pytest.mark.gpu

PLAIN = dict(NX=128, NY=128, NZ=128, XMIN=0.0, XMAX=1000.0, YMIN=0.0, YMAX=1000.0, ZMIN=0.0, ZMAX=1000.0,
             InterpOrder=2, DoInterlacing=1, NK=41, NMU=1, Mink=0.0, Maxk=0.41, Omega_m=0.3089, Redshift=0.1,
             LOS=3, Momentum=0, Odd_Multipoles=0)
HEADLINE = dict(PLAIN, NX=512, NY=512, NZ=512, InterpOrder=3, NK=161, Maxk=1.61)


def _check_counts(st, ref_stats, label):
    for k in ("nread", "nout", "ngrid"):
        assert st[k] == ref_stats[k], f"{label}: {k} {st[k]} vs {ref_stats[k]}"


@pytest.fixture(scope="module")
def plain_case():
    parts = synth.uniform(2097152, L=1000.0, sigma_v=300.0, seed=1)
    po = orc.Params(**PLAIN)
    ref = orc.run(po, *parts, momentum=0, fft=orc.fft_scipy)
    ref.pop("grids")
    return parts, ref


@pytest.mark.parametrize("precision", ["fp32", "fp64", "det"])
def test_plain_run_against_oracle(gpu, plain_case, precision):
    parts, ref = plain_case
    x, y, z, vx, vy, vz = parts
    with cg.PowerSpectrum(cg.Params(**PLAIN), precision=precision) as ps:
        ps.paint(x, y, z, vz)
        st = ps.stats()
        r = ps.power()[0]
    label = f"plain 128^3 CIC {precision}"
    _check_counts(st, ref["stats"], label)
    assert abs(r["norm"] - ref["normf"]) <= 1e-12 * ref["normf"], label
    assert abs(r["shot"] - ref["shot"]) <= 1e-12 * ref["shot"], label
    err = assert_spectrum(r, ref["raw"], np.abs(ref["raw"]["Pk0"]), precision, odd=False, label=label)
    print(label, {f"l{k}": f"{v:.2e}" for k, v in err.items()})


@pytest.fixture(scope="module")
def headline_case(tmp_path_factory):
    parts = synth.zeldovich(256, L=1000.0, mesh=512, rms_cells=1.5, seed=2)
    path = os.path.join(str(tmp_path_factory.mktemp("headline")), "parts.npz")
    orc.save_particles(path, *parts)
    with orc.ParallelRuns(3) as pool:
        out = pool.run(orc.Params(**HEADLINE), path, [0, 1, 2], timeout=1800)
    return parts, {m: out[m][0] for m in (0, 1, 2)}


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_headline_workload_against_oracle(gpu, headline_case, precision):
    parts, refs = headline_case
    x, y, z, vx, vy, vz = parts
    with cg.PowerSpectrum(cg.Params(**HEADLINE), precision=precision, spectra=["dd", "dp", "pp"]) as ps:
        ps.paint(x, y, z, vz)
        st = ps.stats()
        res = ps.power()
    label = f"headline 512^3 TSC {precision}"
    for m in (0, 1, 2):
        _check_counts(st, refs[m]["stats"], label)
    dd, pp = np.abs(refs[0]["raw"]["Pk0"]), np.abs(refs[2]["raw"]["Pk0"])
    for r, m, norm0 in zip(res, (0, 1, 2), (dd, np.sqrt(dd * pp), pp)):
        assert abs(r["norm"] - refs[m]["normf"]) <= 1e-12 * refs[m]["normf"], label
        err = assert_spectrum(r, refs[m]["raw"], norm0, precision, odd=False, label=f"{label} {r['kind']}")
        print(label, r["kind"], {f"l{k}": f"{v:.2e}" for k, v in err.items()})
    # the shot noise of the momentum spectra uses the FP32 velocity moments: bound its effect on P0
    for r, m, norm0 in zip(res, (0, 1, 2), (dd, np.sqrt(dd * pp), pp)):
        nm = np.asarray(refs[m]["raw"]["Nmodes"], dtype=np.float64)
        k = nm > 0
        moved = np.max(np.abs(r["shot"] - refs[m]["shot"]) * nm[k] / norm0[k])
        assert moved <= (1e-10 if precision == "fp64" else 1e-5), (label, r["kind"], moved)
