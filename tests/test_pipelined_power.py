"""capow_power_enqueue / capow_power_result: a stream of host catalogues through one context, each
catalogue's chunked copy (>= 4M particles) overlapping the previous catalogue's power stage. The spectra
equal those of capow_power on each catalogue in a context of its own; the context refuses every other
call while a power stage is pending; a catalogue whose buckets overflow is repainted by
capow_power_result while the next catalogue's paint is queued behind it, and both come out right."""
import numpy as np
import pytest

import capow_gb300 as cg

pytestmark = pytest.mark.gpu

P = dict(NX=64, NY=64, NZ=64, NK=20, Maxk=0.3, XMIN=0.0, XMAX=1000.0, YMIN=0.0, YMAX=1000.0, ZMIN=0.0,
         ZMAX=1000.0, InterpOrder=3, DoInterlacing=1, LOS=3, Momentum=1)
SPECTRA = ["dd", "dp", "pp"]


def catalogue(seed, n=4_500_000, clump=0.0):
    """Uniform float32 particles (host arrays), a fraction `clump` of them packed into a 3-cell cube."""
    rng = np.random.default_rng(seed)
    x, y, z = (rng.uniform(2.0, 998.0, n).astype(np.float32) for _ in range(3))
    v = rng.normal(0.0, 100.0, n).astype(np.float32)
    if clump:
        m, d = int(n * clump), 1000.0 / 64
        for a, c in zip((x, y, z), (370.0, 410.0, 430.0)):
            a[:m] = (c + rng.uniform(-1.5, 1.5, m) * d).astype(np.float32)
    return [x, y, z, v]


def one_by_one(p, cats, precision="fp32"):
    out = []
    for c in cats:
        with cg.PowerSpectrum(p, precision=precision, spectra=SPECTRA) as ps:
            ps.paint(*c)
            out.append(ps.power())
    return out


def pipelined(p, cats, precision="fp32"):
    out = []
    with cg.PowerSpectrum(p, precision=precision, spectra=SPECTRA) as ps:
        ps.paint(*cats[0])
        for i in range(len(cats)):
            ps.power_enqueue()
            if i + 1 < len(cats):
                ps.paint(*cats[i + 1])
            out.append(ps.power_result())
    return out


def assert_same(got, ref, label, scalar_tol=1e-12):
    """The same evaluation twice: equal counts and scalars; bin sums equal up to the order in which the
    bin kernel's FP32 block sums meet (1e-5 of the largest monopole sum; a clumped catalogue's
    cancelling quadrupole sums show a few 1e-6 of it)."""
    for i, (rg, rr) in enumerate(zip(got, ref)):
        for q in range(len(rr)):
            assert np.array_equal(rg[q]["Nmodes"], rr[q]["Nmodes"]), (label, i, q)
            for key in ("shot", "norm", "alpha"):
                assert abs(rg[q][key] - rr[q][key]) <= scalar_tol * abs(rr[q][key]), (label, i, q, key)
            scale = np.abs(np.asarray(rr[q]["Pk0"])).max()
            for l in (0, 2, 4):
                a, b = np.asarray(rg[q][f"Pk{l}"]), np.asarray(rr[q][f"Pk{l}"])
                assert np.abs(a - b).max() <= 1e-5 * scale, (label, i, q, l)


def test_pipelined_catalogues_match_one_context_each(gpu):
    cats = [catalogue(s) for s in (11, 12, 13)]
    assert_same(pipelined(cg.Params(**P), cats), one_by_one(cg.Params(**P), cats), "pipelined")


@pytest.mark.parametrize("precision", ["fp64", "det"])
def test_pipelined_other_precisions(gpu, precision):
    """FP64 and the deterministic mode, with catalogues small enough to be copied on the context's stream
    (no chunks): the staging sets alternate all the same."""
    cats = [catalogue(s, n=300_000) for s in (41, 42, 43)]
    assert_same(pipelined(cg.Params(**P), cats, precision), one_by_one(cg.Params(**P), cats, precision), precision)


def test_pipelined_state_rules(gpu):
    p = cg.Params(**P)
    cats = [catalogue(s, n=200_000) for s in (21, 22)]

    def refused(f, *a):
        with pytest.raises(cg.CapowError) as e:
            f(*a)
        assert e.value.status == cg.ESTATE

    with cg.PowerSpectrum(p, precision="fp32", spectra=SPECTRA) as ps:
        refused(ps.power_result)
        ps.paint(*cats[0])
        ps.power_enqueue()
        for f in (ps.power_enqueue, ps.power, ps.stats, ps.stage_ms):
            refused(f)
        refused(ps.grid, 0)
        ps.paint(*cats[1])
        refused(ps.paint, *cats[0])  # one paint at most behind a pending power stage
        r0 = ps.power_result()
        refused(ps.power_result)
        r1 = ps.power()  # the queued catalogue
    assert_same([r0, r1], one_by_one(p, cats), "state rules")


def test_overflow_with_a_paint_queued_behind(gpu):
    """The first catalogue's clump fills the bucket overflow list: capow_power_result switches the context
    to the two-pass paint, repaints that catalogue from its staging buffer, redoes its power stage and
    paints the queued catalogue again. From then on the context paints in two passes, whose FP32
    statistics sums (the velocity moment of the dp shot noise) add in another order than a fresh
    context's one-pass buckets: the scalars agree to FP32 rounding of those sums."""
    p = cg.Params(**P)
    cats = [catalogue(31, clump=0.3), catalogue(32), catalogue(33, clump=0.3)]
    assert_same(pipelined(p, cats), one_by_one(p, cats), "overflow", scalar_tol=1e-5)
