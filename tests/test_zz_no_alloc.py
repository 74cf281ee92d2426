"""capow_paint_noalloc (the paint with its scratch in a fixed device array) against capow_paint:
the same grids, statistics and spectra on two calls in a row with different catalogues, no change
in free device memory across a call, and the size limit. Collected last, so it runs both alone in
a fresh process and after every other test."""
import re

import numpy as np
import pytest

import capow_gb300 as cg
from parity_util import particles, vlos_of

pytestmark = pytest.mark.gpu

BASE = dict(XMIN=-3.0, XMAX=997.0, YMIN=0.0, YMAX=1000.0, ZMIN=10.0, ZMAX=510.0, NK=24, Maxk=0.55, NMU=5,
            Odd_Multipoles=1, DoInterlacing=1)


def _device(parts, los, gpu):
    import torch

    x, y, z, vx, vy, vz = parts
    v = vlos_of(los, vx, vy, vz)
    return [torch.tensor(np.ascontiguousarray(a), device=gpu) for a in (x, y, z, v)]


def _grids(ps, nfields):
    return [ps.grid(w) for w in ((0, 1) if nfields == 1 else (0, 1, 2, 3))]


@pytest.mark.parametrize("precision,order,los,mom", [("det", 3, 3, 1), ("fp32", 2, 0, 0), ("fp32", 3, 3, 2)])
def test_noalloc_matches_paint_twice(gpu, precision, order, los, mom):
    import torch

    p = cg.Params(NX=64, NY=48, NZ=40, InterpOrder=order, LOS=los, Momentum=mom, **BASE)
    nfields = 2 if mom == 1 else 1
    with cg.PowerSpectrum(p, precision) as ref, cg.PowerSpectrum(p, precision) as na:
        # ascending sizes: the second, larger catalogue is the one capow_paint would grow its buffers for
        for call, (n, seed) in enumerate(((40000, 31), (150000, 32))):
            dev = _device(particles(p, n, seed), los, gpu)
            ref.paint(*dev)
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            na.paint_noalloc(*dev)
            s_na = na.stats()
            free1 = torch.cuda.mem_get_info()[0]
            if call == 1:  # the first call loads the array; later calls must leave free memory as it was
                assert free1 == free0, f"free device memory changed by {free0 - free1} bytes"
            s_ref = ref.stats()
            label = f"{precision} order={order} los={los} mom={mom} call={call}"
            for k in ("nread", "nout", "ngrid"):
                assert s_na[k] == s_ref[k], f"{label}: {k}"
            for k in ("nsq",):
                assert s_na[k] == pytest.approx(s_ref[k], rel=1e-9, abs=1e-9), f"{label}: {k}"
            assert np.allclose(s_na["vr"], s_ref["vr"], rtol=1e-6, atol=1e-3), label
            for q, (a, b) in enumerate(zip(_grids(na, nfields), _grids(ref, nfields))):
                if precision == "det":
                    assert np.array_equal(a, b), f"{label}: grid {q} differs"
                else:
                    scale = max(np.abs(b).max(), 1e-30)
                    assert np.abs(a - b).max() <= 1e-5 * scale, f"{label}: grid {q}"
            r_na, r_ref = na.power()[0], ref.power()[0]
            assert np.array_equal(r_na["Nmodes"], r_ref["Nmodes"]), label
            for l in range(5):
                a, b = r_na[f"Pk{l}"], r_ref[f"Pk{l}"]
                # the bin stage adds FP32 per-CTA partials in whatever order the CTAs run, so the
                # spectra agree to FP32 rounding even where the grids are bit-identical (det)
                scale = np.abs(r_ref["Pk0"]).max()
                assert np.abs(a - b).max() <= 1e-5 * scale, f"{label}: Pk{l}"
            assert r_na["shot"] == pytest.approx(r_ref["shot"], rel=1e-9), label


def test_noalloc_rejects_beyond_limit(gpu):
    import torch

    p = cg.Params(NX=64, NY=64, NZ=64, InterpOrder=3, LOS=0, Momentum=0, **BASE)
    with cg.PowerSpectrum(p, "fp32") as ps, cg.PowerSpectrum(p, "fp32") as ref:
        big = 1_200_000  # well beyond the limit: real device arrays, so nothing is read out of bounds either way
        rng = np.random.default_rng(5)
        pos = [torch.tensor(rng.uniform(lo, hi, big), device=gpu)
               for lo, hi in ((p.XMIN, p.XMAX), (p.YMIN, p.YMAX), (p.ZMIN, p.ZMAX))]
        with pytest.raises(cg.CapowError) as e:
            ps.paint_noalloc(*pos)
        assert e.value.status == cg.EINVAL
        m = re.search(r"at most (\d+) particles fit", str(e.value))
        assert m, str(e.value)
        fit = int(m.group(1))
        assert 100_000 < fit < big
        # exactly the limit is accepted, allocates nothing and matches capow_paint
        sub = [a[:fit].contiguous() for a in pos]
        ps.paint_noalloc(*[a[:1000] for a in sub])  # loads the array on this device before the measured call
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        ps.paint_noalloc(*sub)
        ps.stats()
        assert torch.cuda.mem_get_info()[0] == free0
        ref.paint(*sub)
        s, r = ps.stats(), ref.stats()
        assert s["nread"] == fit and s["ngrid"] == r["ngrid"]
        a, b = ps.grid(0), ref.grid(0)
        assert np.abs(a - b).max() <= 1e-5 * np.abs(b).max()


def test_noalloc_argument_errors(gpu):
    import torch

    p = cg.Params(NX=32, NY=32, NZ=32, InterpOrder=2, LOS=0, Momentum=0, **BASE)
    x = np.linspace(1.0, 900.0, 100)
    with cg.PowerSpectrum(p, "fp64") as ps:  # FP64 contexts have no tile scratch to replace
        d = torch.tensor(x, device=gpu)
        with pytest.raises(cg.CapowError) as e:
            ps.paint_noalloc(d, d, d)
        assert e.value.status == cg.ENOTSUP
    with cg.PowerSpectrum(p, "fp32") as ps:
        with pytest.raises(ValueError):
            ps.paint_noalloc(x, x, x)  # host arrays: refused before the C call
        pc = cg._Particles(len(x), cg.F64, 0, x.ctypes.data, x.ctypes.data, x.ctypes.data, None, None)
        import ctypes

        rc = cg.lib().capow_paint_noalloc(ps._ctx, ctypes.byref(pc))
        assert rc == cg.EINVAL
        assert "device-resident" in cg.lib().capow_last_error(ps._ctx).decode()
        # pinned host memory handed over as if it were device memory: refused by its pointer attributes
        h = torch.tensor(x).pin_memory()
        pc = cg._Particles(len(x), cg.F64, 1, h.data_ptr(), h.data_ptr(), h.data_ptr(), None, None)
        rc = cg.lib().capow_paint_noalloc(ps._ctx, ctypes.byref(pc))
        assert rc == cg.EINVAL
        assert "not device memory" in cg.lib().capow_last_error(ps._ctx).decode()
