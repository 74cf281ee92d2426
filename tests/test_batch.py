"""capow_batch: mocks of different boxes, grids and interpolation orders in one call give the spectra
of running each through its own context (direct enqueue, one CUDA graph, the tile autotuner), and a
failing mock reports its own status without disturbing the others."""
import numpy as np
import pytest

import capow_gb300 as cg
import oracle as orc
from parity_util import TOL, assert_spectrum

pytestmark = pytest.mark.gpu

GRIDS = [(32, 32, 32), (48, 40, 36), (64, 64, 64)]


def make_mocks(torch, gpu, count, seed, los=3):
    rng = np.random.default_rng(seed)
    mocks = []
    for i in range(count):
        nx, ny, nz = GRIDS[i % len(GRIDS)]
        L = float(rng.uniform(500.0, 1500.0))
        p = cg.Params(NX=nx, NY=ny, NZ=nz, XMIN=0.0, XMAX=L, YMIN=0.0, YMAX=L, ZMIN=0.0, ZMAX=L,
                      InterpOrder=2 + (i % 2), DoInterlacing=1, NK=25, Maxk=25 * 0.01 * (1000.0 / L),
                      LOS=los, Momentum=0)
        n = int(np.exp(rng.uniform(np.log(20000), np.log(200000))))
        pos = rng.uniform(0.0, L, size=(3, n))
        vz = rng.normal(0.0, 200.0, n)
        parts = tuple(torch.tensor(a, device=gpu) for a in (pos[0], pos[1], pos[2], vz)) + (None,)
        mocks.append((p, parts))
    return mocks


@pytest.mark.parametrize("graph,autotune", [(False, False), (True, False), (False, True), (True, True)])
def test_batch_matches_single_contexts(gpu, graph, autotune):
    import torch

    mocks = make_mocks(torch, gpu, 12, seed=7)
    out = cg.run_batch(mocks, precision="fp32", graph=graph, autotune=autotune)
    for (p, parts), (status, res) in zip(mocks, out):
        assert status == cg.OK
        with cg.PowerSpectrum(p, precision="fp32") as ps:
            ps.paint(*parts[:4])
            ref = ps.power()[0]
        r = res[0]
        assert np.array_equal(r["Nmodes"], ref["Nmodes"])
        assert r["shot"] == ref["shot"] and r["norm"] == ref["norm"]
        scale = np.abs(ref["Pk0"]).max()
        for l in (0, 2, 4):
            assert np.abs(r[f"Pk{l}"] - ref[f"Pk{l}"]).max() <= TOL["fp32"][0] * scale, (p, l)


def test_batch_reports_per_mock_errors(gpu):
    import torch

    mocks = make_mocks(torch, gpu, 4, seed=9, los=0)
    p, parts = mocks[1]
    x = parts[0].clone()
    x[3] = p.XMAX + 5.0  # LOS == 0: a particle outside the box is the reference's fatal error
    mocks[1] = (p, (x,) + parts[1:])
    out = cg.run_batch(mocks, precision="fp32", graph=True)
    assert [s for s, _ in out] == [cg.OK, cg.EBOUNDS, cg.OK, cg.OK]


def test_batch_mocks_match_the_oracle(gpu):
    """Mocks of three grid shapes (CIC and TSC, interlaced, LOS = z) in one capow_batch call, each against
    the CPU oracle run on its own catalogue: bit-exact mode counts, equal NGRID through the shot noise
    and normalisation, P0/P2/P4 within the FP32 tolerances."""
    import torch

    mocks = make_mocks(torch, gpu, 3, seed=13)
    out = cg.run_batch(mocks, precision="fp32", graph=True, autotune=True)
    for (p, parts), (status, res) in zip(mocks, out):
        assert status == cg.OK
        kw = {f.name: getattr(p, f.name) for f in orc.Params.__dataclass_fields__.values() if hasattr(p, f.name)}
        po = orc.Params(**kw)
        x, y, z, vz = (t.cpu().numpy() for t in parts[:4])
        zero = np.zeros_like(x)
        ref = orc.run(po, x, y, z, zero, zero, vz, momentum=0)
        r = res[0]
        assert r["shot"] == ref["shot"] and abs(r["norm"] - ref["normf"]) <= 1e-12 * ref["normf"], p
        assert_spectrum(r, ref["raw"], np.abs(ref["raw"]["Pk0"]), "fp32", odd=False, label=f"batch {p.NX}")


def test_batch_state_is_reused_across_calls(gpu):
    """capow_batch keeps its device state and instantiated graph for the next call with the same
    signature: new values in the same arrays (the graph relaunched as it is), then new arrays (the
    graph updated in place), each against single contexts; capow_batch_release frees the state and a
    later call sets it up again."""
    import torch

    mocks = make_mocks(torch, gpu, 6, seed=21)

    def check(out, mocks):
        for (p, parts), (status, res) in zip(mocks, out):
            assert status == cg.OK
            with cg.PowerSpectrum(p, precision="fp32") as ps:
                ps.paint(*parts[:4])
                ref = ps.power()[0]
            assert np.array_equal(res[0]["Nmodes"], ref["Nmodes"])
            scale = np.abs(ref["Pk0"]).max()
            for l in (0, 2, 4):
                assert np.abs(res[0][f"Pk{l}"] - ref[f"Pk{l}"]).max() <= TOL["fp32"][0] * scale, (p, l)

    check(cg.run_batch(mocks, precision="fp32", graph=True), mocks)
    for p, parts in mocks:  # same arrays, new values
        L = p.XMAX - p.XMIN
        parts[0].copy_(torch.remainder(parts[0] * 1.37 + 0.1 * L, L))
    check(cg.run_batch(mocks, precision="fp32", graph=True), mocks)
    moved = [(p, tuple(None if a is None else a.clone() for a in parts)) for p, parts in mocks]  # new arrays
    check(cg.run_batch(moved, precision="fp32", graph=True), moved)
    cg.release_batch()
    check(cg.run_batch(moved, precision="fp32", graph=False), moved)
    cg.release_batch()
