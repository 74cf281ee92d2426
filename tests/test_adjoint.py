"""capow_backward (adjoint of the multipoles) against torch autograd through a dense FP64 restatement of
the forward, against central finite differences, and FP32 against FP64 at the C3 workload size: the
density auto-spectrum, the dd + dp + pp selection (density and LOS momentum, their cross and auto
spectra) and reference Momentum runs with other fields and products. The loss is sum over the spectra,
l in {0, 2} and k of (P_l(k) - T_l(k))^2, T from a second seeded realisation."""
import numpy as np
import pytest

import capow_gb300 as cg

pytestmark = pytest.mark.gpu


def rsd_factor(p):
    return (1.0 + p.Redshift) / (100.0 * np.sqrt(p.Omega_m * (1.0 + p.Redshift) ** 3 + 1.0 - p.Omega_m))


def mode_tables(p):
    """Per half-space mode: k-bin (-1 when excluded), mu, NM * grid_cor (* 0.25 when interlaced) and
    the interlace phase, following the binning loop of src/main.c:302-468 (bin from the float
    quantity (float)(fktot - Mink) / binwidth, Nyquist cut, Hermitian weights)."""
    n = (p.NX, p.NY, p.NZ)
    d = [(p.XMAX - p.XMIN) / n[0], (p.YMAX - p.YMIN) / n[1], (p.ZMAX - p.ZMIN) / n[2]]
    f = []
    for a in range(3):
        sc = 1.0 / (np.float64(np.float32(n[a])) * d[a])
        idx = np.arange(n[a] if a < 2 else n[a] // 2 + 1)
        fr = np.where(idx <= n[a] // 2, idx, idx - n[a]).astype(np.float64) * sc if a < 2 else idx * sc
        f.append(fr)
    fx, fy, fz = np.meshgrid(f[0], f[1], f[2], indexing="ij")
    fktot = 2.0 * np.pi * np.sqrt(fx * fx + fy * fy + fz * fz)
    mu = np.where(fktot > 0, 2.0 * np.pi * fz / np.where(fktot > 0, fktot, 1.0), 0.0)
    bw = (p.Maxk - p.Mink) / p.NK
    kb = np.trunc(np.float32(fktot - p.Mink).astype(np.float64) / bw).astype(np.int64)
    ny = min(np.pi / d[0], np.pi / d[1], np.pi / d[2])
    kb = np.where((kb >= 0) & (kb < p.NK) & (fktot <= ny), kb, -1)
    ax, ay, az = np.pi * fx * d[0], np.pi * fy * d[1], np.pi * fz * d[2]
    sinc = lambda t: np.where(t != 0, np.sin(t) / np.where(t != 0, t, 1.0), 1.0)
    gc = (1.0 / (sinc(ax) * sinc(ay) * sinc(az))) ** (2 * p.InterpOrder)
    i, j, k = np.meshgrid(np.arange(n[0]), np.arange(n[1]), np.arange(n[2] // 2 + 1), indexing="ij")
    nm = np.where(k != 0, 2, np.where(j == 0, np.where((i != 0) & (i != n[0] // 2), 1, 2),
                                      np.where(i != n[0] // 2, 1, 2)))
    if p.DoInterlacing:
        gc = gc * 0.25
    kh = ax + ay + az
    return kb, mu, nm * gc, np.cos(kh) + 1j * np.sin(kh), nm


def dense_multipoles(torch, p, x, y, z, v, w, tab):
    """P0, P2 of the density field (TSC, interlaced, LOS = z), normalised as output_power does, for
    particles whose every tap lies inside the grid (then the reference deposit is plain TSC)."""
    n = p.NX
    d = (p.XMAX - p.XMIN) / n
    zs = z + v * rsd_factor(p)

    def paint(px, py, pz):
        g = torch.zeros(n * n * n, dtype=torch.float64, device=x.device)
        s = [(px - p.XMIN) / d, (py - p.YMIN) / d, (pz - p.ZMIN) / d]
        i = [torch.floor(t + 0.5).detach().long() for t in s]
        dd = [t - ii.to(t.dtype) for t, ii in zip(s, i)]
        W = [[0.5 * (0.5 - e) ** 2, 0.75 - e * e, 0.5 * (0.5 + e) ** 2] for e in dd]
        for a in range(3):
            for b in range(3):
                for c in range(3):
                    idx = ((i[0] + a - 1) * n + (i[1] + b - 1)) * n + (i[2] + c - 1)
                    g = g.index_add(0, idx, w * W[0][a] * W[1][b] * W[2][c])
        return g.view(n, n, n)

    N = w.sum()
    h = 0.5 * d
    g, gi = paint(x, y, zs), paint(x + h, y + h, zs + h)
    kb, mu, wgt, e, nm = tab
    dc = torch.zeros(kb.shape, dtype=torch.float64, device=x.device)
    dc[0, 0, 0] = 1.0
    F = torch.fft.rfftn(g)
    Fi = torch.fft.rfftn(gi)
    F = F * (1 - dc) + dc * (g.sum() - N)
    Fi = Fi * (1 - dc) + dc * (gi.sum() - N)
    Fp = F + torch.as_tensor(e, device=x.device) * Fi
    power = torch.as_tensor(wgt, device=x.device) * (Fp.real ** 2 + Fp.imag ** 2)
    m = torch.as_tensor(kb >= 0, device=x.device)
    kbt = torch.as_tensor(np.where(kb >= 0, kb, 0), device=x.device)[m]
    mut = torch.as_tensor(mu, device=x.device)[m]
    S0 = torch.zeros(p.NK, dtype=torch.float64, device=x.device).index_add(0, kbt, power[m])
    S2 = torch.zeros(p.NK, dtype=torch.float64, device=x.device).index_add(0, kbt, power[m] * (1.5 * mut ** 2 - 0.5))
    Nm = np.zeros(p.NK)
    np.add.at(Nm, kb[kb >= 0], nm[kb >= 0])
    V = (p.XMAX - p.XMIN) * (p.YMAX - p.YMIN) * (p.ZMAX - p.ZMIN)
    norm = N * N / V
    Nmt = torch.as_tensor(np.where(Nm > 0, Nm, 1.0), device=x.device)
    keep = Nm > 0
    keep[np.nonzero(Nm > 0)[0].max()] = False  # output_power zeroes the highest filled bin
    kt = torch.as_tensor(keep.astype(np.float64), device=x.device)
    P0 = (S0 - Nmt * N) / (Nmt * norm) * kt
    P2 = 5.0 * S2 / (Nmt * norm) * kt
    return P0, P2


# Fields and spectrum of a reference Momentum run (src/read_data.c:91-130, src/main.c:141-148): the number
# of fields, the exponents e of v in the deposits w v^e of field A and B, whether the spectrum is the
# imaginary part of A*B, whether A is mean-subtracted, and the moment m of the shot noise N sum w v^m / sum w
MOMENTUM_FIELDS = {0: (1, 0, 0, 0, 1, 0), 1: (2, 0, 1, 1, 1, 1), 2: (1, 1, 0, 0, 0, 2), 3: (2, 0, 2, 0, 1, 2),
                   4: (2, 1, 2, 1, 0, 3), 5: (1, 2, 0, 0, 0, 4), 6: (2, 0, 3, 1, 1, 3), 7: (2, 1, 3, 0, 0, 4),
                   8: (2, 0, 4, 0, 1, 4)}


def dense_spectra(torch, p, x, y, z, v, w, tab, exps, mean_sub_a, specs):
    """P0, P2 of every spectrum (TSC, interlaced, LOS = z) for particles whose every tap lies inside the
    grid, normalised as output_power does. exps: the exponents of v of the painted fields (deposits
    w v^e); field A is mean-subtracted when mean_sub_a. specs: (product, shot moment) per spectrum, the
    product 0 |A|^2, 1 Re A*B, 2 Im A*B, 3 |B|^2."""
    n = p.NX
    d = (p.XMAX - p.XMIN) / n
    zs = z + v * rsd_factor(p)

    def paint(px, py, pz, val):
        g = torch.zeros(n * n * n, dtype=torch.float64, device=x.device)
        s = [(px - p.XMIN) / d, (py - p.YMIN) / d, (pz - p.ZMIN) / d]
        i = [torch.floor(t + 0.5).detach().long() for t in s]
        dd = [t - ii.to(t.dtype) for t, ii in zip(s, i)]
        W = [[0.5 * (0.5 - e) ** 2, 0.75 - e * e, 0.5 * (0.5 + e) ** 2] for e in dd]
        for a in range(3):
            for b in range(3):
                for c in range(3):
                    idx = ((i[0] + a - 1) * n + (i[1] + b - 1)) * n + (i[2] + c - 1)
                    g = g.index_add(0, idx, val * W[0][a] * W[1][b] * W[2][c])
        return g.view(n, n, n)

    N = w.sum()
    h = 0.5 * d
    kb, mu, wgt, e, nm = tab
    dc = torch.zeros(kb.shape, dtype=torch.float64, device=x.device)
    dc[0, 0, 0] = 1.0
    et = torch.as_tensor(e, device=x.device)
    fields = []
    for f, ex in enumerate(exps):
        val = w * v ** ex
        g, gi = paint(x, y, zs, val), paint(x + h, y + h, zs + h, val)
        sub = N if (f == 0 and mean_sub_a) else 0.0
        F = torch.fft.rfftn(g) * (1 - dc) + dc * (g.sum() - sub)
        Fi = torch.fft.rfftn(gi) * (1 - dc) + dc * (gi.sum() - sub)
        fields.append(F + et * Fi)
    m = torch.as_tensor(kb >= 0, device=x.device)
    kbt = torch.as_tensor(np.where(kb >= 0, kb, 0), device=x.device)[m]
    mut = torch.as_tensor(mu, device=x.device)[m]
    Nm = np.zeros(p.NK)
    np.add.at(Nm, kb[kb >= 0], nm[kb >= 0])
    V = (p.XMAX - p.XMIN) * (p.YMAX - p.YMIN) * (p.ZMAX - p.ZMIN)
    norm = N * N / V
    Nmt = torch.as_tensor(np.where(Nm > 0, Nm, 1.0), device=x.device)
    keep = Nm > 0
    keep[np.nonzero(Nm > 0)[0].max()] = False  # output_power zeroes the highest filled bin
    kt = torch.as_tensor(keep.astype(np.float64), device=x.device)
    A = fields[0]
    B = fields[1] if len(fields) > 1 else None
    out = []
    for prod, sm in specs:
        pw = [lambda: A.real ** 2 + A.imag ** 2, lambda: A.real * B.real + A.imag * B.imag,
              lambda: A.real * B.imag - A.imag * B.real, lambda: B.real ** 2 + B.imag ** 2][prod]()
        power = torch.as_tensor(wgt, device=x.device) * pw
        S0 = torch.zeros(p.NK, dtype=torch.float64, device=x.device).index_add(0, kbt, power[m])
        S2 = torch.zeros(p.NK, dtype=torch.float64, device=x.device).index_add(0, kbt,
                                                                               power[m] * (1.5 * mut ** 2 - 0.5))
        shot = N * ((w * v ** sm).sum() / w.sum()) if sm else N
        out.append(((S0 / Nmt - shot) / norm * kt, 5.0 * S2 / (Nmt * norm) * kt))
    return out


def lib_spectra(p, parts, precision, spectra=None):
    """P0, P2 of every spectrum of one library evaluation."""
    x, y, z, vz, w = parts
    kw = {"spectra": spectra} if spectra else {}
    with cg.PowerSpectrum(p, precision=precision, **kw) as ps:
        ps.paint(x, y, z, vz, w)
        return [(r["Pk0"], r["Pk2"]) for r in (ps.normalise(q) for q in ps.power())]


def lib_spectra_grads(p, parts, precision, T, spectra=None):
    x, y, z, vz, w = parts
    kw = {"spectra": spectra} if spectra else {}
    with cg.PowerSpectrum(p, precision=precision, **kw) as ps:
        ps.paint(x, y, z, vz, w)
        P = [(r["Pk0"], r["Pk2"]) for r in (ps.normalise(q) for q in ps.power())]
        gr = ps.backward([{"Pk0": 2 * (a - ta), "Pk2": 2 * (b - tb)} for (a, b), (ta, tb) in zip(P, T)])
    return gr, P


def lib_multipoles(p, parts, precision):
    x, y, z, vz, w = parts
    with cg.PowerSpectrum(p, precision=precision) as ps:
        ps.paint(x, y, z, vz, w)
        r = ps.normalise(ps.power()[0])
    return r["Pk0"], r["Pk2"]


def lib_grads(p, parts, precision, T0, T2):
    x, y, z, vz, w = parts
    with cg.PowerSpectrum(p, precision=precision) as ps:
        ps.paint(x, y, z, vz, w)
        r = ps.normalise(ps.power()[0])
        P0, P2 = r["Pk0"], r["Pk2"]
        gr = ps.backward({"Pk0": 2 * (P0 - T0), "Pk2": 2 * (P2 - T2)})
    return gr, P0, P2


def interior_particles(p, n, seed, margin=3.0):
    rng = np.random.default_rng(seed)
    d = (p.XMAX - p.XMIN) / p.NX
    lo, hi = p.XMIN + margin * d, p.XMAX - margin * d
    x, y, z = (rng.uniform(lo, hi, n) for _ in range(3))
    vz = rng.normal(0.0, 50.0, n)
    w = rng.uniform(0.5, 1.5, n)
    return x, y, z, vz, w


BASE = dict(XMIN=0.0, XMAX=1000.0, YMIN=0.0, YMAX=1000.0, ZMIN=0.0, ZMAX=1000.0, InterpOrder=3,
            DoInterlacing=1, LOS=3, Momentum=0)


def test_backward_matches_dense_torch_autograd(gpu):
    torch = pytest.importorskip("torch")
    p = cg.Params(NX=64, NY=64, NZ=64, NK=30, Maxk=0.3, **BASE)
    parts = interior_particles(p, 32 ** 3, seed=41)
    T0, T2 = lib_multipoles(p, interior_particles(p, 32 ** 3, seed=42), "fp64")
    gr, P0, P2 = lib_grads(p, parts, "fp64", T0, T2)
    tab = mode_tables(p)
    t = [torch.tensor(a, dtype=torch.float64, device=gpu, requires_grad=True) for a in parts]
    D0, D2 = dense_multipoles(torch, p, *t, tab)
    scale0 = np.abs(P0).max()
    assert np.abs(D0.detach().cpu().numpy() - P0).max() <= 1e-10 * scale0
    assert np.abs(D2.detach().cpu().numpy() - P2).max() <= 1e-10 * scale0
    loss = ((D0 - torch.as_tensor(T0, device=gpu)) ** 2).sum() + ((D2 - torch.as_tensor(T2, device=gpu)) ** 2).sum()
    loss.backward()
    for name, tt in zip(("dx", "dy", "dz", "dvlos", "dw"), t):
        ref = tt.grad.cpu().numpy()
        err = np.abs(gr[name] - ref).max() / np.abs(ref).max()
        assert err <= 1e-8, f"{name}: {err:.2e}"


def test_autograd_function_matches_dense_torch_autograd(gpu):
    """The same loss written in torch over the multipoles of the test-only autograd.Function (whose
    backward is capow_backward), against autograd through the dense FP64 restatement."""
    torch = pytest.importorskip("torch")
    from capow_autograd import density_multipoles

    p = cg.Params(NX=64, NY=64, NZ=64, NK=30, Maxk=0.3, **BASE)
    parts = interior_particles(p, 32 ** 3, seed=43)
    T0, T2 = (torch.as_tensor(a, device=gpu) for a in lib_multipoles(p, interior_particles(p, 32 ** 3, seed=44),
                                                                          "fp64"))
    t = [torch.tensor(a, dtype=torch.float64, device=gpu, requires_grad=True) for a in parts]
    P = density_multipoles(torch, p, "fp64", *t)
    loss = ((P[0] - T0) ** 2).sum() + ((P[2] - T2) ** 2).sum()
    loss.backward()
    got = [tt.grad.cpu().numpy() for tt in t]
    u = [torch.tensor(a, dtype=torch.float64, device=gpu, requires_grad=True) for a in parts]
    D0, D2 = dense_multipoles(torch, p, *u, mode_tables(p))
    assert np.abs(P[0].detach().cpu().numpy() - D0.detach().cpu().numpy()).max() <= 1e-10 * D0.abs().max().item()
    ((D0 - T0) ** 2).sum().add(((D2 - T2) ** 2).sum()).backward()
    for name, g, uu in zip(("dx", "dy", "dz", "dvlos", "dw"), got, u):
        ref = uu.grad.cpu().numpy()
        err = np.abs(g - ref).max() / np.abs(ref).max()
        assert err <= 1e-8, f"{name}: {err:.2e}"


def test_backward_central_differences(gpu):
    p = cg.Params(NX=32, NY=32, NZ=32, NK=15, Maxk=0.15, **BASE)
    parts = [a.copy() for a in interior_particles(p, 20000, seed=51, margin=0.0)]
    T0, T2 = lib_multipoles(p, interior_particles(p, 20000, seed=52, margin=0.0), "fp64")
    gr, _, _ = lib_grads(p, parts, "fp64", T0, T2)

    def loss():
        P0, P2 = lib_multipoles(p, parts, "fp64")
        return float(((P0 - T0) ** 2).sum() + ((P2 - T2) ** 2).sum())

    d = (p.XMAX - p.XMIN) / p.NX
    rng = np.random.default_rng(53)
    picks = rng.choice(len(parts[0]), 64, replace=False)
    steps = {"dx": 1e-3 * d, "dy": 1e-3 * d, "dz": 1e-3 * d, "dvlos": 1e-3 * d / rsd_factor(p), "dw": 1e-3}
    for a, name in enumerate(("dx", "dy", "dz", "dvlos", "dw")):
        fd = []
        for i in picks:
            v0 = parts[a][i]
            parts[a][i] = v0 + steps[name]
            lp = loss()
            parts[a][i] = v0 - steps[name]
            lm = loss()
            parts[a][i] = v0
            fd.append((lp - lm) / (2 * steps[name]))
        fd = np.array(fd)
        an = gr[name][picks]
        scale = np.abs(fd).max()
        bad = np.abs(an - fd) > 2e-3 * scale
        # a central difference that straddles a TSC kink (a cell face) is off by O(h): allow two
        assert bad.sum() <= 2, f"{name}: {np.c_[an[bad], fd[bad]]}"


def test_backward_particles_outside_the_box(gpu):
    """Particles that the RSD shift puts just below z = 0 are outside the box. The reader counts
    them in NOUT and still calls add_to_grid for both stencils (src/read_data.c:76-97): the normal
    stencil is rejected (z < ZMIN), the interlaced copy at z + dz/2 is painted when it lands at or
    above ZMIN. So the first group's gradient is its interlaced copy's and the second group's is 0."""
    p = cg.Params(NX=32, NY=32, NZ=32, NK=15, Maxk=0.15, **BASE)
    parts = [a.copy() for a in interior_particles(p, 20000, seed=71, margin=0.0)]
    d = (p.XMAX - p.XMIN) / p.NX
    rng = np.random.default_rng(72)
    live, dead = np.arange(0, 8), np.arange(8, 16)
    u = rng.uniform(0.05, 0.4, 16)
    target = np.r_[rng.uniform(-0.45, -0.05, 8), rng.uniform(-0.95, -0.6, 8)]  # shifted z / dz
    parts[2][:16] = p.ZMIN + u * d
    parts[3][:16] = (target - u) * d / rsd_factor(p)
    T0, T2 = lib_multipoles(p, interior_particles(p, 20000, seed=73, margin=0.0), "fp64")

    def loss():
        P0, P2 = lib_multipoles(p, parts, "fp64")
        return float(((P0 - T0) ** 2).sum() + ((P2 - T2) ** 2).sum())

    h = 1e-2 * d
    fd = {}
    for a, name in ((0, "dx"), (1, "dy"), (2, "dz")):
        vals = []
        for i in live:
            v0 = parts[a][i]
            parts[a][i] = v0 + h
            lp = loss()
            parts[a][i] = v0 - h
            lm = loss()
            parts[a][i] = v0
            vals.append((lp - lm) / (2 * h))
        fd[name] = np.array(vals)
    for prec in ("fp64", "fp32"):
        gr, _, _ = lib_grads(p, parts, prec, T0, T2)
        for name in ("dx", "dy", "dz", "dvlos", "dw"):
            assert np.all(gr[name][dead] == 0.0), (prec, name, gr[name][dead])
        for name, f in fd.items():
            assert np.abs(f).max() > 0.0
            an = gr[name][live]
            assert np.all(np.abs(an - f) <= 1e-2 * np.abs(f).max()), (prec, name, np.c_[an, f])


def test_backward_fp32_matches_fp64_at_c3_size(gpu):
    """The C3 workload: 256^3 Zel'dovich particles (f32, unit weights), TSC 256^3, interlaced, LOS = z."""
    import torch

    from capow_gb300 import synth

    p = cg.Params(NX=256, NY=256, NZ=256, NK=80, Maxk=0.8, **BASE)
    x, y, z, vx, vy, vz = synth.zeldovich(256, L=1000.0, mesh=512, rms_cells=1.5, seed=2, torch_device=gpu)
    d = [torch.from_numpy(a).to(gpu) for a in (x, y, z, vz)]
    t = synth.zeldovich(256, L=1000.0, mesh=512, rms_cells=1.5, seed=3, torch_device=gpu)
    with cg.PowerSpectrum(p, precision="fp64") as ps:
        ps.paint(*[torch.from_numpy(a).to(gpu) for a in (t[0], t[1], t[2], t[5])])
        rt = ps.normalise(ps.power()[0])
    out = {}
    for prec in ("fp32", "fp64"):
        with cg.PowerSpectrum(p, precision=prec) as ps:
            ps.paint(*d)
            r = ps.normalise(ps.power()[0])
            g = {k: torch.empty_like(d[0]) for k in ("dx", "dy", "dz", "dvlos", "dw")}
            ps.backward({"Pk0": 2 * (r["Pk0"] - rt["Pk0"]), "Pk2": 2 * (r["Pk2"] - rt["Pk2"])}, out=g)
            out[prec] = {k: v.double().cpu().numpy() for k, v in g.items()}
    for k in out["fp64"]:
        a, b = out["fp32"][k], out["fp64"][k]
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert rel <= 2e-3, f"{k}: relative L2 difference {rel:.2e}"


@pytest.mark.parametrize("fft_path", ["auto", "one_launch", "3d"])
def test_backward_after_power_equals_backward_after_repaint(gpu, fft_path):
    """The transposed power stages (auto, one_launch on a power-of-two grid) read the painted grids out of
    place, so capow_backward starts from them; the 3-D path transforms them in place and capow_backward
    repaints. A second capow_backward (its first left dL/dgrid in the slots) always repaints: both calls
    give the same gradients on every path."""
    import torch

    from capow_gb300 import synth

    p = cg.Params(NX=64, NY=64, NZ=64, NK=30, Maxk=0.3, **BASE)
    x, y, z, vx, vy, vz = synth.zeldovich(48, L=1000.0, mesh=64, rms_cells=1.5, seed=5, torch_device=gpu)
    d = [torch.from_numpy(a).to(gpu) for a in (x, y, z, vz)]
    with cg.PowerSpectrum(p, precision="fp32", spectra=["dd", "dp", "pp"], fft_path=fft_path) as ps:
        ps.paint(*d)
        r = [ps.normalise(s) for s in ps.power()]
        dl = [{"Pk0": 2 * s["Pk0"], "Pk2": 2 * s["Pk2"]} for s in r]
        outs = []
        for _ in range(2):
            g = {k: torch.empty_like(d[0]) for k in ("dx", "dy", "dz", "dvlos", "dw")}
            ps.backward(dl, out=g)
            outs.append({k: v.double().cpu().numpy() for k, v in g.items()})
    for k in outs[0]:
        a, b = outs[0][k], outs[1][k]
        assert np.linalg.norm(b) > 0.0, k
        assert np.linalg.norm(a - b) <= 1e-6 * np.linalg.norm(b), (fft_path, k)


DDPP = (["dd", "dp", "pp"], (0, 1), True, [(0, 0), (2, 1), (3, 2)])


def _two_field_case(p, spectra, seed):
    """Spectra selection, the fields' exponents, mean subtraction and (product, shot moment) per spectrum."""
    if spectra:
        return DDPP
    nf, ea, eb, imag, msub, sm = MOMENTUM_FIELDS[p.Momentum]
    prod = 0 if nf == 1 else (2 if imag else 1)
    return None, ((ea,) if nf == 1 else (ea, eb)), bool(msub), [(prod, sm)]


@pytest.mark.parametrize("momentum,spectra", [(0, True), (1, False), (2, False), (4, False), (7, False)])
def test_backward_two_fields_match_dense_torch_autograd(gpu, momentum, spectra):
    """The density and LOS-momentum fields: the dd + dp + pp selection (|A|^2, Im A*B, |B|^2 with the shot
    moments 0, 1, 2) and reference Momentum runs 1 (Im A*B), 2 (|w v|^2, no mean subtraction), 4
    (Im (w v)* (w v^2), moment 3) and 7 (Re (w v)* (w v^3), moment 4): every gradient against autograd
    through the dense FP64 restatement."""
    torch = pytest.importorskip("torch")
    p = cg.Params(NX=48, NY=48, NZ=48, NK=20, Maxk=0.28, **dict(BASE, Momentum=momentum))
    sel, exps, msub, specs = _two_field_case(p, spectra, 0)
    sel = DDPP[0] if spectra else None
    parts = list(interior_particles(p, 12000, seed=81 + momentum))
    parts[3] = parts[3] / 50.0  # v of order 1: the moments up to v^4 stay comparable to the density
    ref = list(interior_particles(p, 12000, seed=91 + momentum))
    ref[3] = ref[3] / 50.0
    T = lib_spectra(p, ref, "fp64", sel)
    gr, P = lib_spectra_grads(p, parts, "fp64", T, sel)
    tab = mode_tables(p)
    t = [torch.tensor(a, dtype=torch.float64, device=gpu, requires_grad=True) for a in parts]
    D = dense_spectra(torch, p, *t, tab, exps, msub, specs)
    loss = 0.0
    for (d0, d2), (p0, p2), (t0, t2) in zip(D, P, T):
        scale = np.abs(p0).max() + np.abs(p2).max()
        assert np.abs(d0.detach().cpu().numpy() - p0).max() <= 1e-10 * scale
        assert np.abs(d2.detach().cpu().numpy() - p2).max() <= 1e-10 * scale
        loss = loss + ((d0 - torch.as_tensor(t0, device=gpu)) ** 2).sum() + ((d2 - torch.as_tensor(t2, device=gpu)) ** 2).sum()
    loss.backward()
    for name, tt in zip(("dx", "dy", "dz", "dvlos", "dw"), t):
        r = tt.grad.cpu().numpy()
        err = np.abs(gr[name] - r).max() / np.abs(r).max()
        assert err <= 1e-8, f"Momentum {momentum} spectra {spectra} {name}: {err:.2e}"


def test_backward_dd_dp_pp_central_differences(gpu):
    """The dd + dp + pp loss's gradient against central differences of the library's own forward."""
    p = cg.Params(NX=32, NY=32, NZ=32, NK=15, Maxk=0.15, **BASE)
    parts = [a.copy() for a in interior_particles(p, 20000, seed=61, margin=0.0)]
    parts[3] = parts[3] / 50.0
    ref = list(interior_particles(p, 20000, seed=62, margin=0.0))
    ref[3] = ref[3] / 50.0
    T = lib_spectra(p, ref, "fp64", DDPP[0])
    gr, _ = lib_spectra_grads(p, parts, "fp64", T, DDPP[0])

    def loss():
        P = lib_spectra(p, parts, "fp64", DDPP[0])
        return float(sum(((a - ta) ** 2).sum() + ((b - tb) ** 2).sum() for (a, b), (ta, tb) in zip(P, T)))

    d = (p.XMAX - p.XMIN) / p.NX
    rng = np.random.default_rng(63)
    picks = rng.choice(len(parts[0]), 48, replace=False)
    steps = {"dx": 1e-3 * d, "dy": 1e-3 * d, "dz": 1e-3 * d, "dvlos": 1e-3, "dw": 1e-3}
    for a, name in enumerate(("dx", "dy", "dz", "dvlos", "dw")):
        fd = []
        for i in picks:
            v0 = parts[a][i]
            parts[a][i] = v0 + steps[name]
            lp = loss()
            parts[a][i] = v0 - steps[name]
            lm = loss()
            parts[a][i] = v0
            fd.append((lp - lm) / (2 * steps[name]))
        fd = np.array(fd)
        an = gr[name][picks]
        scale = np.abs(fd).max()
        bad = np.abs(an - fd) > 2e-3 * scale
        # a central difference that straddles a TSC kink (a cell face) is off by O(h): allow two
        assert bad.sum() <= 2, f"{name}: {np.c_[an[bad], fd[bad]]}"


def test_backward_dd_dp_pp_fp32_matches_fp64(gpu):
    """The FP32 context's two-field adjoint (FP32 grids, FFTs and readout) against the FP64 one."""
    p = cg.Params(NX=64, NY=64, NZ=64, NK=30, Maxk=0.3, **BASE)
    parts = list(interior_particles(p, 200000, seed=65))
    parts[3] = parts[3] / 50.0
    ref = list(interior_particles(p, 200000, seed=66))
    ref[3] = ref[3] / 50.0
    T = lib_spectra(p, ref, "fp64", DDPP[0])
    g64, _ = lib_spectra_grads(p, parts, "fp64", T, DDPP[0])
    g32, _ = lib_spectra_grads(p, parts, "fp32", T, DDPP[0])
    for name in ("dx", "dy", "dz", "dvlos", "dw"):
        err = np.abs(g32[name] - g64[name]).max() / np.abs(g64[name]).max()
        assert err <= 2e-3, f"{name}: {err:.2e}"
