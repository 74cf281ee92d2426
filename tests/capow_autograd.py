"""A torch.autograd.Function over the C ABI's capow_power / capow_normalise (forward) and capow_backward
(backward), for tests only: it lets a test write a loss in torch over the normalised density multipoles
and get d(loss)/d(positions, velocities, weights) from the library's hand-written adjoint through
loss.backward(). The product has no torch dependency; this wrapper is not part of it."""
from __future__ import annotations

import numpy as np

import capow_gb300 as cg


def density_multipoles(torch, params, precision, x, y, z, vlos, w):
    """P_l(k), l = 0..4, of the density field as output_power writes them (shape [5, NK], float64, on
    x's device); differentiable in x, y, z, vlos and w (device tensors of one dtype)."""

    class _Multipoles(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x, y, z, vlos, w):
            ps = cg.PowerSpectrum(params, precision=precision)
            ps.paint(x, y, z, vlos, w)
            r = ps.normalise(ps.power()[0])
            ctx.ps = ps
            ctx.like = x
            return torch.tensor(np.stack([r[f"Pk{l}"] for l in range(5)]), dtype=torch.float64, device=x.device)

        @staticmethod
        def backward(ctx, g):
            ps = ctx.ps
            gh = g.detach().double().cpu().numpy()
            out = {k: torch.empty_like(ctx.like) for k in ("dx", "dy", "dz", "dvlos", "dw")}
            try:
                ps.backward({f"Pk{l}": gh[l] for l in range(5)}, out=out)
            finally:
                ps.close()
            return out["dx"], out["dy"], out["dz"], out["dvlos"], out["dw"]

    return _Multipoles.apply(x, y, z, vlos, w)
