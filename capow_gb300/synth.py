"""Seeded synthetic catalogues standing in for simulation outputs (no dataset is named or shipped).

* ``uniform``   -- positions uniform in the box, velocities i.i.d. Gaussian (the plain CPU-runnable
                   run: 2,097,152 particles, L = 1000, sigma_v = 300 km/s).
* ``zeldovich`` -- a cubic lattice displaced by the Zel'dovich approximation from a seeded Gaussian
                   random field with P(k) = A k^-1.5 exp(-(k/0.5)^2); A is fixed by the requested rms
                   3-D displacement (in mesh cells of the painting grid). Velocities are
                   0.8 * 100 * Psi plus Gaussian noise. Positions are wrapped into [0, L) and stored
                   as float32 strictly below L.
"""
from __future__ import annotations

import numpy as np


def uniform(n: int, L: float = 1000.0, sigma_v: float = 300.0, seed: int = 1, dtype=np.float64):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0.0, L, size=(3, n))
    vel = rng.normal(0.0, sigma_v, size=(3, n))
    return tuple(pos.astype(dtype)) + tuple(vel.astype(dtype))


def _wrap32(a: np.ndarray, L: float) -> np.ndarray:
    out = np.mod(a, L).astype(np.float32)
    out[out >= np.float32(L)] = 0.0
    out[out < 0] = 0.0
    return out


def zeldovich(n_side: int, L: float = 1000.0, mesh: int = 512, rms_cells: float = 1.5, seed: int = 2,
              growth_v: float = 0.8, sigma_v: float = 150.0, dtype=np.float32, torch_device=None):
    """Zel'dovich-displaced lattice of n_side^3 particles. Returns (x, y, z, vx, vy, vz).

    torch_device: optional torch device to run the FFTs on (same seed, same white noise; the
    displacement field then differs from the NumPy path only by FFT rounding)."""
    rng = np.random.default_rng(seed)
    white = rng.standard_normal((n_side, n_side, n_side)).astype(np.float64)
    kf = 2 * np.pi / L
    k1 = np.fft.fftfreq(n_side, d=1.0 / n_side) * kf
    kz1 = np.fft.rfftfreq(n_side, d=1.0 / n_side) * kf
    if torch_device is None:
        wk = np.fft.rfftn(white)
        kx, ky, kz = np.meshgrid(k1, k1, kz1, indexing="ij")
        k2 = kx * kx + ky * ky + kz * kz
        k = np.sqrt(k2)
        with np.errstate(divide="ignore", invalid="ignore"):
            amp = np.where(k > 0, np.sqrt(k ** -1.5 * np.exp(-(k / 0.5) ** 2)), 0.0)
            inv = np.where(k2 > 0, 1.0 / k2, 0.0)
        psi = []
        for ka in (kx, ky, kz):
            psi.append(np.fft.irfftn(1j * ka * inv * amp * wk, s=white.shape, axes=(0, 1, 2)))
        psi = np.stack(psi)
    else:
        import torch
        w = torch.from_numpy(white).to(torch_device)
        wk = torch.fft.rfftn(w)
        tk1 = torch.from_numpy(k1).to(torch_device)
        tkz = torch.from_numpy(kz1).to(torch_device)
        kx, ky, kz = torch.meshgrid(tk1, tk1, tkz, indexing="ij")
        k2 = kx * kx + ky * ky + kz * kz
        k = torch.sqrt(k2)
        amp = torch.where(k > 0, torch.sqrt(torch.clamp(k, min=1e-30) ** -1.5 * torch.exp(-(k / 0.5) ** 2)),
                          torch.zeros_like(k))
        inv = torch.where(k2 > 0, 1.0 / torch.clamp(k2, min=1e-30), torch.zeros_like(k2))
        psi = torch.stack([torch.fft.irfftn(1j * ka * inv * amp * wk, s=white.shape) for ka in (kx, ky, kz)])
        psi = psi.cpu().numpy()
        del w, wk
    rms = np.sqrt(np.mean(np.sum(psi * psi, axis=0)))
    target = rms_cells * L / mesh
    psi *= target / rms
    q = (np.arange(n_side) + 0.5) * (L / n_side)
    qx, qy, qz = np.meshgrid(q, q, q, indexing="ij")
    x = _wrap32(qx + psi[0], L).ravel()
    y = _wrap32(qy + psi[1], L).ravel()
    z = _wrap32(qz + psi[2], L).ravel()
    vel = growth_v * 100.0 * psi.reshape(3, -1) + rng.normal(0.0, sigma_v, size=(3, n_side ** 3))
    out = (x, y, z) + tuple(vel.astype(np.float32))
    if dtype != np.float32:
        out = tuple(a.astype(dtype) for a in out)
    return out
