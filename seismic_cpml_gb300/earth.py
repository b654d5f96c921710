"""Seeded synthetic earth models (lambda, mu, rho per cell, float32).

The benchmark workloads use layered media with Gaussian velocity anomalies:
cs = cp / sqrt(3) and Gardner density rho = 310 * cp**0.25. Layers are
horizontal, i.e. stacked along y, the reference's vertical axis (y is up in
seismic_CPML_2D_isotropic_second_order.f90:37-56).
"""
from __future__ import annotations

import numpy as np


def lame_from_velocity(cp, cs, rho):
    cp = np.asarray(cp, np.float64)
    cs = np.asarray(cs, np.float64)
    rho = np.asarray(rho, np.float64)
    mu = rho * cs * cs
    lam = rho * (cp * cp - 2.0 * cs * cs)
    return lam.astype(np.float32), mu.astype(np.float32), rho.astype(np.float32)


def layered_cp(shape, nlayers, cp_lo, cp_hi, rng, anomalies=0, amp=0.1, radius=(3, 8)):
    """cp on a grid of ``shape`` ([nz,] ny, nx) with ``nlayers`` layers along y
    (interfaces at sorted uniform depths) and Gaussian anomalies of relative
    amplitude +/-amp and radius uniform in ``radius`` cells."""
    ny = shape[-2]
    tops = np.sort(rng.uniform(0, ny, nlayers - 1))
    vals = rng.uniform(cp_lo, cp_hi, nlayers)
    jj = np.arange(ny)
    layer = np.searchsorted(tops, jj)
    prof = vals[layer]
    cp = np.broadcast_to(prof.reshape([1] * (len(shape) - 2) + [ny, 1]), shape).astype(np.float64).copy()
    if anomalies:
        grids = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
        for _ in range(anomalies):
            c = [rng.uniform(0, n) for n in shape]
            r = rng.uniform(*radius)
            s = rng.choice([-1.0, 1.0]) * amp
            d2 = sum((g - cc) ** 2 for g, cc in zip(grids, c))
            cp *= 1.0 + s * np.exp(-d2 / (2.0 * r * r))
    return cp


def gardner(cp):
    return 310.0 * np.asarray(cp, np.float64) ** 0.25


def layered_model(shape, nlayers, cp_lo, cp_hi, seed, anomalies=0, amp=0.1, radius=(3, 8)):
    rng = np.random.default_rng(seed)
    cp = layered_cp(shape, nlayers, cp_lo, cp_hi, rng, anomalies, amp, radius)
    return lame_from_velocity(cp, cp / np.sqrt(3.0), gardner(cp)), float(cp.max())


def layered_model_3d_device(shape, nlayers=6, cp_lo=1800.0, cp_hi=5000.0, anomalies=8, amp=0.15,
                            radius=(20.0, 80.0), seed=3, device="cuda"):
    """(lambda, mu, rho) as FP32 torch tensors on `device`, shape (nz, ny, nx):
    `nlayers` horizontal layers stacked along y (the reference's vertical
    axis) at sorted uniform depths with cp uniform in [cp_lo, cp_hi], times
    1 +/- amp Gaussian anomalies with radius uniform in `radius` cells and
    centres uniform in the grid (each a separable product of three 1-D
    Gaussians), then cs = cp / sqrt(3) and Gardner density. Built on the
    device because the large workloads hold hundreds of millions of cells; the
    seeded parameters come from numpy (PCG64) so the model is the same on
    every machine."""
    import torch
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    tops = np.sort(rng.uniform(0, ny, nlayers - 1))
    vals = rng.uniform(cp_lo, cp_hi, nlayers)
    prof = torch.tensor(vals[np.searchsorted(tops, np.arange(ny))], dtype=torch.float32, device=device)
    cp = prof.view(1, ny, 1).expand(nz, ny, nx).contiguous()
    axes = [torch.arange(n, dtype=torch.float32, device=device) for n in (nz, ny, nx)]
    for _ in range(anomalies):
        c = [rng.uniform(0, n) for n in (nz, ny, nx)]
        r = rng.uniform(*radius)
        s = rng.choice([-1.0, 1.0]) * amp
        g = [torch.exp(-(a - cc) ** 2 / (2.0 * r * r)) for a, cc in zip(axes, c)]
        cp.mul_(1.0 + s * (g[0].view(nz, 1, 1) * g[1].view(1, ny, 1) * g[2].view(1, 1, nx)))
    cs = cp / float(np.sqrt(3.0))
    rho = 310.0 * cp ** 0.25
    mu = rho * cs * cs
    lam = rho * (cp * cp - 2.0 * cs * cs)
    return lam, mu, rho
