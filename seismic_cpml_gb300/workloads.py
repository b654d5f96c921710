"""Seeded synthetic workloads beyond the reference's own parameter blocks.

batch2d: many 2D shots of uneven size, each with its own layered model,
source frequency and position, receivers on a surface line, DELTAT from a
Courant number of 0.5 with the reference's formula (2D:513) and the shot's
largest P velocity, and NSTEP covering a fixed record length. y is up, so the
surface is the y-max edge.
"""
from __future__ import annotations

import math

import numpy as np

from .earth import layered_model
from .params import STF_RICKER, default_2d


def batch2d_shots(nshots=256, seed=4, interior=(200, 1200), npml=20, delta=5.0, layers=(4, 12),
                  cp_range=(1500.0, 4500.0), anomalies=3, amp=0.10, courant=0.5, record_s=2.0,
                  f0_range=(8.0, 25.0), nrec=128):
    """Return a list of (params, (lam, mu, rho), receivers) for each shot."""
    rng = np.random.default_rng(seed)
    shots = []
    for _ in range(nshots):
        nxi, nyi = (int(v) for v in rng.integers(interior[0], interior[1] + 1, size=2))
        nx, ny = nxi + 2 * npml, nyi + 2 * npml
        nl = int(rng.integers(layers[0], layers[1] + 1))
        (lam, mu, rho), cpmax = layered_model((ny, nx), nl, cp_range[0], cp_range[1],
                                              int(rng.integers(2 ** 31)), anomalies=anomalies,
                                              amp=amp, radius=(5, 40))
        p = default_2d()
        p.nx, p.ny = nx, ny
        p.deltax = p.deltay = delta
        p.npoints_pml = npml
        p.use_pml[:] = [1, 1, 1, 1, 0, 0]
        p.cp = cpmax                       # sets the C-PML d0 (2D:296) and the Courant check
        p.cs = cpmax / math.sqrt(3.0)
        p.rho = 310.0 * cpmax ** 0.25
        p.deltat = courant * delta / (cpmax * math.sqrt(2.0))
        p.nstep = int(math.ceil(record_s / p.deltat))
        p.f0 = float(rng.uniform(*f0_range))
        p.t0 = 1.2 / p.f0
        p.stf = STF_RICKER
        p.angle_force = 0.0                # vertical force
        p.factor = 1.0e7
        p.isource = int(rng.integers(npml + 1, nx - npml + 1))
        p.jsource = ny - npml - 3          # three cells below the top interior row
        p.it_display = 100
        jr = ny - npml - 1
        rec = [(npml + 1 + int(round(r * (nxi - 1) / (nrec - 1))), jr) for r in range(nrec)]
        shots.append((p, (lam, mu, rho), rec))
    return shots
