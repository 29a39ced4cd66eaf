"""Seeded synthetic initial data of the benchmark workloads.

Conservative states are returned component-major, (rank+2, nz, ny, nx),
x fastest -- the layout of the solver context and of the reference's
FArrayBox data.
"""
from __future__ import annotations

import numpy as np

GAMMA = 1.4


def cons_from_prim(rho, vel, p, gamma=GAMMA):
    """rho, p: arrays; vel: list of velocity arrays (one per direction)."""
    rank = len(vel)
    out = np.empty((rank + 2,) + np.shape(rho))
    out[0] = rho
    ke = np.zeros_like(rho)
    for d, v in enumerate(vel):
        out[1 + d] = rho * v
        ke = ke + v * v
    out[1 + rank] = p / (gamma - 1.0) + 0.5 * rho * ke
    return out


def sod_1d(n=1024):
    """1-D Sod shock tube on [0, 1]: (rho, u, p) = (1, 0, 1) for x < 0.5 and
    (0.125, 0, 0.1) otherwise; dx = 1/n."""
    x = (np.arange(n) + 0.5) / n
    rho = np.where(x < 0.5, 1.0, 0.125)
    p = np.where(x < 0.5, 1.0, 0.1)
    return cons_from_prim(rho, [np.zeros(n)], p).reshape(3, 1, 1, n)


def octants_3d(n=256, seed=2024):
    """3-D periodic unit cube, n^3 cells: piecewise-constant octants with
    rho, p ~ U[0.1, 2] and each velocity component ~ U[-0.5, 0.5], plus 8
    Gaussian density bumps (amplitude U[0, 0.5], width U[0.02, 0.08], centre
    U[0, 1]^3)."""
    rng = np.random.default_rng(seed)
    rho_o = rng.uniform(0.1, 2.0, 8)
    p_o = rng.uniform(0.1, 2.0, 8)
    v_o = rng.uniform(-0.5, 0.5, (8, 3))
    amp = rng.uniform(0.0, 0.5, 8)
    width = rng.uniform(0.02, 0.08, 8)
    centre = rng.uniform(0.0, 1.0, (8, 3))
    x = (np.arange(n) + 0.5) / n
    hi = x >= 0.5
    # octant index o = ix + 2 iy + 4 iz, arrays indexed [z, y, x]
    o = (hi[None, None, :].astype(np.int64) + 2 * hi[None, :, None] + 4 * hi[:, None, None])
    rho = rho_o[o].astype(np.float64)
    p = p_o[o].astype(np.float64)
    vel = [v_o[o, 0], v_o[o, 1], v_o[o, 2]]
    for b in range(8):
        gx = np.exp(-((x - centre[b, 0]) ** 2) / (2 * width[b] ** 2))
        gy = np.exp(-((x - centre[b, 1]) ** 2) / (2 * width[b] ** 2))
        gz = np.exp(-((x - centre[b, 2]) ** 2) / (2 * width[b] ** 2))
        rho = rho + amp[b] * gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
    return cons_from_prim(rho, vel, p)


def random_state(shape, rank, seed=0, rho=(0.5, 1.5), p=(0.5, 1.5), v=0.4):
    """Smooth-free random states for parity tests (every cell independent)."""
    rng = np.random.default_rng(seed)
    r = rng.uniform(*rho, shape)
    pp = rng.uniform(*p, shape)
    vel = [rng.uniform(-v, v, shape) for _ in range(rank)]
    return cons_from_prim(r, vel, pp)
