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


def riemann_samples(n, seed=0, gamma=GAMMA, exclude_vacuum=True):
    """Random 1-D Riemann problems: rho_L, rho_R, p_L, p_R log-uniform on
    [1e-3, 1e1]; u_L, u_R uniform on [-3c, 3c] with c the larger sound
    speed.  Problems whose states generate vacuum (u_R - u_L >=
    2 (a_L + a_R) / (gamma - 1)) are redrawn.  Returns six float64 arrays."""
    rng = np.random.default_rng(seed)
    out = [np.empty(0) for _ in range(6)]
    need = n
    while need > 0:
        m = int(need * 1.3) + 16
        lo, hi = np.log(1e-3), np.log(1e1)
        rL, rR, pL, pR = (np.exp(rng.uniform(lo, hi, m)) for _ in range(4))
        aL = np.sqrt(gamma * pL / rL)
        aR = np.sqrt(gamma * pR / rR)
        c = np.maximum(aL, aR)
        uL = rng.uniform(-3, 3, m) * c
        uR = rng.uniform(-3, 3, m) * c
        ok = (uR - uL) < 2 * (aL + aR) / (gamma - 1) if exclude_vacuum else np.ones(m, bool)
        for k, arr in enumerate((rL, uL, pL, rR, uR, pR)):
            out[k] = np.concatenate([out[k], arr[ok]])
        need = n - len(out[0])
    return tuple(a[:n] for a in out)


def quadrants_2d(n=2048, seed=3, gamma=GAMMA, margin=0.8):
    """2-D four-quadrant Riemann problem on the unit square, n^2 cells; the
    four states are drawn from the distribution of riemann_samples, redrawn
    until no interface (in x or y, including the periodic wrap) comes within
    `margin` of generating vacuum."""
    rng = np.random.default_rng(seed)
    lo, hi = np.log(1e-3), np.log(1e1)
    while True:
        rho = np.exp(rng.uniform(lo, hi, 4))
        p = np.exp(rng.uniform(lo, hi, 4))
        a = np.sqrt(gamma * p / rho)
        c = a.max()
        u = rng.uniform(-3, 3, 4) * c
        v = rng.uniform(-3, 3, 4) * c
        # quadrants: 0 = (x<.5,y<.5), 1 = (x>=.5,y<.5), 2 = (x<.5,y>=.5), 3 = (x>=.5,y>=.5)
        ok = True
        for l, r in ((0, 1), (2, 3), (1, 0), (3, 2)):
            ok &= (u[r] - u[l]) < margin * 2 * (a[l] + a[r]) / (gamma - 1)
        for l, r in ((0, 2), (1, 3), (2, 0), (3, 1)):
            ok &= (v[r] - v[l]) < margin * 2 * (a[l] + a[r]) / (gamma - 1)
        if ok:
            break
    x = (np.arange(n) + 0.5) / n
    q = (x[None, :] >= 0.5).astype(np.int64) + 2 * (x[:, None] >= 0.5)
    return cons_from_prim(rho[q], [u[q], v[q]], p[q], gamma).reshape(4, 1, n, n)


def shock_circles_2d(n=1024, seed=5, mach=2.0, gamma=GAMMA, x_shock=0.1, ncirc=8):
    """2-D Mach `mach` planar shock moving in +x into still gas (rho 1, p 1)
    over a union of `ncirc` circles (radii U[0.05, 0.15], centres
    U[0.3, 0.9]^2) on the unit square, n^2 cells.  The post-shock state
    follows from the Rankine-Hugoniot conditions.  Returns (circles [ncirc][3],
    cons (4, 1, n, n)); cells covered by the circles are left to the caller
    (the solver zeroes them)."""
    rng = np.random.default_rng(seed)
    r = rng.uniform(0.05, 0.15, ncirc)
    c = rng.uniform(0.3, 0.9, (ncirc, 2))
    circles = np.column_stack([c, r])
    rho1, p1 = 1.0, 1.0
    a1 = np.sqrt(gamma * p1 / rho1)
    m2 = mach * mach
    rho2 = rho1 * (gamma + 1) * m2 / ((gamma - 1) * m2 + 2)
    p2 = p1 * (1 + 2 * gamma / (gamma + 1) * (m2 - 1))
    u2 = mach * a1 * (1 - rho1 / rho2)
    x = (np.arange(n) + 0.5) / n
    post = np.broadcast_to(x[None, :] < x_shock, (n, n))
    rho = np.where(post, rho2, rho1)
    u = np.where(post, u2, 0.0)
    p = np.where(post, p2, p1)
    cons = cons_from_prim(rho, [u, np.zeros((n, n))], p, gamma).reshape(4, 1, n, n)
    return circles, cons


class AmrHierarchy:
    """A static 2-D block-structured AMR hierarchy with refinement ratio 2:
    `levels[p]` and `boxes[p] = (lo_x, lo_y, hi_x, hi_y)` (half-open, in
    level levels[p]'s index space) for every patch p; level l has
    (n0[0] << l) x (n0[1] << l) cells of size dx0 / 2^l."""

    def __init__(self, nlevels, n0, bc, dx0, levels, boxes):
        self.nlevels = int(nlevels)
        self.n0 = [int(v) for v in n0]
        self.bc = [int(v) for v in bc]
        self.dx0 = float(dx0)
        self.levels = np.ascontiguousarray(levels, dtype=np.int32)
        self.boxes = np.ascontiguousarray(boxes, dtype=np.int32).reshape(-1, 4)

    @property
    def npatches(self):
        return len(self.levels)

    def cells(self):
        ext = (self.boxes[:, 2] - self.boxes[:, 0]).astype(np.int64) * \
            (self.boxes[:, 3] - self.boxes[:, 1])
        return np.bincount(self.levels, weights=ext, minlength=self.nlevels).astype(np.int64)

    def cell_centres(self, p):
        l = int(self.levels[p])
        dx = self.dx0 / (1 << l)
        x0, y0, x1, y1 = (int(v) for v in self.boxes[p])
        x = (np.arange(x0, x1) + 0.5) * dx
        y = (np.arange(y0, y1) + 0.5) * dx
        return np.meshgrid(x, y)  # [ny][nx]

    def cons_from(self, fn):
        """Concatenated patch interiors [4][ny][nx] of cons = fn(X, Y)."""
        return np.concatenate([np.asarray(fn(*self.cell_centres(p))).reshape(-1)
                               for p in range(self.npatches)])

    def split(self, flat):
        """Per-patch views [4][ny][nx] of a concatenated array."""
        out, off = [], 0
        for p in range(self.npatches):
            x0, y0, x1, y1 = (int(v) for v in self.boxes[p])
            n = 4 * (x1 - x0) * (y1 - y0)
            out.append(flat[off:off + n].reshape(4, y1 - y0, x1 - x0))
            off += n
        return out


def _tile_axis(n, rng, sizes=(8, 16, 32, 64)):
    """Extents drawn from `sizes` that add up to n (a multiple of 8)."""
    out, left = [], n
    while left > 0:
        s = int(rng.choice(sizes))
        while s > left:
            s //= 2
        out.append(s)
        left -= s
    return out


def _tiling(n, rng, sizes=(8, 16, 32, 64)):
    w = _tile_axis(n, rng, sizes)
    h = _tile_axis(n, rng, sizes)
    xs = np.concatenate([[0], np.cumsum(w)])
    ys = np.concatenate([[0], np.cumsum(h)])
    return [(int(xs[i]), int(ys[j]), int(xs[i + 1]), int(ys[j + 1]))
            for j in range(len(h)) for i in range(len(w))]


def amr_hierarchy(n0=1024, nlevels=3, seed=7, centre=None, radius=0.1, bands=None,
                  bc=(1, 1), target=4096, sizes=(8, 16, 32, 64)):
    """Patches placed by refinement of the ring |r - radius| < band around a
    blast centre: level 0 tiles the n0^2 domain, level l >= 1 keeps the tiles
    of a random tiling of its index space (extents from {8, 16, 32, 64} per
    axis) that meet the ring of width bands[l-1] and whose footprint grown by
    the 2 ghost cells lies inside level l-1 (proper nesting).  Without
    `bands` the widths are scaled until the patch count is close to `target`.
    Returns (hierarchy, centre)."""
    rng = np.random.default_rng(seed)
    if centre is None:
        centre = rng.uniform(0.3, 0.7, 2)
    dx0 = 1.0 / n0
    base_state = rng.bit_generator.state

    def build(bands):
        rng.bit_generator.state = base_state
        levels, boxes = [], []
        tiles0 = _tiling(n0, rng, sizes)
        levels += [0] * len(tiles0)
        boxes += tiles0
        covered_prev = np.ones((n0, n0), dtype=bool)
        for l in range(1, nlevels):
            n = n0 << l
            dx = dx0 / (1 << l)
            band = bands[l - 1]
            cov = np.zeros((n, n), dtype=bool)
            for (x0, y0, x1, y1) in _tiling(n, rng, sizes):
                # does the tile meet the ring?
                xs = (np.array([x0, x1]) * dx) - centre[0]
                ys = (np.array([y0, y1]) * dx) - centre[1]
                nx_ = np.clip(0.0, xs[0], xs[1])
                ny_ = np.clip(0.0, ys[0], ys[1])
                dmin = np.hypot(nx_, ny_)
                dmax = np.hypot(np.abs(xs).max(), np.abs(ys).max())
                if dmax < radius - band or dmin > radius + band:
                    continue
                # nesting: the grown footprint must lie in level l-1
                gx0, gy0 = max(x0 - 2, 0), max(y0 - 2, 0)
                gx1, gy1 = min(x1 + 2, n), min(y1 + 2, n)
                if not covered_prev[gy0 // 2:(gy1 + 1) // 2, gx0 // 2:(gx1 + 1) // 2].all():
                    continue
                levels.append(l)
                boxes.append((x0, y0, x1, y1))
                cov[y0:y1, x0:x1] = True
            covered_prev = cov
        return levels, boxes

    if bands is None:
        lo, hi = 0.002, 0.2
        best = None
        for _ in range(16):
            mid = 0.5 * (lo + hi)
            bs = [mid / (1.5 ** (l - 1)) for l in range(1, nlevels)]
            lv, bx = build(bs)
            if best is None or abs(len(lv) - target) < abs(len(best[0]) - target):
                best = (lv, bx)
            if len(lv) < target:
                lo = mid
            else:
                hi = mid
        levels, boxes = best
    else:
        levels, boxes = build(bands)
    return AmrHierarchy(nlevels, (n0, n0), bc, dx0, levels, boxes), centre


def amr_blast_2d(n0=1024, nlevels=3, seed=7, target=4096, bc=(1, 1), gamma=GAMMA,
                 sizes=(8, 16, 32, 64)):
    """Blast wave on an AMR patch set: rho 1, p 1, p 10 inside radius 0.1
    about a seeded centre, at rest.  Returns (hierarchy, cons)."""
    h, centre = amr_hierarchy(n0, nlevels, seed, target=target, bc=bc, sizes=sizes)

    def fn(X, Y):
        r = np.hypot(X - centre[0], Y - centre[1])
        rho = np.ones_like(X)
        p = np.where(r < 0.1, 10.0, 1.0)
        return cons_from_prim(rho, [np.zeros_like(X), np.zeros_like(X)], p, gamma)

    return h, h.cons_from(fn)
