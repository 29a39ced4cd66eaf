"""CPU checks of the characteristic and primitive MUSCL-Hancock restatements
(perfect_gas::MusclHancockCharacteristic,
src/equations/perfect_gas/MusclHancockCharacteristicMethod.hpp, and
perfect_gas::MusclHancockPrim, src/equations/perfect_gas/MusclHancockPrimMethod.hpp,
both with the Hllem<PerfectGas, Larrouturou> face flux).

The reference's own tests hold no vectors for these methods, so the oracle is
checked by (1) a second, independent pure-Python transcription of both
reconstructions, fed through the oracle's HLLEM flux and compared bit for bit;
(2) consistency: a uniform stencil gives the physical flux; (3) mirror
symmetry; (4) second-order convergence of a smooth advected density wave."""
import math

import numpy as np
import pytest

GAMMA = 1.4


def complete(rank, rho, vel, p):
    m = [rho * v for v in vel]
    E = p / (GAMMA - 1) + 0.5 * rho * sum(v * v for v in vel)
    return np.array([rho, *m, E, p, math.sqrt(GAMMA * p / rho)])


def random_complete(rng, rank):
    return complete(rank, rng.uniform(0.3, 2.0), list(rng.uniform(-0.8, 0.8, rank)),
                    rng.uniform(0.3, 2.0))


def sqnorm(rank, m):
    if rank == 1:
        return m[0] * m[0]
    if rank == 2:
        return m[0] * m[0] + m[1] * m[1]
    return m[0] * m[0] + (m[1] * m[1] + m[2] * m[2])


def from_prim(rank, rho, vel, p):
    """PerfectGas::CompleteFromPrim (src/equations/PerfectGas.cpp:160-174)."""
    m = [rho * v for v in vel]
    e_kin = 0.5 * sqnorm(rank, m) / rho
    return np.array([rho, *m, e_kin + p * (1.0 / (GAMMA - 1.0)),
                     p, math.sqrt(GAMMA * p / rho)])


def van_leer(sl, sr):
    r = 2.0 * sl * sr
    return r / (sl + sr) if r > 0.0 else 0.0


def char_rec(rank, s, lam, ix, sign):
    """Characteristic reconstruction of s[1] at its right (sign +1) or left
    (sign -1) face (MusclHancockCharacteristicMethod.hpp:51-256)."""
    iy, iz = (ix + 1) % 3, (ix + 2) % 3
    rho, E, p, c = s[1][0], s[1][1 + rank], s[1][2 + rank], s[1][3 + rank]
    vel = [[q[1 + d] / q[0] if d < rank else 0.0 for d in range(3)] for q in s]
    u = s[1][1 + ix] / rho
    rhoc, ooc2 = rho * c, 1.0 / (c * c)

    def amps(lq, rq, lv, rv):
        dp, du, drho = rq[2 + rank] - lq[2 + rank], rv[ix] - lv[ix], rq[0] - lq[0]
        return [dp - rhoc * du, drho - ooc2 * dp, dp + rhoc * du, rv[iy] - lv[iy],
                rv[iz] - lv[iz]]

    aL = amps(s[0], s[1], vel[0], vel[1])
    aR = amps(s[1], s[2], vel[1], vel[2])
    sl = [van_leer(a, b) for a, b in zip(aL, aR)]
    speeds = [u - c, u, u + c, u, u]
    am = [sign * 0.5 * sl[k] * (1.0 - sign * lam * speeds[k]) for k in range(5)]
    dp = 0.5 * (am[0] + am[2])
    drho = ooc2 * dp + am[1]
    dv = [0.0] * 3
    dv[ix] = 0.5 * (am[2] - am[0]) / rhoc
    dv[iy], dv[iz] = am[3], am[4]
    return from_prim(rank, drho + rho, [dv[d] + s[1][1 + d] / s[1][0] for d in range(rank)],
                     dp + p)


def prim_limiter(ql, qm, qr):
    dq = 0.5 * (qr - ql)
    rel = abs(dq) > 1e-12
    den = dq if rel else 1.0
    rl = (qm - ql) / den if rel else 0.0
    rr = (qr - qm) / den if rel else 0.0
    r = (rl if rl < rr else rr) if (rl > 0.0 and rr > 0.0) else 0.0
    sigma = 2.0 * r / (1.0 + r) if r < 1.0 else 0.5 * (r + 1.0)
    return sigma * dq


def prim_rec(rank, s, lam, d, side):
    """Primitive reconstruction of s[1] at its right (+1) or left (-1) face
    (MusclHancockPrimMethod.hpp:63-175)."""
    u = [[q[1 + i] / q[0] for i in range(rank)] for q in s]
    rho, p, a = s[1][0], s[1][2 + rank], s[1][3 + rank]
    drho = prim_limiter(s[0][0], rho, s[2][0])
    dp = prim_limiter(s[0][2 + rank], p, s[2][2 + rank])
    du = [prim_limiter(u[0][i], u[1][i], u[2][i]) for i in range(rank)]
    ud = u[1][d]
    if side > 0:
        rr = rho + 0.5 * (drho - lam * (ud * drho + rho * du[d]))
        pp = p + 0.5 * (dp - lam * (rho * a * a * du[d] + ud * dp))
        uu = [u[1][i] + 0.5 * (du[i] - lam * (ud * du[i])) for i in range(rank)]
    else:
        rr = rho - 0.5 * (drho + lam * (ud * drho + rho * du[d]))
        pp = p - 0.5 * (dp + lam * (rho * a * a * du[d] + ud * dp))
        uu = [u[1][i] - 0.5 * (du[i] + lam * (ud * du[i])) for i in range(rank)]
    uu[d] -= 0.5 * lam * dp / rho
    m = [rr * v for v in uu]
    return np.array([rr, *m, 0.5 * rr * sqnorm(rank, uu) + pp * (1.0 / (GAMMA - 1.0)), pp,
                     math.sqrt(GAMMA * pp / rr)])


def stencil_flux(orc, kind, rank, cells, dt, dx, d):
    """Flux of the one face in the middle of a four-cell stencil along d."""
    n = [1, 1, 1]
    n[d] = len(cells)
    st = np.zeros((rank + 4, n[2], n[1], n[0]))
    for i, q in enumerate(cells):
        idx = [0, 0, 0]
        idx[d] = i
        st[:, idx[2], idx[1], idx[0]] = q
    flo, fhi = [0, 0, 0], [1, 1, 1]
    flo[d], fhi[d] = len(cells) // 2, len(cells) // 2 + 1
    f = orc.compute_numeric_fluxes(orc.method(kind), rank, st, ([0, 0, 0], n), (flo, fhi),
                                   dt, dx, d)
    return f.reshape(rank + 2)


@pytest.mark.parametrize("kind", ["char", "prim"])
@pytest.mark.parametrize("rank", [1, 2, 3])
def test_independent_transcription_bit_exact(orc, kind, rank):
    rng = np.random.default_rng(7 + rank)
    okind = orc.MUSCL_CHAR if kind == "char" else orc.MUSCL_PRIM
    for trial in range(24):
        d = trial % rank
        cells = [random_complete(rng, rank) for _ in range(4)]
        if trial % 3 == 0:  # smooth data: unclipped slopes
            base = random_complete(rng, rank)
            cells = [complete(rank, base[0] * (1 + 0.05 * i),
                              [base[1 + k] / base[0] + 0.02 * i for k in range(rank)],
                              base[2 + rank] * (1 + 0.03 * i)) for i in range(4)]
        dt, dx = 2e-3 * (1 + trial % 5), 0.01
        lam = dt / dx
        if kind == "char":
            L = char_rec(rank, cells[0:3], lam, d, 1.0)
            R = char_rec(rank, cells[1:4], lam, d, -1.0)
        else:
            L = prim_rec(rank, cells[0:3], lam, d, 1)
            R = prim_rec(rank, cells[1:4], lam, d, -1)
        want = stencil_flux(orc, orc.HLLEM, rank, [L, R], dt, dx, d)
        got = stencil_flux(orc, okind, rank, cells, dt, dx, d)
        np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("kind", ["char", "prim"])
@pytest.mark.parametrize("rank", [1, 2, 3])
def test_uniform_stencil_gives_physical_flux(orc, kind, rank):
    okind = orc.MUSCL_CHAR if kind == "char" else orc.MUSCL_PRIM
    q = complete(rank, 1.3, [0.3, -0.7, 0.2][:rank], 0.8)
    for d in range(rank):
        f = stencil_flux(orc, okind, rank, [q] * 4, 1e-3, 0.1, d)
        rho, m, E, p = q[0], q[1:1 + rank], q[1 + rank], q[2 + rank]
        u = m[d] / rho
        phys = [m[d], *(u * m[k] + (p if k == d else 0.0) for k in range(rank)), u * (E + p)]
        np.testing.assert_allclose(f, phys, rtol=1e-14, atol=1e-15)


@pytest.mark.parametrize("kind", ["char", "prim"])
def test_mirror_symmetry(orc, kind):
    okind = orc.MUSCL_CHAR if kind == "char" else orc.MUSCL_PRIM
    rng = np.random.default_rng(3)

    def mirror(q):
        r = q.copy()
        r[1] = -r[1]
        return r

    for _ in range(20):
        cells = [random_complete(rng, 2) for _ in range(4)]
        f = stencil_flux(orc, okind, 2, cells, 3e-3, 0.01, 0)
        g = stencil_flux(orc, okind, 2, [mirror(q) for q in reversed(cells)], 3e-3, 0.01, 0)
        np.testing.assert_allclose([f[0], f[1], f[2], f[3]], [-g[0], g[1], -g[2], -g[3]],
                                   rtol=1e-11, atol=1e-12)


@pytest.mark.parametrize("kind", ["char", "prim"])
def test_second_order_on_smooth_advection(orc, kind):
    """Density wave rho = 1 + 0.2 sin(2 pi x) advected at u = 1, p = 1 through
    one period: the L1 error falls by about 4 per halving of dx."""
    okind = orc.MUSCL_CHAR if kind == "char" else orc.MUSCL_PRIM
    errs = []
    for n in (64, 128):
        x = (np.arange(n) + 0.5) / n
        rho = 1.0 + 0.2 * np.sin(2 * np.pi * x)
        cons = np.stack([rho, rho * 1.0, 1.0 / (GAMMA - 1) + 0.5 * rho]).reshape(3, 1, 1, n)
        g = orc.Grid(1, [n], [0], [1.0 / n])
        out, dts, _ = g.run(orc.method(okind), cons, 0.5, 1.0, max_steps=100000)
        assert abs(dts.sum() - 1.0) < 1e-12
        # cell averages of the exact solution after one period
        exact = 1.0 + 0.2 * (np.cos(2 * np.pi * (x - 0.5 / n)) -
                             np.cos(2 * np.pi * (x + 0.5 / n))) / (2 * np.pi / n)
        errs.append(np.abs(out[0].ravel() - exact).mean())
    order = math.log2(errs[0] / errs[1])
    assert order > 1.7, (errs, order)
