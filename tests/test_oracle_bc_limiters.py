"""CPU checks of the oracle's reflective walls and slope limiters.

Reflective walls (ReflectiveBoundary, ReflectIndex, Reflect) are pinned
against the periodic path: a reflective domain of n cells advances exactly
like the left half of a periodic domain of 2n cells holding the state and its
mirror image (the momentum normal to the wall negated), because the periodic
images of that doubled domain are the reflective ghosts.  The limiters are
pinned by identities: NoGradient (slope 0) makes MUSCL-Hancock + HLLE the
first-order HLLE flux, and NoLimiter's central slope agrees with van Leer's
on monotone linear data."""
import numpy as np
import pytest

from finitevolumesolver_gb300 import workloads


def _mirror(cons, rank, axis_dir):
    """Doubled state along direction axis_dir: [U, mirror(U)], the mirrored
    half with the momentum of that direction negated."""
    ax = cons.ndim - 1 - axis_dir  # array axis of the direction (x fastest)
    m = np.flip(cons, axis=ax).copy()
    m[1 + axis_dir] *= -1.0
    return np.concatenate([cons, m], axis=ax)


CASES = [
    (1, [48], 0),
    (2, [24, 20], 0),
    (2, [24, 20], 1),
    (3, [12, 10, 8], 2),
]


@pytest.mark.parametrize("limiter", [0, 1, 2, 3])
@pytest.mark.parametrize("rank,n,d", CASES)
def test_reflective_equals_mirrored_periodic(orc, rank, n, d, limiter):
    shape = tuple(reversed(n))
    cons = workloads.random_state(shape, rank, seed=3 + rank + d, v=0.6)
    cons = cons.reshape([rank + 2] + [1] * (3 - rank) + list(shape))
    big = _mirror(cons, rank, d)
    n2 = list(n)
    n2[d] *= 2
    bc = [0] * rank
    bc[d] = 2
    dx = [0.1, 0.07, 0.05][:rank]
    m = orc.method(limiter=limiter)
    g = orc.Grid(rank, n, bc, dx)
    g2 = orc.Grid(rank, n2, [0] * rank, dx)
    assert g.stable_dt(m, cons) == g2.stable_dt(m, big)
    dt = 0.4 * g.stable_dt(m, cons)
    ax = cons.ndim - 1 - d
    half = [slice(None)] * cons.ndim
    half[ax] = slice(0, n[d])
    for sd in range(rank):
        np.testing.assert_array_equal(g.sweep(m, cons, dt, sd),
                                      g2.sweep(m, big, dt, sd)[tuple(half)])
    np.testing.assert_array_equal(g.step(m, cons, dt, 1), g2.step(m, big, dt, 1)[tuple(half)])


def test_reflective_box_conserves_mass_and_energy(orc):
    """Walls on all sides: the HLLE flux between a cell and its reflected
    image carries no mass and no energy."""
    n = [40, 32]
    cons = workloads.random_state((32, 40), 2, seed=5, v=0.8).reshape(4, 1, 32, 40)
    g = orc.Grid(2, n, [2, 2], [1.0 / 40, 1.0 / 32])
    out, dts, _ = g.run(orc.method(), cons, 0.8, 10.0, max_steps=20)
    assert len(dts) == 20
    for c in (0, 3):
        assert abs(out[c].sum() - cons[c].sum()) <= 1e-13 * abs(cons[c]).sum()


def test_reflective_state_at_rest_stays_at_rest(orc):
    n = [16, 12, 10]
    cons = workloads.cons_from_prim(np.full((10, 12, 16), 1.3), [np.zeros((10, 12, 16))] * 3,
                                    np.full((10, 12, 16), 0.7)).reshape(5, 10, 12, 16)
    g = orc.Grid(3, n, [2, 2, 2], [0.1] * 3)
    out, _, _ = g.run(orc.method(), cons, 0.8, 10.0, max_steps=3)
    np.testing.assert_array_equal(out, cons)


def _stencil_fluxes(orc, kind, limiter, rank, cons, w, d, dt, dx):
    n = list(reversed(cons.shape[1:]))[:rank]
    states = orc.complete_from_cons(rank, cons.reshape(rank + 2, -1)).reshape(
        (rank + 4,) + cons.shape[1:])
    clo = [0] * rank
    chi = list(n)
    flo = [0] * rank
    fhi = list(n)
    flo[d] = w
    fhi[d] = n[d] - w + 1
    return orc.compute_numeric_fluxes(orc.method(kind, limiter), rank, states, (clo, chi),
                                      (flo, fhi), dt, dx, d)


@pytest.mark.parametrize("rank", [1, 2, 3])
def test_no_gradient_is_first_order_hlle(orc, rank):
    n = [14, 9, 7][:rank]
    cons = workloads.random_state(tuple(reversed(n)), rank, seed=11 + rank, v=0.7)
    cons = cons.reshape([rank + 2] + [1] * (3 - rank) + list(reversed(n)))
    for d in range(rank):
        # faces whose MUSCL stencil (2 cells each side) lies in the box
        muscl = _stencil_fluxes(orc, orc.MUSCL_HLLE, orc.NO_GRADIENT, rank, cons, 2, d, 0.01,
                                0.1)
        hlle = _stencil_fluxes(orc, orc.HLLE, orc.VAN_LEER, rank, cons, 1, d, 0.01, 0.1)
        ax = hlle.ndim - 1 - d
        inner = [slice(None)] * hlle.ndim
        inner[ax] = slice(1, hlle.shape[ax] - 1)
        np.testing.assert_array_equal(muscl, hlle[tuple(inner)])


def test_no_limiter_is_the_central_slope(orc):
    """On monotone linear data every limiter's slope is the central one, so
    NoLimiter and van Leer fluxes agree to round-off; at an extremum van Leer
    flattens the slope and NoLimiter does not."""
    n = 12
    x = np.arange(n, dtype=float)
    # every conservative component linear in x
    cons = np.stack([1.0 + 0.01 * x, 0.1 + 0.002 * x, 2.5 + 0.05 * x]).reshape(3, 1, 1, n)
    a = _stencil_fluxes(orc, orc.MUSCL_HLLE, orc.NO_LIMITER, 1, cons, 2, 0, 0.01, 0.1)
    b = _stencil_fluxes(orc, orc.MUSCL_HLLE, orc.VAN_LEER, 1, cons, 2, 0, 0.01, 0.1)
    np.testing.assert_allclose(a, b, rtol=1e-13, atol=1e-15)
    rho = 1.0 + 0.1 * np.cos(x)  # extrema
    cons = workloads.cons_from_prim(rho, [np.zeros(n)], np.ones(n)).reshape(3, 1, 1, n)
    a = _stencil_fluxes(orc, orc.MUSCL_HLLE, orc.NO_LIMITER, 1, cons, 2, 0, 0.01, 0.1)
    b = _stencil_fluxes(orc, orc.MUSCL_HLLE, orc.VAN_LEER, 1, cons, 2, 0, 0.01, 0.1)
    assert np.abs(a - b).max() > 1e-6
