"""CPU checks of the HLLEM restatement (Hllem<PerfectGas, Larrouturou>,
src/equations/perfect_gas/HllemMethod.hpp:711-1216): consistency with the
physical flux, exact preservation of a stationary contact (which HLLE
smears), mirror symmetry, and its stable dt."""
import numpy as np
import pytest

GAMMA = 1.4


def complete(rank, rho, vel, p):
    rho = np.asarray(rho, float)
    m = [rho * np.asarray(v, float) for v in vel]
    E = p / (GAMMA - 1) + 0.5 * rho * sum(np.asarray(v, float) ** 2 for v in vel)
    c = np.sqrt(GAMMA * p / rho)
    return np.stack([rho, *m, E, np.broadcast_to(p, rho.shape), c])


def face_flux(orc, kind, rank, left, right, dir=0):
    """Flux of the one face between two cells along x."""
    st = np.stack([left, right], axis=1).reshape(rank + 4, 1, 1, 2)
    f = orc.compute_numeric_fluxes(orc.method(kind), rank, st, ([0], [2]), ([1], [2]), 1e-3,
                                   0.1, dir)
    return f.reshape(rank + 2)


def physical_flux(rank, q):
    rho, m, E, p = q[0], q[1:1 + rank], q[1 + rank], q[2 + rank]
    u = m[0] / rho
    return np.array([m[0], *(u * m[k] + (p if k == 0 else 0.0) for k in range(rank)),
                     u * (E + p)])


@pytest.mark.parametrize("rank", [1, 2, 3])
def test_consistent_with_physical_flux(orc, rank):
    vel = [0.3, -0.7, 0.2][:rank]
    q = complete(rank, [1.3], [[v] for v in vel], 0.8)[:, 0]
    f = face_flux(orc, orc.HLLEM, rank, q, q)
    np.testing.assert_allclose(f, physical_flux(rank, q), rtol=1e-14, atol=1e-15)


@pytest.mark.parametrize("rank", [1, 2, 3])
def test_stationary_contact_is_exact(orc, rank):
    vel = [0.0, 0.4, -0.3][:rank]
    L = complete(rank, [1.0], [[v] for v in vel], 1.0)[:, 0]
    R = complete(rank, [0.125], [[v] for v in vel], 1.0)[:, 0]
    f = face_flux(orc, orc.HLLEM, rank, L, R)
    assert abs(f[0]) < 1e-14
    assert abs(f[1] - 1.0) < 1e-14          # pressure only
    fh = face_flux(orc, orc.HLLE, rank, L, R)
    assert abs(fh[0]) > 1e-2                # HLLE diffuses the contact


def test_mirror_symmetry(orc):
    rng = np.random.default_rng(0)
    for _ in range(20):
        rl, rr, pl, pr = rng.uniform(0.2, 2.0, 4)
        ul, ur, vl, vr = rng.uniform(-1, 1, 4)
        L = complete(2, [rl], [[ul], [vl]], pl)[:, 0]
        R = complete(2, [rr], [[ur], [vr]], pr)[:, 0]
        Lm = complete(2, [rr], [[-ur], [vr]], pr)[:, 0]
        Rm = complete(2, [rl], [[-ul], [vl]], pl)[:, 0]
        f = face_flux(orc, orc.HLLEM, 2, L, R)
        g = face_flux(orc, orc.HLLEM, 2, Lm, Rm)
        np.testing.assert_allclose([f[0], f[1], f[2], f[3]], [-g[0], g[1], -g[2], -g[3]],
                                   rtol=1e-12, atol=1e-13)


def test_stable_dt_uses_max_sound_speed(orc):
    L = complete(1, [1.0], [[0.5]], 1.0)
    R = complete(1, [0.5], [[0.5]], 2.0)
    st = np.concatenate([L, R], axis=1).reshape(5, 1, 1, 2)
    dt = orc.compute_stable_dt(orc.method(orc.HLLEM), 1, st, ([0], [2]), 0.1, 0, window_rule=1)
    aL, aR = L[4, 0], R[4, 0]
    # sR = max(roeU + roeA, uR + max(aL, aR)) >= 0.5 + max(aL, aR)
    assert dt <= 0.1 / (0.5 + max(aL, aR)) + 1e-15
