"""CPU checks of the AMR oracle (oracle/fvs_oracle_amr.cpp): a one-level
patch set reproduces the uniform-grid oracle bit for bit, a uniform state
stays uniform across levels, and a three-level blast conserves mass,
momentum and energy to round-off (refluxing and average-down)."""
import numpy as np
import pytest

from finitevolumesolver_gb300 import workloads


def _single_level(n, seed, bc):
    rng = np.random.default_rng(seed)
    boxes = workloads._tiling(n, rng, sizes=(8, 16, 32))
    return workloads.AmrHierarchy(1, (n, n), bc, 1.0 / n, [0] * len(boxes), boxes)


def _to_grid(h, flat, n):
    g = np.zeros((4, n, n))
    for p, a in enumerate(h.split(flat)):
        x0, y0, x1, y1 = h.boxes[p]
        g[:, y0:y1, x0:x1] = a
    return g


def _from_grid(h, g):
    parts = []
    for p in range(h.npatches):
        x0, y0, x1, y1 = h.boxes[p]
        parts.append(g[:, y0:y1, x0:x1].reshape(-1))
    return np.concatenate(parts)


@pytest.mark.parametrize("bc", [(1, 1), (0, 0), (0, 1)])
def test_single_level_patch_set_matches_uniform_grid(orc, bc):
    n = 64
    h = _single_level(n, 3, bc)
    cons = workloads.random_state((n, n), 2, seed=6)
    out, dts, rs = orc.amr_run(h, _from_grid(h, cons), 0.8, 10.0, max_steps=5)
    grid = orc.Grid(2, [n, n], list(bc), [1.0 / n, 1.0 / n])
    ref, ref_dts, ref_rs = grid.run(orc.method(), cons.reshape(4, 1, n, n), 0.8, 10.0,
                                    max_steps=5)
    assert rs == ref_rs
    np.testing.assert_array_equal(dts, ref_dts)
    np.testing.assert_array_equal(_to_grid(h, out, n), ref.reshape(4, n, n))


def _totals(h, flat):
    """Volume-weighted totals over the cells not covered by a finer level."""
    n0 = h.n0[0]
    tot = np.zeros(4)
    cover = [np.zeros((n0 << l, n0 << l), bool) for l in range(h.nlevels)]
    for p in range(h.npatches):
        l = h.levels[p]
        if l > 0:
            x0, y0, x1, y1 = h.boxes[p]
            cover[l - 1][y0 // 2:y1 // 2, x0 // 2:x1 // 2] = True
    for p, a in enumerate(h.split(flat)):
        l = h.levels[p]
        x0, y0, x1, y1 = h.boxes[p]
        m = ~cover[l][y0:y1, x0:x1]
        dx = h.dx0 / (1 << l)
        tot += (a[:, m]).sum(axis=1) * dx * dx
    return tot


def test_uniform_state_stays_uniform(orc):
    h, _ = workloads.amr_blast_2d(64, 3, target=80, sizes=(8, 16))
    cons = h.cons_from(lambda X, Y: workloads.cons_from_prim(
        np.full_like(X, 1.3), [np.full_like(X, 0.2), np.full_like(X, -0.1)],
        np.full_like(X, 0.7)))
    out, dts, rs = orc.amr_run(h, cons, 0.8, 10.0, max_steps=3)
    np.testing.assert_array_equal(out, cons)


def test_three_level_blast_conserves(orc):
    h, cons = workloads.amr_blast_2d(64, 3, target=80, sizes=(8, 16))
    assert (np.bincount(h.levels, minlength=3) > 0).all()
    t0 = _totals(h, cons)
    out, dts, rs = orc.amr_run(h, cons, 0.8, 10.0, max_steps=6)
    assert len(dts) == 6 and np.all(np.isfinite(out))
    t1 = _totals(h, out)
    scale = np.abs(cons).max() * 1.0
    np.testing.assert_allclose(t1, t0, rtol=0, atol=1e-13 * scale)
    # the blast moved: the state changed on every level
    for l in range(3):
        sel = [p for p in range(h.npatches) if h.levels[p] == l]
        a = np.concatenate([h.split(out)[p].ravel() for p in sel])
        b = np.concatenate([h.split(cons)[p].ravel() for p in sel])
        assert np.abs(a - b).max() > 1e-3
