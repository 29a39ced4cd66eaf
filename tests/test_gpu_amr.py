"""GPU tests of the batched AMR patch update against the oracle
(oracle/fvs_oracle_amr.cpp): a one-level patch set advances exactly like the
uniform grid, a three-level blast matches the oracle bit for bit (exact
FP64: ghost gathers, subcycling, refluxing, average-down, dt selection), the
launch shape and the autotuner leave results unchanged, and the mixed and
fast flavours stay conservative and close to exact FP64."""
import numpy as np
import pytest

from finitevolumesolver_gb300 import workloads

pytestmark = pytest.mark.gpu


def _single_level(n, seed, bc):
    rng = np.random.default_rng(seed)
    boxes = workloads._tiling(n, rng, sizes=(8, 16, 32))
    return workloads.AmrHierarchy(1, (n, n), bc, 1.0 / n, [0] * len(boxes), boxes)


def _grid_of(h, flat, n):
    g = np.zeros((4, n, n))
    for p, a in enumerate(h.split(flat)):
        x0, y0, x1, y1 = h.boxes[p]
        g[:, y0:y1, x0:x1] = a
    return g


def _flat_of(h, g):
    return np.concatenate([g[:, y0:y1, x0:x1].reshape(-1) for (x0, y0, x1, y1) in h.boxes])


@pytest.mark.parametrize("bc", [(1, 1), (0, 0), (0, 1)])
def test_single_level_matches_uniform_solver(fvs, orc, bc):
    n = 64
    h = _single_level(n, 3, bc)
    cons = workloads.random_state((n, n), 2, seed=6)
    a = fvs.AmrSolver(h)
    a.upload(_flat_of(h, cons))
    st, dts = a.run(cfl=0.8, t_end=10.0, max_steps=5, log_len=8)
    assert st.steps == 5
    s = fvs.Solver([n, n], [1.0 / n, 1.0 / n], [("periodic", "transmissive")[b] for b in bc])
    s.upload(cons.reshape(4, 1, n, n))
    st2, dts2 = s.run(cfl=0.8, t_end=10.0, max_steps=5, log_len=8)
    np.testing.assert_array_equal(dts, dts2)
    np.testing.assert_array_equal(_grid_of(h, a.download(), n), s.download().reshape(4, n, n))
    ref, ref_dts, rs = orc.amr_run(h, _flat_of(h, cons), 0.8, 10.0, max_steps=5)
    np.testing.assert_array_equal(a.download(), ref)


@pytest.mark.parametrize("n0,target", [(64, 80), (96, 150)])
def test_three_level_blast_bit_exact(fvs, orc, n0, target):
    h, cons = workloads.amr_blast_2d(n0, 3, target=target, sizes=(8, 16))
    a = fvs.AmrSolver(h)
    a.upload(cons)
    st, dts = a.run(cfl=0.8, t_end=10.0, max_steps=6, log_len=8)
    ref, ref_dts, rs = orc.amr_run(h, cons, 0.8, 10.0, max_steps=6)
    assert st.steps == 6 and st.restarts == rs
    np.testing.assert_array_equal(dts, ref_dts)
    np.testing.assert_array_equal(a.download(), ref)


def test_launch_shape_and_autotune_do_not_change_results(fvs, orc):
    h, cons = workloads.amr_blast_2d(64, 3, target=80, sizes=(8, 16))
    ref, _, _ = orc.amr_run(h, cons, 0.8, 10.0, max_steps=4)
    for tpr in (1, 2, 4, 8):
        a = fvs.AmrSolver(h)
        for l in range(3):
            for d in range(2):
                a.set_launch(l, d, 32, 3, tpr)
        a.upload(cons)
        a.run(cfl=0.8, t_end=10.0, max_steps=4)
        np.testing.assert_array_equal(a.download(), ref)
    b = fvs.AmrSolver(h)
    b.upload(cons)
    cfg = b.autotune()
    assert cfg.shape == (3, 2, 3) and (cfg > 0).all()
    b.run(cfl=0.8, t_end=10.0, max_steps=4)
    np.testing.assert_array_equal(b.download(), ref)


@pytest.mark.parametrize("bc", [(1, 1), (0, 0), (2, 2)])
def test_mixed_row_warp_x_sweep_matches_marching(fvs, bc):
    """The mixed x sweep with the lanes of a warp along x (rows laid end to
    end as slots, threads_per_row 32) gives the marching kernel's results bit
    for bit: halo cells from the same level and the coarser one, reflective
    images, flux-register captures and patch widths 8 to 32."""
    h, cons = workloads.amr_blast_2d(96, 3, target=150, sizes=(8, 16, 32))
    h = workloads.AmrHierarchy(h.nlevels, h.n0, bc, h.dx0, h.levels, h.boxes)
    outs = []
    for tpr, block, grid in ((1, 128, 64), (32, 128, 64), (32, 64, 3)):
        a = fvs.AmrSolver(h, fvs.make_method(precision="mixed"))
        for l in range(3):
            a.set_launch(l, 0, block, grid, tpr)
        a.upload(cons)
        st, _ = a.run(cfl=0.8, t_end=10.0, max_steps=4)
        assert st.steps == 4
        outs.append(a.download())
        if tpr == 32:
            with pytest.raises(fvs.FvsError):
                a.set_launch(0, 1, 128, 64, 32)  # y rows have no lanes-along-x kernel
        a.close()
    np.testing.assert_array_equal(outs[0], outs[1])
    np.testing.assert_array_equal(outs[0], outs[2])


def test_uniform_state_stays_uniform(fvs):
    h, _ = workloads.amr_blast_2d(64, 3, target=80, sizes=(8, 16))
    cons = h.cons_from(lambda X, Y: workloads.cons_from_prim(
        np.full_like(X, 1.3), [np.full_like(X, 0.2), np.full_like(X, -0.1)],
        np.full_like(X, 0.7)))
    for prec in ("fp64_exact", "fp64_fast", "mixed"):
        a = fvs.AmrSolver(h, fvs.make_method(precision=prec))
        a.upload(cons)
        a.run(cfl=0.8, t_end=10.0, max_steps=3)
        out = a.download()
        if prec == "fp64_exact":
            np.testing.assert_array_equal(out, cons)
        else:
            np.testing.assert_allclose(out, cons, rtol=1e-6)


def _totals(h, flat):
    n0 = h.n0[0]
    cover = [np.zeros((n0 << l, n0 << l), bool) for l in range(h.nlevels)]
    for p in range(h.npatches):
        l = h.levels[p]
        if l > 0:
            x0, y0, x1, y1 = h.boxes[p]
            cover[l - 1][y0 // 2:y1 // 2, x0 // 2:x1 // 2] = True
    tot = np.zeros(4)
    for p, a in enumerate(h.split(flat)):
        l = h.levels[p]
        x0, y0, x1, y1 = h.boxes[p]
        m = ~cover[l][y0:y1, x0:x1]
        dx = h.dx0 / (1 << l)
        tot += a[:, m].sum(axis=1) * dx * dx
    return tot


@pytest.mark.parametrize("prec", ["fp64_fast", "mixed"])
def test_flavours_conserve_and_track_exact(fvs, orc, prec):
    h, cons = workloads.amr_blast_2d(96, 3, target=150, sizes=(8, 16))
    ref, _, _ = orc.amr_run(h, cons, 0.8, 10.0, max_steps=8)
    a = fvs.AmrSolver(h, fvs.make_method(precision=prec))
    a.upload(cons)
    a.run(cfl=0.8, t_end=10.0, max_steps=8)
    out = a.download()
    t0, t1 = _totals(h, cons), _totals(h, out)
    np.testing.assert_allclose(t1, t0, rtol=0, atol=1e-13 * np.abs(cons).max())
    rho_err = np.abs(out - ref).max()
    assert rho_err < (1e-10 if prec == "fp64_fast" else 1e-4), rho_err
