"""GPU tests of the fast FP64 and the mixed-precision flavours.

fast FP64 ("fp64_fast") and double-float ("fp64_df"): within 1e-12 relative
per cell of the oracle (the tolerance stated for the plain FP64 path: FMA
contraction and reordered divisions), per call and over whole runs: purely
relative for density and energy, relative to the cell's value plus the
component's largest magnitude for the momenta, which cross zero
(tests/tolerance.py).

mixed ("mixed"): FP32 reconstruction and flux, FP64 state and update.  The
state after a step differs from the FP64 oracle by FP32 round-off in the
fluxes (L1 density error per step bounded below), while mass, momentum and
energy of a periodic box are conserved to FP64 round-off.
"""
import numpy as np
import pytest

from finitevolumesolver_gb300 import workloads
from tolerance import assert_close_fp64

pytestmark = pytest.mark.gpu

RTOL_FP64 = 1e-12


GRIDS = [
    (1, [64], [1]),
    (2, [40, 24], [0, 1]),
    (3, [24, 20, 16], [0, 0, 0]),
]


@pytest.mark.parametrize("prec", ["fp64_fast", "fp64_df"])
@pytest.mark.parametrize("rank,n,bc", GRIDS)
def test_fast_fp64_sweeps_and_steps(fvs, orc, rank, n, bc, prec):
    cons = workloads.random_state(tuple(reversed(n)), rank, seed=7 + rank, v=0.6)
    cons = cons.reshape([rank + 2] + [1] * (3 - rank) + list(reversed(n)))
    dx = [0.1, 0.07, 0.05][:rank]
    g = orc.Grid(rank, n, bc, dx)
    m = orc.method()
    s = fvs.Solver(n, dx, bc, method=fvs.make_method(precision=prec))
    s.upload(cons)
    dt_ref = g.stable_dt(m, cons)
    assert s.ComputeStableDt(-1) == pytest.approx(dt_ref, rel=RTOL_FP64)
    dt = 0.4 * dt_ref
    for d in range(rank):
        s.upload(cons)
        level = s.sweep(d, dt)
        assert level == pytest.approx(g.stable_dt(m, cons, d, 0), rel=RTOL_FP64)
        assert_close_fp64(s.download(), g.sweep(m, cons, dt, d), rank, RTOL_FP64)
    for cycle in (0, 1):
        s.upload(cons)
        s.step(dt, cycle)
        assert_close_fp64(s.download(), g.step(m, cons, dt, cycle), rank, RTOL_FP64)
    s.close()


@pytest.mark.parametrize("prec", ["fp64_fast", "fp64_df"])
def test_fast_fp64_octants_run(fvs, orc, prec):
    n = 32
    cons = workloads.octants_3d(n, seed=5)
    dx = [1.0 / n] * 3
    g = orc.Grid(3, [n] * 3, [0, 0, 0], dx)
    ref, ref_dts, _ = g.run(orc.method(), cons, 0.8, 10.0, max_steps=4)
    s = fvs.Solver([n] * 3, dx, "periodic", method=fvs.make_method(precision=prec))
    s.upload(cons)
    st, dts = s.run(cfl=0.8, t_end=10.0, max_steps=4, log_len=8)
    assert st.steps == 4
    np.testing.assert_allclose(dts, ref_dts, rtol=1e-12)
    assert_close_fp64(s.download(), ref, 3, RTOL_FP64)


def test_mixed_precision_step_accuracy_and_conservation(fvs, orc):
    n = 48
    cons = workloads.octants_3d(n, seed=9)
    dx = [1.0 / n] * 3
    g = orc.Grid(3, [n] * 3, [0, 0, 0], dx)
    m = orc.method()
    s = fvs.Solver([n] * 3, dx, "periodic", method=fvs.make_method(precision="mixed"))
    s.upload(cons)
    dt = 0.8 * g.stable_dt(m, cons)
    s.step(dt, 0)
    out = s.download()
    ref = g.step(m, cons, dt, 0)
    # L1 density error of one Strang step, relative to the mean density
    l1 = np.abs(out[0] - ref[0]).mean() / np.abs(ref[0]).mean()
    assert l1 < 2e-7, l1
    # conservation to FP64 round-off over several steps
    tot0 = cons.reshape(5, -1).sum(1)
    scale = np.abs(cons).reshape(5, -1).sum(1)
    s.upload(cons)
    st, _ = s.run(cfl=0.8, t_end=10.0, max_steps=10)
    tot = s.download().reshape(5, -1).sum(1)
    assert np.all(np.abs(tot - tot0) <= 1e-13 * scale), (tot - tot0) / scale


def test_mixed_sod_1d(fvs, orc):
    n = 1024
    cons = workloads.sod_1d(n)
    g = orc.Grid(1, [n], [1], [1.0 / n])
    ref, ref_dts, _ = g.run(orc.method(), cons, 0.8, 0.2)
    s = fvs.Solver([n], [1.0 / n], "transmissive", method=fvs.make_method(precision="mixed"))
    s.set_tiling(32)
    s.upload(cons)
    st, dts = s.run(cfl=0.8, t_end=0.2, log_len=4096)
    assert st.time == pytest.approx(0.2, abs=1e-12)
    out = s.download()
    l1 = np.abs(out[0] - ref[0]).mean()
    assert l1 < 1e-5, l1


@pytest.mark.parametrize("bc", ["periodic", "transmissive"])
@pytest.mark.parametrize("nx", [256, 100, 33, 32, 31])  # full and partial last chunks of 32
def test_mixed_x_sweep_matches_marching_kernel(fvs, bc, nx):
    """The mixed x sweep (lanes along x, shuffles) and the marching y sweep
    evaluate the same per-face and per-cell arithmetic.  A state that varies
    only along the sweep direction, with zero transverse momentum, must give
    bit-identical results in x and in y."""
    rng = np.random.default_rng(nx)
    ny = 8
    rho = rng.uniform(0.5, 1.5, nx)
    u = rng.uniform(-0.5, 0.5, nx)
    p = rng.uniform(0.5, 1.5, nx)
    A = workloads.cons_from_prim(np.tile(rho, (ny, 1)), [np.tile(u, (ny, 1)), np.zeros((ny, nx))],
                                 np.tile(p, (ny, 1))).reshape(4, 1, ny, nx)
    B = workloads.cons_from_prim(np.tile(rho[:, None], (1, ny)),
                                 [np.zeros((nx, ny)), np.tile(u[:, None], (1, ny))],
                                 np.tile(p[:, None], (1, ny))).reshape(4, 1, nx, ny)
    m = fvs.make_method(precision="mixed")
    sa = fvs.Solver([nx, ny], [0.01, 0.01], bc, method=m)
    sb = fvs.Solver([ny, nx], [0.01, 0.01], bc, method=m)
    sa.upload(A)
    sb.upload(B)
    la = sa.sweep(0, 1e-3)
    lb = sb.sweep(1, 1e-3)
    assert la == lb
    a = sa.download()
    b = sb.download()
    np.testing.assert_array_equal(a[0, 0], b[0, 0].T)
    np.testing.assert_array_equal(a[1, 0], b[2, 0].T)
    np.testing.assert_array_equal(a[3, 0], b[3, 0].T)


@pytest.mark.parametrize("xvariant", [0, 4, 5, 10, 14, 15])
def test_mixed_launch_variants(fvs, orc, xvariant):
    """Every launch variant of the mixed x sweep (lanes along x or marching,
    three register budgets) gives the same accuracy and conservation, and the
    y/z variants run too."""
    n = 40
    cons = workloads.octants_3d(n, seed=12)
    dx = [1.0 / n] * 3
    g = orc.Grid(3, [n] * 3, [0, 0, 0], dx)
    m = orc.method()
    s = fvs.Solver([n] * 3, dx, "periodic", method=fvs.make_method(precision="mixed"))
    s.set_launch(0, 16, xvariant)
    s.set_launch(1, 16, xvariant % 10)
    s.set_launch(2, 32, xvariant % 10)
    assert s.tuning()[1] == [xvariant, xvariant % 10, xvariant % 10]
    s.upload(cons)
    dt = 0.8 * g.stable_dt(m, cons)
    s.step(dt, 0)
    out = s.download()
    ref = g.step(m, cons, dt, 0)
    l1 = np.abs(out[0] - ref[0]).mean() / np.abs(ref[0]).mean()
    assert l1 < 2e-7, l1
    s.upload(cons)
    s.run(cfl=0.8, t_end=10.0, max_steps=6)
    tot0 = cons.reshape(5, -1).sum(1)
    scale = np.abs(cons).reshape(5, -1).sum(1)
    tot = s.download().reshape(5, -1).sum(1)
    assert np.all(np.abs(tot - tot0) <= 1e-13 * scale)
    with pytest.raises(fvs.FvsError):
        s.set_launch(1, 16, 10)  # the marching-x variants exist for x only
    s.close()


@pytest.mark.parametrize("rank,nx,bc,seg", [
    (3, 50, "periodic", 16), (3, 64, "transmissive", 0), (3, 34, "reflective", 7),
    (2, 98, "periodic", 0), (2, 66, "reflective", 24)])
@pytest.mark.parametrize("variant", [20, 24, 25])
def test_mixed_tma_sweeps_match_marching(fvs, rank, nx, bc, seg, variant):
    """The TMA-staged y/z sweep (cells staged into shared memory by
    cp.async.bulk.tensor) runs the marching sweep's arithmetic on the same
    cells: its Strang steps equal the marching kernel's bit for bit, for x
    extents that are not multiples of the 32-cell box, ragged segments and
    every boundary kind."""
    shape = [nx, 28, 20][:rank]
    dx = [1.0 / 64] * rank
    cons = (workloads.octants_3d(64, seed=31)[:, :shape[2], :shape[1], :shape[0]]
            if rank == 3 else workloads.random_state((shape[1], shape[0]), 2, seed=31, v=0.6))
    cons = np.ascontiguousarray(cons.reshape(rank + 2, *shape[::-1]))
    outs = []
    for v in (variant % 10, variant):
        s = fvs.Solver(shape, dx, bc, method=fvs.make_method(precision="mixed"))
        for d in range(1, rank):
            s.set_launch(d, seg, v)
        s.upload(cons)
        st, _ = s.run(cfl=0.8, t_end=10.0, max_steps=4)
        assert st.steps == 4
        outs.append(s.download())
        s.close()
    np.testing.assert_array_equal(outs[0], outs[1])


def test_mixed_tma_variant_needs_even_nx(fvs):
    """TMA rows must start on 16-byte boundaries: an odd x extent has no
    TMA-staged variant, and x sweeps never have one."""
    s = fvs.Solver([33, 16, 8], [0.1] * 3, "periodic", method=fvs.make_method(precision="mixed"))
    with pytest.raises(fvs.FvsError):
        s.set_launch(1, 16, 20)
    s.close()
    s = fvs.Solver([32, 16, 8], [0.1] * 3, "periodic", method=fvs.make_method(precision="mixed"))
    s.set_launch(1, 16, 20)
    with pytest.raises(fvs.FvsError):
        s.set_launch(0, 16, 20)
    s.close()
