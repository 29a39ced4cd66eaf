"""GPU parity of reflective walls and of the NoLimiter / NoGradient slopes
against the oracle, through the C ABI: exact FP64 bit for bit, fast FP64
within 1e-12 per cell (tests/tolerance.py), the mixed flavour by its L1
error and by exact mass and energy balance in a closed box."""
import numpy as np
import pytest

from finitevolumesolver_gb300 import workloads
from tolerance import assert_close_fp64

pytestmark = pytest.mark.gpu

LIMITERS = {"van_leer": 0, "no_limiter": 2, "no_gradient": 3}

GRIDS = [
    (1, [64], ["reflective"]),
    (2, [40, 24], ["reflective", "periodic"]),
    (2, [36, 28], ["transmissive", "reflective"]),
    (3, [24, 20, 16], ["periodic", "reflective", "reflective"]),
]
BCI = {"periodic": 0, "transmissive": 1, "reflective": 2}


def _state(rank, n, seed):
    cons = workloads.random_state(tuple(reversed(n)), rank, seed=seed, v=0.7)
    return cons.reshape([rank + 2] + [1] * (3 - rank) + list(reversed(n)))


@pytest.mark.parametrize("limiter", list(LIMITERS))
@pytest.mark.parametrize("rank,n,bc", GRIDS)
def test_exact_sweeps_steps_and_run(fvs, orc, rank, n, bc, limiter):
    cons = _state(rank, n, 20 + rank)
    dx = [0.1, 0.07, 0.05][:rank]
    g = orc.Grid(rank, n, [BCI[b] for b in bc], dx)
    m = orc.method(limiter=LIMITERS[limiter])
    s = fvs.Solver(n, dx, bc, method=fvs.make_method(limiter=limiter))
    s.upload(cons)
    assert s.ComputeStableDt(-1) == g.stable_dt(m, cons)
    dt = 0.4 * g.stable_dt(m, cons)
    for d in range(rank):
        s.upload(cons)
        assert s.sweep(d, dt) == g.stable_dt(m, cons, d, 0)
        np.testing.assert_array_equal(s.download(), g.sweep(m, cons, dt, d))
    for cycle in (0, 1):
        s.upload(cons)
        s.step(dt, cycle)
        np.testing.assert_array_equal(s.download(), g.step(m, cons, dt, cycle))
    s.upload(cons)
    s.set_cycle(0)
    s.set_time(0.0)
    st, dts = s.run(cfl=0.8, t_end=10.0, max_steps=5, log_len=8)
    ref, ref_dts, _ = g.run(m, cons, 0.8, 10.0, max_steps=5)
    np.testing.assert_array_equal(dts, ref_dts)
    np.testing.assert_array_equal(s.download(), ref)
    s.close()


@pytest.mark.parametrize("prec", ["fp64_fast", "fp64_df"])
@pytest.mark.parametrize("rank,n,bc", GRIDS)
def test_fast_flavours_reflective(fvs, orc, rank, n, bc, prec):
    cons = _state(rank, n, 30 + rank)
    dx = [0.1, 0.07, 0.05][:rank]
    g = orc.Grid(rank, n, [BCI[b] for b in bc], dx)
    s = fvs.Solver(n, dx, bc, method=fvs.make_method(precision=prec, limiter="no_limiter"))
    s.upload(cons)
    st, dts = s.run(cfl=0.8, t_end=10.0, max_steps=4, log_len=8)
    ref, ref_dts, _ = g.run(orc.method(limiter=orc.NO_LIMITER), cons, 0.8, 10.0, max_steps=4)
    np.testing.assert_allclose(dts, ref_dts, rtol=1e-12)
    assert_close_fp64(s.download(), ref, rank, 1e-12, f"{prec} reflective")
    s.close()


@pytest.mark.parametrize("xvariant", [0, 4, 10])
def test_mixed_closed_box(fvs, orc, xvariant):
    """Walls on every side, mixed precision: the state tracks the FP64
    oracle to the FP32 reconstruction error, and the interior fluxes cancel
    exactly in the FP64 update, so mass and energy change only through the
    walls.  There the flux of a state and its mirror image is an FP32
    expression (with FMA contraction) whose mass and energy parts cancel to
    FP32 round-off rather than to zero (exactly zero in the exact flavour):
    5e-12 relative after 10 steps, bounded here by 1e-10.  The lanes-along-x
    variants (0, 4) run their x sweeps with the marching kernel on reflective
    rows."""
    n = 48
    cons = workloads.octants_3d(n, seed=9)
    dx = [1.0 / n] * 3
    g = orc.Grid(3, [n] * 3, [2, 2, 2], dx)
    m = orc.method()
    s = fvs.Solver([n] * 3, dx, "reflective", method=fvs.make_method(precision="mixed"))
    s.set_launch(0, 16, xvariant)
    s.upload(cons)
    dt = 0.8 * g.stable_dt(m, cons)
    s.step(dt, 0)
    l1 = np.abs(s.download()[0] - g.step(m, cons, dt, 0)[0]).mean()
    assert l1 < 2e-7, l1
    s.upload(cons)
    s.run(cfl=0.8, t_end=10.0, max_steps=10)
    out = s.download()
    for c in (0, 4):
        assert abs(out[c].sum() - cons[c].sum()) <= 1e-10 * abs(cons[c]).sum()
    s.close()


@pytest.mark.parametrize("kind", ["godunov", "muscl_hllem"])
def test_other_methods_reflective(fvs, orc, kind):
    n = [40, 32]
    cons = _state(2, n, 41)
    dx = [1.0 / 40, 1.0 / 32]
    g = orc.Grid(2, n, [2, 2], dx)
    if kind == "godunov":
        m = orc.method(orc.GODUNOV, tol=1e-12, max_iterations=200)
        fm = fvs.make_method("godunov", tolerance=1e-12, max_iterations=200)
    else:
        m = orc.method(orc.MUSCL_HLLEM)
        fm = fvs.make_method("muscl_hllem")
    s = fvs.Solver(n, dx, "reflective", method=fm)
    s.upload(cons)
    st, dts = s.run(cfl=0.8, t_end=10.0, max_steps=3, log_len=4)
    ref, ref_dts, _ = g.run(m, cons, 0.8, 10.0, max_steps=3)
    if kind == "godunov":  # CUDA's pow differs from glibc's in the last bits
        np.testing.assert_allclose(dts, ref_dts, rtol=1e-12)
        assert_close_fp64(s.download(), ref, 2, 1e-11, "Godunov reflective")
    else:
        np.testing.assert_array_equal(dts, ref_dts)
        np.testing.assert_array_equal(s.download(), ref)
    s.close()


@pytest.mark.parametrize("limiter", list(LIMITERS))
def test_cutcell_reflective_walls(fvs, orc, limiter):
    n = 96
    circles, cons = workloads.shock_circles_2d(n, seed=5)
    ref = orc.CutCellGeometry(n, n, circles)
    s = fvs.Solver([n, n], [1.0 / n, 1.0 / n], "reflective",
                   method=fvs.make_method(limiter=limiter))
    s.set_embedded_circles(circles)
    s.upload(cons)
    st, dts = s.run(cfl=0.5, t_end=10.0, max_steps=6, log_len=8)
    out, ref_dts, rs = ref.run(cons, 0.5, 10.0, max_steps=6, bc=(2, 2),
                               limiter=LIMITERS[limiter])
    assert st.steps == 6 and st.restarts == rs
    np.testing.assert_array_equal(dts, ref_dts)
    np.testing.assert_array_equal(s.download(), out)
    s.close()


def test_amr_reflective_walls(fvs, orc):
    """A 3-level patch set in a closed box whose flow runs into every wall
    (a swirl of speed up to 0.5 plus density and pressure waves), so the
    reflected halo states of every level are exercised."""
    h, _ = workloads.amr_blast_2d(64, 3, target=60, bc=(2, 2), sizes=(8, 16))

    def fn(X, Y):
        rho = 1.0 + 0.3 * np.sin(7 * X) * np.cos(5 * Y)
        u = 0.5 * np.sin(np.pi * Y)
        v = -0.4 * np.cos(np.pi * X)
        p = 1.0 + 0.2 * np.cos(9 * X + 4 * Y)
        return workloads.cons_from_prim(rho, [u, v], p)

    cons = h.cons_from(fn)
    a = fvs.AmrSolver(h)
    a.upload(cons)
    st, dts = a.run(cfl=0.8, t_end=10.0, max_steps=2, log_len=2)
    ref, ref_dts, _ = orc.amr_run(h, cons, 0.8, 10.0, max_steps=2)
    assert st.steps == 2
    np.testing.assert_array_equal(dts, ref_dts)
    np.testing.assert_array_equal(a.download(), ref)
    a.close()
