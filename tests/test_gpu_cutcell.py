"""GPU tests of the KBN h-box cut-cell path (exact FP64) against the oracle:
the library's own union-of-circles geometry, the cut-cell flags, single
sweeps and a Strang-split run, all bit for bit."""
import numpy as np
import pytest

from finitevolumesolver_gb300 import workloads

pytestmark = pytest.mark.gpu

CASES = [
    (64, [[0.5, 0.5, 0.2]]),
    (100, [[0.35, 0.4, 0.12], [0.5, 0.45, 0.1], [0.7, 0.7, 0.15]]),   # overlapping
    (96, [[0.85, 0.9, 0.15], [0.4, 0.6, 0.07]]),                       # crosses the boundary
]


def solver_with(fvs, n, circles, bc="transmissive"):
    s = fvs.Solver([n, n], [1.0 / n, 1.0 / n], bc)
    s.set_embedded_circles(circles)
    return s


@pytest.mark.parametrize("n,circles", CASES)
def test_geometry_bit_exact(fvs, orc, n, circles):
    s = solver_with(fvs, n, circles)
    g = s.cutcell_geometry()
    ref = orc.CutCellGeometry(n, n, circles)
    assert g["ghost"] == ref.G
    for key in ("alpha", "betax", "betay", "normal", "center"):
        np.testing.assert_array_equal(g[key], getattr(ref, key), err_msg=key)
    G = ref.G
    np.testing.assert_array_equal(g["cut"][G:-G, G:-G].astype(np.int32), ref.cut_cells())
    names = ("us", "sL", "sR", "us_rel", "sL_rel", "sR_rel")
    for d in (0, 1):
        for name, a, b in zip(names, s.cutcell_shielded(d), ref.shielded(d)):
            np.testing.assert_array_equal(a, b, err_msg=f"{name} dir {d}")
    s.close()


def _initial(n, circles, seed):
    rng = np.random.default_rng(seed)
    rho = rng.uniform(0.5, 1.5, (n, n))
    u = rng.uniform(-0.4, 0.4, (n, n))
    v = rng.uniform(-0.4, 0.4, (n, n))
    p = rng.uniform(0.5, 1.5, (n, n))
    return workloads.cons_from_prim(rho, [u, v], p).reshape(4, 1, n, n)


@pytest.mark.parametrize("n,circles", CASES)
def test_sweeps_bit_exact(fvs, orc, n, circles):
    s = solver_with(fvs, n, circles)
    ref = orc.CutCellGeometry(n, n, circles)
    cons = _initial(n, circles, n)
    s.upload(cons)
    dt_ref = ref.stable_dt(cons)
    assert s.ComputeStableDt(-1) == dt_ref
    dt = 0.4 * dt_ref
    for d in (0, 1):
        s.upload(cons)
        level = s.sweep(d, dt)
        assert level == ref.stable_dt(cons, d)
        np.testing.assert_array_equal(s.download(), ref.sweep(cons, cons, dt, d))
    s.close()


@pytest.mark.parametrize("launch", ["default", "tuned", "seg32"])
def test_shock_over_circles_run_bit_exact(fvs, orc, launch):
    n = 96
    circles, cons = workloads.shock_circles_2d(n, seed=5)
    ref = orc.CutCellGeometry(n, n, circles)
    s = solver_with(fvs, n, circles)
    s.upload(cons)
    if launch == "tuned":  # timed on the live state, which it leaves unchanged
        s.autotune()
    elif launch == "seg32":  # regular-cell segments of 32 cells (FP64 flavours)
        s.set_launch(0, 32, 0)
        s.set_launch(1, 32, 0)
        with pytest.raises(fvs.FvsError):
            s.set_launch(1, 32, 3)  # cut-cell grids have no occupancy variants
    st, dts = s.run(cfl=0.5, t_end=10.0, max_steps=6, log_len=8)
    out, ref_dts, rs = ref.run(cons, 0.5, 10.0, max_steps=6)
    assert st.steps == 6 and st.restarts == rs
    np.testing.assert_array_equal(dts, ref_dts)
    np.testing.assert_array_equal(s.download(), out)
    s.close()


def _totals(a):
    return a.reshape(4, -1).sum(axis=1)


@pytest.mark.parametrize("prec", ["fp64_fast", "mixed"])
@pytest.mark.parametrize("variant", [False, True])
def test_flavours_track_exact_and_conserve(fvs, orc, prec, variant):
    """Fast FP64 stays within 1e-12 of the exact flavour; mixed within the
    FP32 reconstruction error.  Periodic in x and y with the body inside the
    domain: the volume-weighted mass and energy change only through the FP64
    round-off of the cut-cell update (the wall flux carries no mass or
    energy); 1e-11 relative over 10 steps of 16k cells.  variant: segments of
    24 cells (rounded up to whole tiles of 8) for the FP64 flavours'
    regular-cell sweep."""
    n = 128
    circles = np.array([[0.5, 0.5, 0.15], [0.3, 0.7, 0.08]])
    cons = workloads.random_state((n, n), 2, seed=9).reshape(4, 1, n, n)
    ex = fvs.Solver([n, n], [1.0 / n, 1.0 / n], "periodic")
    ex.set_embedded_circles(circles)
    geo = ex.cutcell_geometry()
    G = geo["ghost"]
    alpha = geo["alpha"][G:-G, G:-G]
    cons = cons * (alpha > 0)[None, None]
    ex.upload(cons)
    st_e, dts_e = ex.run(cfl=0.5, t_end=10.0, max_steps=10, log_len=10)
    s = fvs.Solver([n, n], [1.0 / n, 1.0 / n], "periodic", method=fvs.make_method(precision=prec))
    s.set_embedded_circles(circles)
    if variant:
        for d in (0, 1):
            s.set_launch(d, 24, 0)
    s.upload(cons)
    st, dts = s.run(cfl=0.5, t_end=10.0, max_steps=10, log_len=10)
    out, ref = s.download(), ex.download()
    w = alpha[None, None]
    l1 = float(np.abs(out[0] - ref[0]).mean())
    assert l1 < (1e-12 if prec == "fp64_fast" else 2e-6), l1
    t0 = (cons * w).reshape(4, -1).sum(axis=1)
    t1 = (out * w).reshape(4, -1).sum(axis=1)
    scale = (np.abs(cons) * w).reshape(4, -1).sum(axis=1)
    drift = np.abs(t1 - t0) / scale
    assert drift[0] < 1e-11 and drift[3] < 1e-11, drift


def test_mixed_regular_cells_tile_and_march_agree(fvs):
    """The mixed flavour's regular cells of a y sweep, tiled in shared memory
    (variant 0) or marched along the column (variant 10, several segment
    lengths), and after the autotuner: the same results bit for bit."""
    n = 256
    circles, cons = workloads.shock_circles_2d(n, seed=5)
    outs = []
    for v, seg in ((0, 0), (10, 16), (10, 40), ("tuned", 0)):
        s = fvs.Solver([n, n], [1.0 / n, 1.0 / n], "transmissive",
                       method=fvs.make_method(precision="mixed"))
        s.set_embedded_circles(circles)
        s.upload(cons)
        if v == "tuned":
            s.autotune()
        else:
            s.set_launch(1, seg, v)
        st, _ = s.run(cfl=0.5, t_end=10.0, max_steps=6)
        assert st.steps == 6
        outs.append(s.download())
        if v == 10:
            with pytest.raises(fvs.FvsError):
                s.set_launch(0, seg, 10)  # x sweeps always tile
        s.close()
    for o in outs[1:]:
        np.testing.assert_array_equal(outs[0], o)


def _star_polygon(cx, cy, r0, r1, n=5, phase=0.3):
    import math
    pts = []
    for k in range(2 * n):
        r = r0 if k % 2 == 0 else r1
        t = phase + math.pi * k / n
        pts.append((cx + r * math.cos(t), cy + r * math.sin(t)))
    return pts + [pts[0]]


SHAPE_CASES = {
    "ramp": [{"kind": "halfspace", "p": (0.5, -1.0, -0.35)}],  # body below y = 0.35 + x/2
    "star": [{"kind": "polygon", "xy": _star_polygon(0.5, 0.5, 0.3, 0.18)}],
    "channel": [{"kind": "polygon", "inverted": True,
                 "xy": [(-0.1, 0.2), (1.1, 0.3), (1.1, 0.8), (-0.1, 0.7), (-0.1, 0.2)]}],
    "union": [{"kind": "halfspace", "p": (-0.2, 1.0, 0.85)},
              {"kind": "circle", "p": (0.55, 0.4, 0.15)},
              {"kind": "polygon", "xy": [(0.1, 0.1), (0.3, 0.1), (0.2, 0.3), (0.1, 0.1)]}],
}


@pytest.mark.parametrize("case", list(SHAPE_CASES))
def test_general_geometry_bit_exact(fvs, orc, case):
    n = 100
    shapes = SHAPE_CASES[case]
    s = fvs.Solver([n, n], [1.0 / n, 1.0 / n], "transmissive")
    s.set_embedded_geometry(shapes)
    g = s.cutcell_geometry()
    ref = orc.CutCellGeometry(n, n, shapes=shapes)
    for key in ("alpha", "betax", "betay", "normal", "center"):
        np.testing.assert_array_equal(g[key], getattr(ref, key), err_msg=key)
    G = ref.G
    np.testing.assert_array_equal(g["cut"][G:-G, G:-G].astype(np.int32), ref.cut_cells())
    assert ref.cut_cells().sum() > 0
    s.close()


@pytest.mark.parametrize("case", ["ramp", "union"])
def test_shock_over_general_geometry_run_bit_exact(fvs, orc, case):
    n = 96
    shapes = SHAPE_CASES[case]
    _, cons = workloads.shock_circles_2d(n, seed=5)
    ref = orc.CutCellGeometry(n, n, shapes=shapes)
    s = fvs.Solver([n, n], [1.0 / n, 1.0 / n], "transmissive")
    s.set_embedded_geometry(shapes)
    s.upload(cons)
    st, dts = s.run(cfl=0.5, t_end=10.0, max_steps=6, log_len=8)
    out, ref_dts, rs = ref.run(cons, 0.5, 10.0, max_steps=6)
    assert st.steps == 6 and st.restarts == rs
    np.testing.assert_array_equal(dts, ref_dts)
    np.testing.assert_array_equal(s.download(), out)
    s.close()


# The wedge of the reference's tests/test.AMReX.EB.plane_nan.cpp:32-53 (the
# cone y < 0.1 - 0.9 |x| on [-0.5, 0.5] x [0, 1], 64 x 64 cells, its apex on
# the grid line x = 0), as a polygon cut off below the domain.
WEDGE = [{"kind": "polygon", "xy": [(0.0, 0.1), (1.0, -0.8), (-1.0, -0.8), (0.0, 0.1)]}]


def test_wedge_geometry_and_run_bit_exact(fvs, orc):
    n = 64
    ref = orc.CutCellGeometry(n, n, x0=-0.5, y0=0.0, shapes=WEDGE)
    s = fvs.Solver([n, n], [1.0 / n, 1.0 / n], "transmissive")
    s.set_embedded_geometry(WEDGE, x0=-0.5, y0=0.0)
    g = s.cutcell_geometry()
    for key in ("alpha", "betax", "betay", "normal", "center"):
        assert np.isfinite(g[key]).all(), key
        np.testing.assert_array_equal(g[key], getattr(ref, key), err_msg=key)
    G = ref.G
    np.testing.assert_array_equal(g["cut"][G:-G, G:-G].astype(np.int32), ref.cut_cells())
    for d in (0, 1):
        for a, b in zip(s.cutcell_shielded(d), ref.shielded(d)):
            np.testing.assert_array_equal(a, b)
    _, cons = workloads.shock_circles_2d(n, seed=5, x_shock=0.38)  # reaches the wedge
    s.upload(cons)
    st, dts = s.run(cfl=0.5, t_end=10.0, max_steps=8, log_len=8)
    out, ref_dts, rs = ref.run(cons, 0.5, 10.0, max_steps=8)
    assert st.steps == 8 and st.restarts == rs
    np.testing.assert_array_equal(dts, ref_dts)
    np.testing.assert_array_equal(s.download(), out)
    assert np.isfinite(out).all()
    s.close()
