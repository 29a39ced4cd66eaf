"""GPU against the oracle at the sizes of the benchmark workloads.

The other GPU tests compare small grids bit for bit; these run the full-size
workloads the bench times, where the index paths differ (multi-block row
tables, segment splits, tens of thousands of patch rows per level, thousands
of cut cells):

* 3-D octants, 256^3 periodic: one Strang step in exact FP64 (bit for bit,
  also through the host-resident step fvs_solver_step_host) and in fast FP64
  (1e-12 relative per cell, tests/tolerance.py);
* 2-D AMR blast, 4096 patches on 3 levels (level 0 1024^2): one subcycled
  coarse step in exact FP64, launch shapes from the autotuner, bit for bit;
* 2-D Mach-2 shock over 8 circles, 1024^2 with 4171 cut cells: geometry,
  shielded fractions and cut flags bit for bit, two Strang steps in exact
  FP64 (bit for bit) and fast FP64 (1e-12 per cell);
* 2-D four-quadrant Godunov, 2048^2: one Strang step with the exact Riemann
  solver at Newton tolerance 1e-7 (1e-9 relative: CUDA's pow differs from
  glibc's in the last bits, which moves an iterate by ulps and can at most
  flip whether one more Newton step is taken) and at 1e-12 (1e-11).
"""
import numpy as np
import pytest

from finitevolumesolver_gb300 import workloads
from tolerance import assert_close_fp64

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


@pytest.fixture(scope="module")
def octants256():
    return workloads.octants_3d(256)


def test_octants_256_exact_strang_step_bit_exact(fvs, orc, octants256):
    n = 256
    cons = octants256
    dx = [1.0 / n] * 3
    g = orc.Grid(3, [n] * 3, [0, 0, 0], dx)
    m = orc.method()
    s = fvs.Solver([n] * 3, dx, "periodic")
    s.upload(cons)
    s.autotune()
    s.upload(cons)
    st, dts = s.run(cfl=0.8, t_end=1e9, max_steps=1, log_len=1)
    ref, ref_dts, _ = g.run(m, cons, 0.8, 1e9, max_steps=1)
    assert st.steps == 1
    np.testing.assert_array_equal(dts, ref_dts)
    np.testing.assert_array_equal(s.download(), ref)
    s.close()
    # the host-resident step of the e2e benchmark (slabbed upload and stable
    # dt, slabbed last sweep with overlapped write-back): the same bits
    import torch
    h = fvs.Solver([n] * 3, dx, "periodic")
    host = torch.from_numpy(cons.copy()).pin_memory()
    sh = h.step_host(host, cfl=0.8, t_end=1e9)
    assert sh.steps == 1 and sh.last_dt == ref_dts[0]
    np.testing.assert_array_equal(host.numpy(), ref)
    h.close()


def test_octants_256_fast_strang_step_within_1e12(fvs, orc, octants256):
    n = 256
    cons = octants256
    dx = [1.0 / n] * 3
    g = orc.Grid(3, [n] * 3, [0, 0, 0], dx)
    m = orc.method()
    s = fvs.Solver([n] * 3, dx, "periodic", method=fvs.make_method(precision="fp64_fast"))
    s.upload(cons)
    s.autotune()
    s.upload(cons)
    st, dts = s.run(cfl=0.8, t_end=1e9, max_steps=1, log_len=1)
    ref, ref_dts, _ = g.run(m, cons, 0.8, 1e9, max_steps=1)
    assert st.steps == 1
    np.testing.assert_allclose(dts, ref_dts, rtol=1e-12)
    # the same dt on both sides: compare one step of the oracle's dt
    s.upload(cons)
    s.step(float(ref_dts[0]), 0)
    worst = assert_close_fp64(s.download(), ref, 3, 1e-12, "fp64_fast 256^3")
    print("fp64_fast 256^3 worst relative error per component", worst)
    s.close()


def test_amr_4096_patches_coarse_step_bit_exact(fvs, orc):
    h, cons = workloads.amr_blast_2d(1024, 3, seed=7, target=4096)
    assert h.npatches == 4096
    a = fvs.AmrSolver(h)
    a.upload(cons)
    a.autotune()
    a.upload(cons)
    st, dts = a.run(cfl=0.8, t_end=1e9, max_steps=1, log_len=1)
    ref, ref_dts, ref_restarts = orc.amr_run(h, cons, 0.8, 1e9, max_steps=1)
    assert st.steps == 1 and st.restarts == ref_restarts
    np.testing.assert_array_equal(dts, ref_dts)
    np.testing.assert_array_equal(a.download(), ref)
    a.close()


@pytest.fixture(scope="module")
def shock1024(orc):
    n = 1024
    circles, cons = workloads.shock_circles_2d(n, seed=5)
    return n, circles, cons, orc.CutCellGeometry(n, n, circles)


def test_cutcell_1024_geometry_bit_exact(fvs, shock1024):
    n, circles, _, ref = shock1024
    s = fvs.Solver([n, n], [1.0 / n, 1.0 / n], "transmissive")
    s.set_embedded_circles(circles)
    g = s.cutcell_geometry()
    for key in ("alpha", "betax", "betay", "normal", "center"):
        np.testing.assert_array_equal(g[key], getattr(ref, key), err_msg=key)
    G = ref.G
    cut = ref.cut_cells()
    assert int(cut.sum()) == 4171
    np.testing.assert_array_equal(g["cut"][G:-G, G:-G].astype(np.int32), cut)
    names = ("us", "sL", "sR", "us_rel", "sL_rel", "sR_rel")
    for d in (0, 1):
        for name, x, y in zip(names, s.cutcell_shielded(d), ref.shielded(d)):
            np.testing.assert_array_equal(x, y, err_msg=f"{name} dir {d}")
    s.close()


@pytest.mark.parametrize("prec", ["fp64_exact", "fp64_fast"])
def test_cutcell_1024_two_steps(fvs, shock1024, prec):
    n, circles, cons, ref = shock1024
    s = fvs.Solver([n, n], [1.0 / n, 1.0 / n], "transmissive",
                   method=fvs.make_method(precision=prec))
    s.set_embedded_circles(circles)
    s.upload(cons)
    s.autotune()
    s.upload(cons)
    out, ref_dts, rs = ref.run(cons, 0.5, 1e9, max_steps=2)
    st, dts = s.run(cfl=0.5, t_end=1e9, max_steps=2, log_len=2)
    assert st.steps == 2 and st.restarts == rs
    got = s.download()
    if prec == "fp64_exact":
        np.testing.assert_array_equal(dts, ref_dts)
        np.testing.assert_array_equal(got, out)
    else:
        np.testing.assert_allclose(dts, ref_dts, rtol=1e-12)
        # covered cells hold zeros on both sides; compare the fluid cells
        G = ref.G
        fluid = ref.alpha[G:-G, G:-G] > 0
        worst = assert_close_fp64(got[:, 0][:, fluid], out[:, 0][:, fluid], 2, 1e-12,
                                  "fp64_fast cut cells 1024^2")
        print("fp64_fast cut cells worst relative error per component", worst)
        assert np.all(got[:, 0][:, ~fluid] == out[:, 0][:, ~fluid])
    s.close()


@pytest.mark.parametrize("tol,rtol", [(1e-7, 1e-9), (1e-12, 1e-11)])
def test_godunov_2048_strang_step(fvs, orc, tol, rtol):
    n = 2048
    cons = workloads.quadrants_2d(n, seed=3)
    dx = [1.0 / n, 1.0 / n]
    g = orc.Grid(2, [n, n], [1, 1], dx)
    m = orc.method(orc.GODUNOV, tol=tol)
    s = fvs.Solver([n, n], dx, "transmissive", method=fvs.make_method("godunov", tolerance=tol))
    s.upload(cons)
    dt_ref = g.stable_dt(m, cons)
    assert s.ComputeStableDt(-1) == pytest.approx(dt_ref, rel=rtol)
    dt = 0.8 * dt_ref
    s.step(dt, 0)
    got = s.download()
    ref = g.step(m, cons, dt, 0)
    worst = assert_close_fp64(got, ref, 2, rtol, f"Godunov 2048^2 tol {tol:g}")
    print(f"Godunov tol {tol:g} worst relative error per component", worst)
    it, fails = s.newton_stats(reset=True)
    assert it > 0 and fails == 0
    s.close()
