"""GPU parity of the exact-FP64 path against the oracle, through the C ABI.

Exact FP64 (precision "fp64_exact") performs the reference's operations in
the reference's order without FMA, so every comparison here is bit-exact
(np.testing.assert_array_equal)."""
import math

import numpy as np
import pytest

from finitevolumesolver_gb300 import workloads

pytestmark = pytest.mark.gpu
X, Y, Z = 0, 1, 2


def fromhex(a):
    return np.array([float.fromhex(x) for x in a])


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def host(t):
    return t.detach().cpu().numpy()


def complete_np(orc, rank, cons):
    shp = cons.shape[1:]
    return orc.complete_from_cons(rank, cons.reshape(rank + 2, -1)).reshape((rank + 4,) + shp)


def test_complete_from_cons(fvs, orc, torch_cuda):
    torch = torch_cuda
    for rank in (1, 2, 3):
        cons = workloads.random_state((3, 4, 5), rank, seed=rank)
        ref = complete_np(orc, rank, cons)
        u = dev(torch, cons)
        q = torch.full(ref.shape, float("nan"), dtype=torch.float64, device="cuda")
        b = ((0, 0, 0), (5, 4, 3))
        fvs.CompleteFromCons(fvs.PerfectGas(rank), q, b, u, b, b)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(host(q), ref)


@pytest.mark.parametrize("name,d", [("hlle_sin16_X", X), ("hlle_sin16_Y", Y)])
def test_hlle_sin_patch(fvs, orc, golden, torch_cuda, name, d):
    # reference tests/test.simd_FluxMethod.cpp:107-186 on the GPU
    torch = torch_cuda
    g = golden[name]
    lo, hi = g["cell_lo"], g["cell_hi"]
    ny, nx = hi[1] - lo[1], hi[0] - lo[0]
    cons = np.zeros((4, 1, ny, nx))
    for j in range(lo[1], hi[1]):
        for i in range(lo[0], hi[0]):
            x, y = float(i) * g["dx"], float(j) * g["dx"]
            cons[:, 0, j - lo[1], i - lo[0]] = [1.0, 0, 0, 1.0 + 0.5 * math.sin(x * x + y * y)]
    states = complete_np(orc, 2, cons)
    fm = fvs.FluxMethod(fvs.PerfectGas(2), "hlle")
    st = dev(torch, states)
    dt = fm.ComputeStableDt(st, (lo, hi), g["dx"], d, window_rule=0)
    assert dt == float.fromhex(g["dt"])
    fl, fh = g["face_lo"], g["face_hi"]
    fluxes = torch.full((4, 1, fh[1] - fl[1], fh[0] - fl[0]), float("nan"), dtype=torch.float64,
                        device="cuda")
    fm.ComputeNumericFluxes(fluxes, (fl, fh), st, (lo, hi), dt, g["dx"], d)
    torch.cuda.synchronize()
    ref = np.stack([fromhex(c) for c in g["fluxes"]])
    np.testing.assert_array_equal(host(fluxes).reshape(4, -1), ref)


def test_muscl_golden_stencils(fvs, orc, golden, torch_cuda):
    torch = torch_cuda
    g = golden["muscl_minmod_single"]
    cons = np.array(g["stencil"]).T.reshape(4, 1, 1, 4)
    st = dev(torch, complete_np(orc, 2, cons))
    fm = fvs.FluxMethod(fvs.PerfectGas(2), "muscl_hlle", "minmod")
    out = torch.zeros((4, 1, 1, 1), dtype=torch.float64, device="cuda")
    fm.ComputeNumericFluxes(out, ((0, 0), (1, 1)), st, ((-2, 0), (2, 1)), g["dt"], g["dx"], X)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(host(out).ravel(), fromhex(g["flux"]))
    g = golden["muscl_vanleer_3d_random"]
    fm3 = fvs.FluxMethod(fvs.PerfectGas(3))
    k = 0
    for sten in g["stencils"]:
        for d in range(3):
            shape = [1, 1, 1]
            shape[2 - d] = 4
            cons = np.array(sten).T.reshape([5] + shape)
            st = dev(torch, complete_np(orc, 3, cons))
            lo, hi = [0, 0, 0], [1, 1, 1]
            lo[d], hi[d] = -2, 2
            out = torch.zeros((5, 1, 1, 1), dtype=torch.float64, device="cuda")
            fm3.ComputeNumericFluxes(out, ((0, 0, 0), (1, 1, 1)), st, (lo, hi), g["dt"], g["dx"], d)
            torch.cuda.synchronize()
            np.testing.assert_array_equal(host(out).ravel(), fromhex(g["fluxes"][k]))
            k += 1


@pytest.mark.parametrize("rank", [1, 2, 3])
@pytest.mark.parametrize("kind", ["muscl_hlle", "hlle"])
def test_patch_fluxes_dt_update_random(fvs, orc, torch_cuda, rank, kind):
    torch = torch_cuda
    n = [11, 7, 6][:rank]
    w = 2 if kind == "muscl_hlle" else 1
    m = orc.method(orc.MUSCL_HLLE if kind == "muscl_hlle" else orc.HLLE, orc.VAN_LEER)
    fm = fvs.FluxMethod(fvs.PerfectGas(rank), kind)
    integ = fvs.HyperbolicPatchIntegrator()
    for d in range(rank):
        clo = [0] * rank
        chi = list(n)
        clo[d] -= w
        chi[d] += w
        shape = [chi[k] - clo[k] for k in range(rank)]
        cons = workloads.random_state(tuple(reversed(shape)), rank, seed=10 * rank + d)
        full = [1] * (3 - rank)
        cons = cons.reshape([rank + 2] + full + list(reversed(shape)))
        states = complete_np(orc, rank, cons)
        dx = 0.05
        for rule in (0, 1):
            dt_ref = orc.compute_stable_dt(m, rank, states, (clo, chi), dx, d, window_rule=rule)
            dt_gpu = fm.ComputeStableDt(dev(torch, states), (clo, chi), dx, d, window_rule=rule)
            assert dt_gpu == dt_ref
        dt = 0.4 * dt_ref
        flo = [0] * rank
        fhi = list(n)
        fhi[d] += 1
        ref = orc.compute_numeric_fluxes(m, rank, states, (clo, chi), (flo, fhi), dt, dx, d)
        fl = torch.full(ref.shape, float("nan"), dtype=torch.float64, device="cuda")
        st = dev(torch, states)
        fm.ComputeNumericFluxes(fl, (flo, fhi), st, (clo, chi), dt, dx, d)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(host(fl), ref)
        # update the interior cells (cons components of the complete states)
        prev = np.ascontiguousarray(states[: rank + 2])
        nxt_ref = orc.update_conservatively((flo, n), prev, (clo, chi), ref, (flo, fhi), dt, dx, d)
        nxt = torch.full(nxt_ref.shape, float("nan"), dtype=torch.float64, device="cuda")
        integ.UpdateConservatively(nxt, (flo, n), dev(torch, prev), (clo, chi), fl, (flo, fhi),
                                   rank + 2, dt, dx, d)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(host(nxt), nxt_ref)


def test_update_hand_vectors(fvs, golden, torch_cuda):
    # tests/test.HyperbolicSplitPatchIntegrator.cpp:37-71
    torch = torch_cuda
    integ = fvs.HyperbolicPatchIntegrator()
    g = golden["update_8cell"]
    prev = dev(torch, np.array(g["prev"]).reshape(1, 1, 1, 8))
    flux = dev(torch, np.array(g["flux"]).reshape(1, 1, 1, 9))
    nxt = torch.full((1, 1, 1, 8), float("nan"), dtype=torch.float64, device="cuda")
    integ.UpdateConservatively(nxt, ((0,), (8,)), prev, ((0,), (8,)), flux, ((0,), (9,)), 1,
                               1.0, 1.0, 0)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(host(nxt).ravel(), fromhex(g["next"]))


GRIDS = [
    (1, [40], [1]),
    (2, [24, 18], [0, 1]),
    (3, [20, 12, 10], [0, 0, 0]),
    (3, [9, 16, 7], [1, 0, 1]),
]


@pytest.mark.parametrize("rank,n,bc", GRIDS)
def test_solver_sweeps_and_dt(fvs, orc, rank, n, bc):
    cons = workloads.random_state(tuple(reversed(n)), rank, seed=sum(n))
    cons = cons.reshape([rank + 2] + [1] * (3 - rank) + list(reversed(n)))
    dx = [0.1, 0.07, 0.05][:rank]
    g = orc.Grid(rank, n, bc, dx)
    m = orc.method()
    s = fvs.Solver(n, dx, bc)
    for rule in (0, 1):
        s2 = fvs.Solver(n, dx, bc, dt_rule=rule)
        s2.upload(cons)
        assert s2.ComputeStableDt(-1) == g.stable_dt(m, cons, -1, rule)
        for d in range(rank):
            assert s2.ComputeStableDt(d) == g.stable_dt(m, cons, d, rule)
        s2.close()
    dt = 0.4 * g.stable_dt(m, cons)
    for seg in (0, 3):
        s.set_tiling(seg)
        for d in range(rank):
            s.upload(cons)
            level = s.sweep(d, dt)
            assert level == g.stable_dt(m, cons, d, 0)
            np.testing.assert_array_equal(s.download(), g.sweep(m, cons, dt, d))
    for cycle in (0, 1):
        s.upload(cons)
        s.step(dt, cycle)
        np.testing.assert_array_equal(s.download(), g.step(m, cons, dt, cycle))
    # the autotuner only picks segment lengths: results stay bit-identical
    s.set_tiling(0)
    s.upload(cons)
    segs = s.autotune()
    assert len(segs) == rank and all(v > 0 for v in segs)
    np.testing.assert_array_equal(s.download(), cons)
    s.step(dt, 0)
    np.testing.assert_array_equal(s.download(), g.step(m, cons, dt, 0))
    s.close()


def test_sod_1d_run_bit_exact(fvs, orc):
    n = 1024
    cons = workloads.sod_1d(n)
    g = orc.Grid(1, [n], [1], [1.0 / n])
    ref, ref_dts, ref_restarts = g.run(orc.method(), cons, 0.8, 0.2)
    s = fvs.Solver([n], [1.0 / n], "transmissive")
    s.set_tiling(32)
    s.upload(cons)
    st, dts = s.run(cfl=0.8, t_end=0.2, log_len=4096)
    assert st.steps == len(ref_dts) and st.restarts == ref_restarts
    np.testing.assert_array_equal(dts, ref_dts)
    assert st.time == pytest.approx(0.2, abs=1e-12)
    np.testing.assert_array_equal(s.download(), ref)


@pytest.mark.parametrize("rule", [0, 1])
def test_octants_3d_run_bit_exact(fvs, orc, rule):
    n = 32
    cons = workloads.octants_3d(n, seed=7)
    dx = [1.0 / n] * 3
    g = orc.Grid(3, [n] * 3, [0, 0, 0], dx)
    ref, ref_dts, ref_restarts = g.run(orc.method(), cons, 0.8, 10.0, max_steps=7, dt_rule=rule)
    s = fvs.Solver([n] * 3, dx, "periodic", dt_rule=rule)
    s.upload(cons)
    st, dts = s.run(cfl=0.8, t_end=10.0, max_steps=7, log_len=16)
    assert st.steps == 7 and st.restarts == ref_restarts
    np.testing.assert_array_equal(dts, ref_dts)
    np.testing.assert_array_equal(s.download(), ref)


def test_restart_path_matches_oracle(fvs, orc):
    # cfl 1.9 on fast random states makes later sweeps of a step fail their
    # check; the solver must redo those steps exactly like the reference's
    # backup/restart (RunSimulation.hpp:141-151)
    n = [32, 32]
    cons = workloads.random_state((32, 32), 2, seed=3, rho=(0.2, 2.0), p=(0.2, 3.0), v=1.0)
    cons = cons.reshape(4, 1, 32, 32)
    dx = [1.0 / 32, 1.0 / 32]
    g = orc.Grid(2, n, [0, 0], dx)
    ref, ref_dts, ref_restarts = g.run(orc.method(), cons, 1.9, 10.0, max_steps=10)
    assert ref_restarts == 2
    s = fvs.Solver(n, dx, "periodic")
    s.upload(cons)
    st, dts = s.run(cfl=1.9, t_end=10.0, max_steps=10, log_len=16)
    assert st.restarts == ref_restarts and st.steps == len(ref_dts)
    np.testing.assert_array_equal(dts, ref_dts)
    np.testing.assert_array_equal(s.download(), ref)


@pytest.mark.slow
def test_octants_256_full_size(fvs, orc):
    """The bench workload at full size: one sweep per direction bit-exact
    against the oracle, and a Strang step conserving mass, momentum and
    energy to round-off (periodic box)."""
    n = 256
    cons = workloads.octants_3d(n)
    dx = [1.0 / n] * 3
    g = orc.Grid(3, [n] * 3, [0, 0, 0], dx)
    m = orc.method()
    s = fvs.Solver([n] * 3, dx, "periodic")
    s.upload(cons)
    stable = s.ComputeStableDt(-1)
    assert stable == g.stable_dt(m, cons, -1, 0)
    dt = 0.8 * stable
    for d in (X, Z):
        s.upload(cons)
        s.sweep(d, 0.5 * dt)
        np.testing.assert_array_equal(s.download(), g.sweep(m, cons, 0.5 * dt, d))
    s.upload(cons)
    s.step(dt, 0)
    out = s.download()
    tot0 = cons.reshape(5, -1).sum(1)
    tot1 = out.reshape(5, -1).sum(1)
    scale = np.abs(cons).reshape(5, -1).sum(1)
    assert np.all(np.abs(tot1 - tot0) <= 1e-12 * scale)
