"""GPU tests of the exact Riemann solver and the Godunov flux against the
oracle.  The device solver performs the reference's operations in its order
(no FMA) except that CUDA's pow differs from glibc's by a few ulps, so the
comparisons use a relative tolerance: 1e-9 at the reference's Newton
tolerance (1e-7 on |f|), where an ulp-level difference can at most flip
whether one more Newton step is taken, and 1e-12 at tolerance 1e-12."""
import numpy as np
import pytest

from finitevolumesolver_gb300 import workloads

pytestmark = pytest.mark.gpu

REF_STATES = [
    (1.0, 0.0, 1.0, 0.125, 0.0, 0.1),
    (1.0, -2.0, 0.4, 1.0, 2.0, 0.4),
    (1.0, 0.0, 1000.0, 1.0, 0.0, 0.01),
    (1.0, 0.0, 0.1, 1.0, 0.0, 100.0),
    (2.52667, 1204.31 / 2.52667, 312160.0, 2.28972, 1150.82 / 2.28972, 278308.0),
    (2.28972, 1150.82 / 2.28972, 278308.0, 2.06243, 1084.96 / 2.06243, 248331.0),
]


def gpu_star(fvs, torch, arrays, guess="mean", tol=1e-7, max_iterations=5000):
    dev = [torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda() for a in arrays]
    n = dev[0].numel()
    ps = torch.empty(n, dtype=torch.float64, device="cuda")
    us = torch.empty_like(ps)
    it = torch.empty(n, dtype=torch.int32, device="cuda")
    stt = torch.empty_like(it)
    m = fvs.make_method("godunov", guess=guess, tolerance=tol, max_iterations=max_iterations)
    fvs.exact_riemann_star(m, *dev, ps, us, it, stt)
    torch.cuda.synchronize()
    return ps.cpu().numpy(), us.cpu().numpy(), it.cpu().numpy(), stt.cpu().numpy()


@pytest.mark.parametrize("tol,rtol", [(1e-7, 1e-9), (1e-12, 1e-12)])
def test_star_states_reference_cases(fvs, orc, torch_cuda, tol, rtol):
    arr = np.array(REF_STATES).T
    ps, us, it, st = gpu_star(fvs, torch_cuda, arr, tol=tol)
    rp, ru, rit, rcv = orc.exact_star(*arr, tol=tol)
    assert (st == 1).all() and rcv.all()
    np.testing.assert_allclose(ps, rp, rtol=rtol)
    np.testing.assert_allclose(us, ru, rtol=rtol, atol=rtol * np.abs(ru).max())
    # published exact solutions (Toro, 3rd ed., Table 4.2, tests 1-3)
    # (table values carry 5-6 significant digits: 0.00189 only three)
    np.testing.assert_allclose(ps[:3], [0.30313, 0.00189, 460.894], rtol=5e-4, atol=1e-5)


@pytest.mark.parametrize("guess", ["mean", "pvrs_tr"])
def test_star_states_random_distribution(fvs, orc, torch_cuda, guess):
    arr = workloads.riemann_samples(20000, seed=4)
    g = 0 if guess == "mean" else 1
    ps, us, it, st = gpu_star(fvs, torch_cuda, arr, guess=guess, tol=1e-12, max_iterations=200)
    rp, ru, rit, rcv = orc.exact_star(*arr, guess=g, tol=1e-12, max_iterations=200)
    ok = rcv.astype(bool)
    assert ok.mean() > 0.99
    assert ((st == 1) == ok).mean() > 0.999
    np.testing.assert_allclose(ps[ok], rp[ok], rtol=1e-10)
    scale = np.maximum(np.abs(arr[1]), np.abs(arr[4]))[ok]
    assert np.all(np.abs(us[ok] - ru[ok]) <= 1e-10 * (np.abs(ru[ok]) + scale))
    # identical Newton paths up to pow's last bits: iteration counts agree
    assert (it[ok] == rit[ok]).mean() > 0.999


def test_pvrs_guess_saves_iterations(fvs, torch_cuda):
    arr = workloads.riemann_samples(20000, seed=5)
    _, _, it_mean, st_mean = gpu_star(fvs, torch_cuda, arr, guess="mean", tol=1e-12,
                                      max_iterations=200)
    _, _, it_pv, st_pv = gpu_star(fvs, torch_cuda, arr, guess="pvrs_tr", tol=1e-12,
                                  max_iterations=200)
    both = (st_mean == 1) & (st_pv == 1)
    assert it_pv[both].mean() < it_mean[both].mean()


def _complete(orc, rank, cons):
    shp = cons.shape[1:]
    return orc.complete_from_cons(rank, cons.reshape(rank + 2, -1)).reshape((rank + 4,) + shp)


@pytest.mark.parametrize("kind", ["godunov", "muscl_godunov"])
def test_patch_godunov_fluxes(fvs, orc, torch_cuda, kind):
    torch = torch_cuda
    rank = 2
    n = [13, 9]
    w = 2 if kind == "muscl_godunov" else 1
    m = orc.method(orc.GODUNOV if kind == "godunov" else orc.MUSCL_GODUNOV, orc.VAN_LEER)
    fm = fvs.FluxMethod(fvs.PerfectGas(rank), kind)
    for d in range(rank):
        clo, chi = [0, 0], list(n)
        clo[d] -= w
        chi[d] += w
        shape = [chi[k] - clo[k] for k in range(rank)]
        cons = workloads.random_state(tuple(reversed(shape)), rank, seed=31 + d, v=0.8)
        cons = cons.reshape([rank + 2, 1] + list(reversed(shape)))
        states = _complete(orc, rank, cons)
        dx = 0.05
        dt_ref = orc.compute_stable_dt(m, rank, states, (clo, chi), dx, d, window_rule=0)
        st = torch.from_numpy(states).cuda()
        dt_gpu = fm.ComputeStableDt(st, (clo, chi), dx, d, window_rule=0)
        assert dt_gpu == pytest.approx(dt_ref, rel=1e-9)
        dt = 0.4 * dt_ref
        flo, fhi = [0, 0], list(n)
        fhi[d] += 1
        ref = orc.compute_numeric_fluxes(m, rank, states, (clo, chi), (flo, fhi), dt, dx, d)
        out = torch.full(ref.shape, float("nan"), dtype=torch.float64, device="cuda")
        fm.ComputeNumericFluxes(out, (flo, fhi), st, (clo, chi), dt, dx, d)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        scale = np.abs(ref).reshape(rank + 2, -1).max(1).reshape(-1, 1, 1, 1)
        assert np.all(np.abs(got - ref) <= 1e-9 * (np.abs(ref) + scale))


def test_solver_godunov_quadrants(fvs, orc):
    n = 48
    cons = workloads.quadrants_2d(n, seed=8)
    dx = [1.0 / n, 1.0 / n]
    g = orc.Grid(2, [n, n], [1, 1], dx)
    m = orc.method(orc.GODUNOV, guess=0, tol=1e-12, max_iterations=200)
    s = fvs.Solver([n, n], dx, "transmissive",
                   method=fvs.make_method("godunov", tolerance=1e-12, max_iterations=200))
    s.upload(cons)
    dt_ref = g.stable_dt(m, cons)
    assert s.ComputeStableDt(-1) == pytest.approx(dt_ref, rel=1e-12)
    dt = 0.8 * dt_ref
    for cycle in (0, 1):
        s.upload(cons)
        s.step(dt, cycle)
        ref = g.step(m, cons, dt, cycle)
        got = s.download()
        scale = np.abs(ref).reshape(4, -1).max(1).reshape(-1, 1, 1, 1)
        assert np.all(np.abs(got - ref) <= 1e-11 * (np.abs(ref) + scale))
    it, fails = s.newton_stats(reset=True)
    assert it > 0 and fails == 0
    s.upload(cons)
    st, dts = s.run(cfl=0.8, t_end=10.0, max_steps=3, log_len=4)
    ref, ref_dts, _ = g.run(m, cons, 0.8, 10.0, max_steps=3)
    np.testing.assert_allclose(dts, ref_dts, rtol=1e-12)
    got = s.download()
    scale = np.abs(ref).reshape(4, -1).max(1).reshape(-1, 1, 1, 1)
    assert np.all(np.abs(got - ref) <= 1e-10 * (np.abs(ref) + scale))
