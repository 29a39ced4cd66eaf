"""GPU parity of the characteristic and primitive MUSCL-Hancock methods (both
with the HLLEM face flux) against the oracle, bit for bit: patch-level fluxes
and stable dt in every rank and direction, whole Strang runs, and runs with
the reference's tiled stable-dt rule, whose windows depend on the method's
stencil width (checked here for every HLLEM and Godunov method)."""
import numpy as np
import pytest

from finitevolumesolver_gb300 import workloads
from tolerance import assert_close_fp64

pytestmark = pytest.mark.gpu

KINDS = {"muscl_char": "MUSCL_CHAR", "muscl_prim": "MUSCL_PRIM"}


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def complete_np(orc, rank, cons):
    shp = cons.shape[1:]
    return orc.complete_from_cons(rank, cons.reshape(rank + 2, -1)).reshape((rank + 4,) + shp)


@pytest.mark.parametrize("kind", list(KINDS))
@pytest.mark.parametrize("rank", [1, 2, 3])
def test_patch_fluxes_and_dt_bit_exact(fvs, orc, torch_cuda, kind, rank):
    torch = torch_cuda
    n = [10, 8, 7][:rank] + [1] * (3 - rank)
    cons = workloads.random_state(tuple(reversed(n)), rank, seed=40 + rank)
    states = complete_np(orc, rank, cons)
    okind = getattr(orc, KINDS[kind])
    fm = fvs.FluxMethod(fvs.PerfectGas(rank), kind)
    st = dev(torch, states)
    lo, hi = [0, 0, 0], n[:]
    for d in range(rank):
        flo, fhi = lo[:], hi[:]
        flo[d] = 2
        fhi[d] = n[d] - 1
        shape = (rank + 2,) + tuple(fhi[k] - flo[k] for k in (2, 1, 0))
        for dt in (1e-3, 7e-3):
            out = torch.full(shape, float("nan"), dtype=torch.float64, device="cuda")
            fm.ComputeNumericFluxes(out, (flo, fhi), st, (lo, hi), dt, 0.05, d)
            torch.cuda.synchronize()
            ref = orc.compute_numeric_fluxes(orc.method(okind), rank, states, (lo, hi),
                                             (flo, fhi), dt, 0.05, d)
            np.testing.assert_array_equal(out.cpu().numpy(), ref)
        for rule in (0, 1):
            dt = fm.ComputeStableDt(st, (lo, hi), 0.05, d, window_rule=rule)
            rdt = orc.compute_stable_dt(orc.method(okind), rank, states, (lo, hi), 0.05, d,
                                        window_rule=rule)
            assert dt == rdt


@pytest.mark.parametrize("kind,rank,n,bc", [("muscl_char", 2, 48, "periodic"),
                                             ("muscl_prim", 2, 40, "transmissive"),
                                             ("muscl_char", 3, 16, "transmissive"),
                                             ("muscl_prim", 3, 16, "periodic"),
                                             ("muscl_char", 1, 200, "transmissive"),
                                             ("muscl_prim", 1, 160, "periodic")])
def test_runs_bit_exact(fvs, orc, kind, rank, n, bc):
    shape = (n,) * rank
    cons = workloads.random_state(tuple(reversed(shape)), rank, seed=rank + 11,
                                  rho=(0.5, 1.5), p=(0.5, 1.5), v=0.3)
    cons = cons.reshape((rank + 2,) + (1,) * (3 - rank) + tuple(reversed(shape)))
    okind = getattr(orc, KINDS[kind])
    b = 0 if bc == "periodic" else 1
    g = orc.Grid(rank, [n] * rank, [b] * rank, [1.0 / n] * rank)
    ref, ref_dts, rs = g.run(orc.method(okind), cons, 0.6, 10.0, max_steps=6)
    s = fvs.Solver([n] * rank, [1.0 / n] * rank, bc, method=fvs.make_method(kind))
    s.upload(cons)
    st, dts = s.run(cfl=0.6, t_end=10.0, max_steps=6, log_len=8)
    assert st.steps == 6 and st.restarts == rs
    np.testing.assert_array_equal(dts, ref_dts)
    np.testing.assert_array_equal(s.download(), ref.reshape(s.download().shape))
    s.close()


def test_sod_octants_3d_bit_exact(fvs, orc):
    """The 3-D octant problem (strong discontinuities, clipped slopes) with the
    characteristic method."""
    n = 24
    cons = workloads.octants_3d(n, seed=2)
    g = orc.Grid(3, [n] * 3, [1] * 3, [1.0 / n] * 3)
    ref, ref_dts, _ = g.run(orc.method(orc.MUSCL_CHAR), cons, 0.8, 10.0, max_steps=4)
    s = fvs.Solver([n] * 3, [1.0 / n] * 3, "transmissive", method=fvs.make_method("muscl_char"))
    s.upload(cons)
    st, dts = s.run(cfl=0.8, t_end=10.0, max_steps=4, log_len=4)
    np.testing.assert_array_equal(dts, ref_dts)
    np.testing.assert_array_equal(s.download(), ref)
    s.close()


@pytest.mark.parametrize("kind", ["hllem", "muscl_hllem", "muscl_char", "muscl_prim",
                                  "godunov", "muscl_godunov", "muscl_hlle"])
def test_tiled_dt_rule_uses_stencil_width(fvs, orc, kind):
    """dt_rule 1 takes the faces of the reference's MFIter tiles, whose
    windows span 2 w cells for a stencil width w.  Bit for bit, except for
    the exact Riemann solver, whose powers of pressure ratios (n-th roots on
    the GPU, glibc's pow() in the oracle) differ in the last bits: dt within
    1e-12 relative and the state within 1e-12 per cell there (momenta
    relative to the component's largest magnitude, as they cross zero)."""
    n = (20, 21)
    cons = workloads.random_state((n[1], n[0]), 2, seed=5, rho=(0.5, 1.5), p=(0.5, 1.5),
                                  v=0.4).reshape(4, 1, n[1], n[0])
    okind = getattr(orc, kind.upper())
    g = orc.Grid(2, list(n), [1, 1], [1.0 / n[0], 1.0 / n[1]])
    ref, ref_dts, _ = g.run(orc.method(okind), cons, 0.6, 10.0, max_steps=3, dt_rule=1)
    s = fvs.Solver(list(n), [1.0 / n[0], 1.0 / n[1]], "transmissive",
                   method=fvs.make_method(kind), dt_rule=1)
    s.upload(cons)
    st, dts = s.run(cfl=0.6, t_end=10.0, max_steps=3, log_len=4)
    if "godunov" in kind:
        np.testing.assert_allclose(dts, ref_dts, rtol=1e-12)
        assert_close_fp64(s.download(), ref, 2, 1e-12, kind)
    else:
        np.testing.assert_array_equal(dts, ref_dts)
        np.testing.assert_array_equal(s.download(), ref)
    s.close()


def test_variants_reject_limiter_and_precision(fvs):
    for kind in KINDS:
        with pytest.raises(fvs.FvsError):
            fvs.Solver([16, 16], [1 / 16, 1 / 16], "periodic",
                       method=fvs.make_method(kind, limiter="minmod"))
        with pytest.raises(fvs.FvsError):
            fvs.Solver([16, 16], [1 / 16, 1 / 16], "periodic",
                       method=fvs.make_method(kind, precision="mixed"))


@pytest.mark.parametrize("kind", ["hllem", "muscl_hllem", "muscl_char"])
@pytest.mark.parametrize("bc", ["transmissive", "periodic"])
@pytest.mark.parametrize("rule", [0, 1])
def test_3d_stable_dt_faces(fvs, orc, kind, bc, rule):
    """The 3-D stable-dt pass (rows of 31 cells per warp, marching in z) takes
    every face of the reference's rule: x rows longer than a warp, odd
    extents, both boundary kinds, both window rules; bit for bit."""
    n = (35, 9, 13)
    cons = workloads.random_state((n[2], n[1], n[0]), 3, seed=8, rho=(0.5, 1.5),
                                  p=(0.5, 1.5), v=0.4)
    okind = getattr(orc, kind.upper())
    b = 0 if bc == "periodic" else 1
    dx = [1.0 / n[0], 1.0 / n[1], 1.0 / n[2]]
    g = orc.Grid(3, list(n), [b] * 3, dx)
    ref, ref_dts, _ = g.run(orc.method(okind), cons, 0.6, 10.0, max_steps=2, dt_rule=rule)
    s = fvs.Solver(list(n), dx, bc, method=fvs.make_method(kind), dt_rule=rule)
    s.upload(cons)
    st, dts = s.run(cfl=0.6, t_end=10.0, max_steps=2, log_len=2)
    np.testing.assert_array_equal(dts, ref_dts)
    np.testing.assert_array_equal(s.download(), ref)
    s.close()
