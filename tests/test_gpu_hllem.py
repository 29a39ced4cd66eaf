"""GPU parity of the HLLEM flux (Hllem<PerfectGas, Larrouturou>) and of
MUSCL-Hancock + HLLEM against the oracle, bit for bit: patch-level fluxes
and stable dt in every direction and rank, and whole Strang runs."""
import numpy as np
import pytest

from finitevolumesolver_gb300 import workloads

pytestmark = pytest.mark.gpu


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def complete_np(orc, rank, cons):
    shp = cons.shape[1:]
    return orc.complete_from_cons(rank, cons.reshape(rank + 2, -1)).reshape((rank + 4,) + shp)


@pytest.mark.parametrize("kind", ["hllem", "muscl_hllem"])
@pytest.mark.parametrize("rank", [1, 2, 3])
def test_patch_fluxes_and_dt_bit_exact(fvs, orc, torch_cuda, kind, rank):
    torch = torch_cuda
    n = [9, 7, 6][:rank] + [1] * (3 - rank)
    cons = workloads.random_state(tuple(reversed(n)), rank, seed=10 + rank)
    states = complete_np(orc, rank, cons)
    okind = orc.HLLEM if kind == "hllem" else orc.MUSCL_HLLEM
    w = 1 if kind == "hllem" else 2
    fm = fvs.FluxMethod(fvs.PerfectGas(rank), kind)
    st = dev(torch, states)
    lo, hi = [0, 0, 0], n[:]
    for d in range(rank):
        flo = lo[:]
        fhi = hi[:]
        flo[d] = w
        fhi[d] = n[d] - w + 1
        shape = (rank + 2,) + tuple(fhi[k] - flo[k] for k in (2, 1, 0))
        out = torch.full(shape, float("nan"), dtype=torch.float64, device="cuda")
        fm.ComputeNumericFluxes(out, (flo, fhi), st, (lo, hi), 1e-3, 0.05, d)
        torch.cuda.synchronize()
        ref = orc.compute_numeric_fluxes(orc.method(okind), rank, states, (lo, hi), (flo, fhi),
                                         1e-3, 0.05, d)
        np.testing.assert_array_equal(out.cpu().numpy(), ref)
        for rule in (0, 1):
            dt = fm.ComputeStableDt(st, (lo, hi), 0.05, d, window_rule=rule)
            rdt = orc.compute_stable_dt(orc.method(okind), rank, states, (lo, hi), 0.05, d,
                                        window_rule=rule)
            assert dt == rdt


@pytest.mark.parametrize("kind,rank,n,bc", [("muscl_hllem", 2, 48, "periodic"),
                                             ("hllem", 2, 40, "transmissive"),
                                             ("muscl_hllem", 3, 16, "periodic"),
                                             ("muscl_hllem", 1, 200, "transmissive")])
def test_runs_bit_exact(fvs, orc, kind, rank, n, bc):
    shape = (n,) * rank
    cons = workloads.random_state(tuple(reversed(shape)), rank, seed=rank + 3,
                                  rho=(0.5, 1.5), p=(0.5, 1.5), v=0.3)
    cons = cons.reshape((rank + 2,) + (1,) * (3 - rank) + tuple(reversed(shape)))
    okind = orc.HLLEM if kind == "hllem" else orc.MUSCL_HLLEM
    b = 0 if bc == "periodic" else 1
    g = orc.Grid(rank, [n] * rank, [b] * rank, [1.0 / n] * rank)
    ref, ref_dts, rs = g.run(orc.method(okind), cons, 0.6, 10.0, max_steps=5)
    s = fvs.Solver([n] * rank, [1.0 / n] * rank, bc, method=fvs.make_method(kind))
    s.upload(cons)
    st, dts = s.run(cfl=0.6, t_end=10.0, max_steps=5, log_len=8)
    assert st.steps == 5 and st.restarts == rs
    np.testing.assert_array_equal(dts, ref_dts)
    np.testing.assert_array_equal(s.download(), ref.reshape(s.download().shape))


def test_hllem_needs_exact_fp64(fvs):
    with pytest.raises(fvs.FvsError):
        fvs.Solver([16, 16], [1 / 16, 1 / 16], "periodic",
                   method=fvs.make_method("muscl_hllem", precision="mixed"))
