"""The patch-level calls on host-resident patches (fvs_*_host through a patch
context) equal the device-pointer calls and the oracle bit for bit, for
patches of different sizes through one context (its staging buffers grow)."""
import numpy as np
import pytest

from finitevolumesolver_gb300 import workloads

pytestmark = pytest.mark.gpu


def _complete(orc, rank, cons):
    shp = cons.shape[1:]
    return orc.complete_from_cons(rank, cons.reshape(rank + 2, -1)).reshape((rank + 4,) + shp)


@pytest.mark.parametrize("kind", ["muscl_hlle", "hlle", "muscl_hllem"])
def test_host_patch_calls_match_oracle(fvs, orc, torch_cuda, kind):
    torch = torch_cuda
    ctx = fvs.HostPatchContext()
    kinds = {"muscl_hlle": orc.MUSCL_HLLE, "hlle": orc.HLLE, "muscl_hllem": orc.MUSCL_HLLEM}
    for rank, n in ((1, [40]), (2, [17, 11]), (3, [9, 7, 6]), (2, [33, 29])):
        fm = fvs.FluxMethod(fvs.PerfectGas(rank), kind)
        m = orc.method(kinds[kind])
        w = fm.GetStencilWidth()
        integ = fvs.HyperbolicPatchIntegrator()
        for d in range(rank):
            clo, chi = [0] * rank, list(n)
            clo[d] -= w
            chi[d] += w
            shape = [chi[k] - clo[k] for k in range(rank)]
            cons = workloads.random_state(tuple(reversed(shape)), rank, seed=7 * rank + d, v=0.7)
            cons = np.ascontiguousarray(
                cons.reshape([rank + 2] + [1] * (3 - rank) + list(reversed(shape))))
            # CompleteFromCons on the host patch
            states = np.full((rank + 4,) + cons.shape[1:], np.nan)
            ctx.CompleteFromCons(fvs.PerfectGas(rank), states, (clo, chi), cons, (clo, chi),
                                 (clo, chi))
            np.testing.assert_array_equal(states, _complete(orc, rank, cons))
            dx = 0.05
            dt_h = ctx.ComputeStableDt(fm, states, (clo, chi), dx, d, window_rule=0)
            assert dt_h == orc.compute_stable_dt(m, rank, states, (clo, chi), dx, d,
                                                 window_rule=0)
            dt = 0.4 * dt_h
            flo, fhi = [0] * rank, list(n)
            fhi[d] += 1
            ref = orc.compute_numeric_fluxes(m, rank, states, (clo, chi), (flo, fhi), dt, dx, d)
            fl = np.full(ref.shape, np.nan)
            ctx.ComputeNumericFluxes(fm, fl, (flo, fhi), states, (clo, chi), dt, dx, d)
            np.testing.assert_array_equal(fl, ref)
            # the same call through device pointers
            st = torch.from_numpy(states).cuda()
            fd = torch.full(ref.shape, float("nan"), dtype=torch.float64, device="cuda")
            fm.ComputeNumericFluxes(fd, (flo, fhi), st, (clo, chi), dt, dx, d)
            torch.cuda.synchronize()
            np.testing.assert_array_equal(fd.cpu().numpy(), fl)
            # UpdateConservatively of the interior
            sl = [slice(None)] * 4
            sl[3 - d] = slice(w, w + n[d])  # the interior cells along d
            prev = np.ascontiguousarray(cons[tuple(sl)])
            ibox = (flo, list(n))
            nxt = np.full(prev.shape, np.nan)
            ctx.UpdateConservatively(nxt, ibox, prev, ibox, fl, (flo, fhi), rank + 2, dt, dx, d)
            np.testing.assert_array_equal(
                nxt, orc.update_conservatively(ibox, prev, ibox, fl, (flo, fhi), dt, dx, d))
    ctx.close()
