"""fvs_solver_step_host: one split step of a host-resident state, whose
last sweep runs in slabs with each slab's copy to the host started as soon
as the slab is final, equals uploading, running one step and downloading,
bit for bit: ranks 1-3, both cycle parities (the last sweep is x or the
last direction), every boundary kind, the exact, fast and mixed flavours,
the end-time clamp and restarts after failed checks."""
import numpy as np
import pytest

from finitevolumesolver_gb300 import workloads

pytestmark = pytest.mark.gpu


def _state(rank, shape, seed):
    if rank == 3:
        full = workloads.octants_3d(max(shape), seed=seed)
        return np.ascontiguousarray(full[:, :shape[2], :shape[1], :shape[0]])
    st = workloads.random_state(tuple(shape[::-1]), rank, seed=seed, v=0.7)
    return np.ascontiguousarray(st.reshape(rank + 2, *shape[::-1]))


@pytest.mark.parametrize("rank,shape,bc", [
    (1, [300], "transmissive"), (2, [70, 45], "periodic"), (2, [33, 64], "reflective"),
    (3, [40, 36, 28], "periodic"), (3, [24, 20, 30], "transmissive")])
@pytest.mark.parametrize("precision", ["fp64_exact", "fp64_fast", "mixed"])
def test_step_host_matches_upload_run_download(fvs, torch_cuda, rank, shape, bc, precision):
    torch = torch_cuda
    cons = _state(rank, shape, 5)
    dx = [1.0 / 64] * rank
    m = fvs.make_method(precision=precision)
    a = fvs.Solver(shape, dx, bc, method=m)
    b = fvs.Solver(shape, dx, bc, method=m)
    host = torch.from_numpy(cons.copy()).pin_memory()
    ref = cons.copy()
    b.upload(ref)
    for step in range(3):  # both parities of the split sequence
        st = a.step_host(host, cfl=0.8)
        sb, _ = b.run(cfl=0.8, t_end=1e300, max_steps=1)
        assert st.steps == 1 and sb.steps == 1
        assert st.last_dt == sb.last_dt and st.time == sb.time
        np.testing.assert_array_equal(host.numpy(), b.download().reshape(host.shape))
    np.testing.assert_array_equal(a.download(), b.download())
    a.close()
    b.close()


def test_step_host_end_time_and_pageable_memory(fvs):
    n = 32
    cons = _state(3, [n] * 3, 9)
    s = fvs.Solver([n] * 3, [1.0 / n] * 3, "periodic", method=fvs.make_method(precision="fp64_fast"))
    host = cons.copy()  # pageable numpy memory works too (copies are staged)
    st = s.step_host(host, cfl=0.8, t_end=1e-4)
    assert st.steps == 1 and st.time == 1e-4 and st.last_dt == 1e-4
    before = host.copy()
    st = s.step_host(host, cfl=0.8, t_end=1e-4)  # t >= t_end: nothing to do
    assert st.steps == 0
    np.testing.assert_array_equal(host, before)
    s.close()


def test_step_host_restarts_like_run(fvs, torch_cuda):
    """cfl 1.2 makes per-sweep checks fail on the blast: both paths restart
    the same number of times and end in the same state."""
    torch = torch_cuda
    n = 48
    cons = _state(3, [n] * 3, 3)
    m = fvs.make_method(precision="fp64_exact")
    a = fvs.Solver([n] * 3, [1.0 / n] * 3, "periodic", method=m)
    b = fvs.Solver([n] * 3, [1.0 / n] * 3, "periodic", method=m)
    host = torch.from_numpy(cons.copy()).pin_memory()
    b.upload(cons)
    ra = rb = 0
    for _ in range(4):
        st = a.step_host(host, cfl=1.2)
        sb, _ = b.run(cfl=1.2, t_end=1e300, max_steps=1)
        ra += st.restarts
        rb += sb.restarts
        np.testing.assert_array_equal(host.numpy(), b.download())
    assert ra == rb
    a.close()
    b.close()


def test_step_host_refuses_cut_cells(fvs):
    s = fvs.Solver([32, 32], [1 / 32, 1 / 32], "transmissive", method=fvs.make_method(precision="fp64_fast"))
    s.set_embedded_circles([[0.5, 0.5, 0.2]])
    with pytest.raises(fvs.FvsError):
        s.step_host(np.zeros((4, 1, 32, 32)))
    s.close()


@pytest.mark.parametrize("flux_method", ["godunov", "muscl_godunov", "hllem", "muscl_char"])
def test_step_host_other_flux_methods(fvs, torch_cuda, flux_method):
    """The slabbed last sweep and the unpiped upload of methods other than
    MUSCL-HLLE / HLLE (whose stable-dt pass has no plane ranges) give the same
    steps as upload, run and download."""
    torch = torch_cuda
    shape = [24, 20, 18]
    cons = _state(3, shape, 7)
    m = fvs.make_method(flux_method=flux_method)
    a = fvs.Solver(shape, [1.0 / 32] * 3, "transmissive", method=m)
    b = fvs.Solver(shape, [1.0 / 32] * 3, "transmissive", method=m)
    host = torch.from_numpy(cons.copy()).pin_memory()
    b.upload(cons)
    for _ in range(2):
        st = a.step_host(host, cfl=0.8)
        sb, _ = b.run(cfl=0.8, t_end=1e300, max_steps=1)
        assert st.steps == 1 and st.last_dt == sb.last_dt
        np.testing.assert_array_equal(host.numpy(), b.download())
    a.close()
    b.close()
