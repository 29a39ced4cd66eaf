"""fvs_compute_stable_dt_noalloc -- the allocation-free stable-dt entry point.

It exists for callers that cannot let a library allocate device memory (an
integrator that owns every device byte through its own arena, where a hidden
cudaMalloc/cudaFree would synchronise the device, escape the arena's budget
and can fail once the arena holds the memory).  It reduces through a fixed
array inside the library instead of a per-call allocation, and must return
the same dt as fvs_compute_stable_dt -- bit for bit, the tolerance of every
exact-FP64 test here -- on consecutive calls that reuse that array.

The file name sorts last so that a run stopping at the first failure has
already run every other test.  The test inputs are placed on the device by
the test itself; the entry point under test allocates nothing.
"""
import ctypes as C

import numpy as np
import pytest

from finitevolumesolver_gb300 import workloads

pytestmark = pytest.mark.gpu


def _complete_on_device(fvs, torch, rank, cons):
    """Complete states (rank+4 components) computed on the GPU from cons."""
    shape = cons.shape[1:]
    u = torch.from_numpy(np.ascontiguousarray(cons)).cuda()
    q = torch.empty((rank + 4,) + shape, dtype=torch.float64, device="cuda")
    n = list(reversed(shape))
    b = fvs.box([0, 0, 0], n)
    fvs.CompleteFromCons(fvs.PerfectGas(rank), q, b, u, b, b)
    return q


def _both(fvs, L, method, rank, q, cell_box, dx, d, rule):
    a = C.c_double(-1.0)
    b = C.c_double(-2.0)
    r1 = L.fvs_compute_stable_dt(C.byref(method), rank, q.data_ptr(), cell_box, dx, d, rule,
                                 C.byref(a), None)
    r2 = L.fvs_compute_stable_dt_noalloc(C.byref(method), rank, q.data_ptr(), cell_box, dx, d,
                                         rule, C.byref(b), None)
    assert r1 == 0 and r2 == 0, L.fvs_last_error()
    return a.value, b.value


def test_noalloc_stable_dt_matches_allocating_entry_point(fvs, torch_cuda):
    torch = torch_cuda
    L = fvs.lib()
    # two calls in a row: a large patch (many blocks of partial maxima) and
    # then a smaller one, so the second call runs over the slots the first
    # one left behind
    cases = [
        (3, (40, 64, 96), "muscl_hlle", 0, 1, 11),
        (2, (1, 50, 70), "hlle", 1, 0, 12),
    ]
    for rank, shape, kind, d, rule, seed in cases:
        cons = workloads.random_state(shape[3 - rank:], rank, seed=seed, v=0.8)
        cons = cons.reshape((rank + 2,) + shape)
        q = _complete_on_device(fvs, torch, rank, cons)
        torch.cuda.synchronize()
        m = fvs.make_method(kind)
        n = list(reversed(shape))
        cell_box = fvs.box([0, 0, 0], n)
        dt_alloc, dt_noalloc = _both(fvs, L, m, rank, q, cell_box, 0.01, d, rule)
        assert np.isfinite(dt_alloc) and dt_alloc > 0
        assert dt_noalloc == dt_alloc


def test_noalloc_rejects_oversized_patch(fvs):
    L = fvs.lib()
    m = fvs.make_method()
    out = C.c_double(0.0)
    # 300 x 100 x 100 cells: 297 x 100 x 100 windows > 2,097,152
    r = L.fvs_compute_stable_dt_noalloc(C.byref(m), 3, 1, fvs.box([0, 0, 0], [300, 100, 100]),
                                        0.01, 0, 1, C.byref(out), None)
    assert r == 1  # FVS_ERR_INVALID, nothing launched
    assert b"2097152" in L.fvs_last_error()
