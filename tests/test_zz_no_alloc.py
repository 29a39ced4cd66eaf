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
import ctypes.util

import numpy as np
import pytest

from finitevolumesolver_gb300 import workloads

pytestmark = pytest.mark.gpu

_USED_MEM_HIGH = 8  # cudaMemPoolAttrUsedMemHigh


def _cudart():
    """The CUDA runtime the library links (already loaded by it)."""
    for name in ("libcudart.so.13", ctypes.util.find_library("cudart"),
                 "/usr/local/cuda/lib64/libcudart.so"):
        if not name:
            continue
        try:
            return C.CDLL(name)
        except OSError:
            continue
    pytest.fail("libcudart not found")


class _PoolHigh:
    """High-water mark of the device's default memory pool, the pool that
    cudaMallocAsync draws from."""

    def __init__(self):
        self.rt = _cudart()
        dev = C.c_int(0)
        assert self.rt.cudaGetDevice(C.byref(dev)) == 0
        self.pool = C.c_void_p()
        assert self.rt.cudaDeviceGetDefaultMemPool(C.byref(self.pool), dev) == 0

    def reset(self):
        zero = C.c_uint64(0)  # resets the high-water mark to the current use
        assert self.rt.cudaMemPoolSetAttribute(self.pool, _USED_MEM_HIGH, C.byref(zero)) == 0

    def high(self):
        v = C.c_uint64(0)
        assert self.rt.cudaMemPoolGetAttribute(self.pool, _USED_MEM_HIGH, C.byref(v)) == 0
        return v.value


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
        (1, (1, 1, 4099), "muscl_hlle", 0, 0, 13),
        # exactly the limit: 128 x 128 x (131 - 3) = 2,097,152 windows, which
        # fills all 8192 partial slots next to the result slot
        (3, (128, 128, 131), "muscl_hlle", 0, 1, 14),
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
        del q
        torch.cuda.empty_cache()


def test_noalloc_allocates_nothing(fvs, torch_cuda):
    """The allocating entry point raises the default pool's high-water mark
    (which shows the probe sees a cudaMallocAsync); the allocation-free one
    leaves it and torch's allocator untouched."""
    torch = torch_cuda
    L = fvs.lib()
    rank, shape = 2, (1, 64, 80)
    cons = workloads.random_state(shape[1:], rank, seed=21, v=0.8).reshape((4,) + shape)
    q = _complete_on_device(fvs, torch, rank, cons)
    torch.cuda.synchronize()
    m = fvs.make_method()
    cell_box = fvs.box([0, 0, 0], list(reversed(shape)))
    pool = _PoolHigh()
    out = C.c_double(0.0)
    pool.reset()
    before = pool.high()
    assert L.fvs_compute_stable_dt(C.byref(m), rank, q.data_ptr(), cell_box, 0.01, 0, 0,
                                   C.byref(out), None) == 0
    assert pool.high() > before
    dt_alloc = out.value
    torch.cuda.synchronize()
    pool.reset()
    before = pool.high()
    torch_before = torch.cuda.memory_allocated()
    for _ in range(2):
        assert L.fvs_compute_stable_dt_noalloc(C.byref(m), rank, q.data_ptr(), cell_box, 0.01,
                                               0, 0, C.byref(out), None) == 0
        assert out.value == dt_alloc
    assert pool.high() == before
    assert torch.cuda.memory_allocated() == torch_before


def test_noalloc_skips_nan_speed_in_lane_zero(fvs, torch_cuda, orc):
    """A cell of negative pressure (NaN sound speed) whose window is the first
    one of a warp gives a NaN face speed in lane 0; the other windows' maxima
    must survive the reduction, so dt equals the oracle's NaN-skipping dt."""
    torch = torch_cuda
    L = fvs.lib()
    rank, shape = 2, (1, 40, 300)
    cons = workloads.random_state(shape[1:], rank, seed=31, v=0.8).reshape((4,) + shape)
    states = orc.complete_from_cons(rank, cons.reshape(rank + 2, -1)).reshape((rank + 4,) + shape)
    # window 0 of dir 0 (MUSCL, w = 2) has its inner pair at x = 1, 2: the
    # right cell's NaN sound speed makes the face speed NaN
    states[rank + 2, 0, 0, 2] = -0.05
    states[rank + 3, 0, 0, 2] = np.nan
    m = fvs.make_method()
    n = list(reversed(shape))
    cell_box = fvs.box([0, 0, 0], n)
    ref = orc.compute_stable_dt(orc.method(), rank, states, ([0, 0, 0], n), 0.01, 0,
                                window_rule=0)
    assert np.isfinite(ref) and ref > 0
    q = torch.from_numpy(np.ascontiguousarray(states)).cuda()
    torch.cuda.synchronize()
    for _ in range(2):
        dt_alloc, dt_noalloc = _both(fvs, L, m, rank, q, cell_box, 0.01, 0, 0)
        assert dt_alloc == ref
        assert dt_noalloc == ref


def test_noalloc_rejects_oversized_patch(fvs):
    L = fvs.lib()
    m = fvs.make_method()
    out = C.c_double(0.0)
    # 300 x 100 x 100 cells: 297 x 100 x 100 windows > 2,097,152
    r = L.fvs_compute_stable_dt_noalloc(C.byref(m), 3, 1, fvs.box([0, 0, 0], [300, 100, 100]),
                                        0.01, 0, 1, C.byref(out), None)
    assert r == 1  # FVS_ERR_INVALID, nothing launched
    assert b"2097152" in L.fvs_last_error()
