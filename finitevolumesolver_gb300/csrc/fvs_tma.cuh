// fvs_tma.cuh -- mbarrier and TMA (cp.async.bulk.tensor) primitives in
// inline PTX, shared by the tensor-core GEMM and the TMA-staged sweeps, and
// the host-side tensor-map encoder.
#pragma once

#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

namespace fvs {
namespace tma {

__device__ __forceinline__ uint32_t SmemAddr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void MbarInit(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(SmemAddr(bar)), "r"(count));
}

// Makes barrier initialisations visible to the asynchronous proxy.
__device__ __forceinline__ void FenceMbarInit() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Bounded wait for the mbarrier phase `parity`; returns false on timeout.
__device__ __forceinline__ bool MbarWait(uint64_t* bar, uint32_t parity, uint32_t max_polls) {
  uint32_t done = 0;
  for (uint32_t i = 0; i < max_polls; ++i) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(SmemAddr(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Orders this thread's earlier shared-memory accesses (generic proxy) before
// its later asynchronous-proxy operations on shared memory.
__device__ __forceinline__ void FenceProxyAsync() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// The next phase of `bar` completes once `bytes` of asynchronous copies
// have landed (plus this one arrival).
__device__ __forceinline__ void MbarArriveExpectTx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(SmemAddr(bar)),
               "r"(bytes)
               : "memory");
}

// TMA loads of one box of a tensor map at element coordinates into shared
// memory, completing on `bar`.  The innermost coordinate times the element
// size must be a multiple of 16 bytes; elements outside the tensor are
// filled with zeros.
__device__ __forceinline__ void TmaLoad2D(void* smem_dst, const void* tensor_map, int x, int y,
                                          uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3}], [%4];" ::"r"(SmemAddr(smem_dst)),
      "l"(reinterpret_cast<uint64_t>(tensor_map)), "r"(x), "r"(y), "r"(SmemAddr(bar))
      : "memory");
}

__device__ __forceinline__ void TmaLoad3D(void* smem_dst, const void* tensor_map, int x, int y,
                                          int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(SmemAddr(smem_dst)),
      "l"(reinterpret_cast<uint64_t>(tensor_map)), "r"(x), "r"(y), "r"(z), "r"(SmemAddr(bar))
      : "memory");
}

__device__ __forceinline__ void TmaLoad4D(void* smem_dst, const void* tensor_map, int x, int y,
                                          int z, int w, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(SmemAddr(smem_dst)),
      "l"(reinterpret_cast<uint64_t>(tensor_map)), "r"(x), "r"(y), "r"(z), "r"(w),
      "r"(SmemAddr(bar))
      : "memory");
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled from the driver, found through the runtime (no
// link-time dependency on libcuda); NULL where the driver has none.
inline EncodeTiledFn EncodeTiled() {
  static EncodeTiledFn fn = nullptr;
  static bool looked = false;
  if (!looked) {
    looked = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
    else
      cudaGetLastError();
  }
  return fn;
}

}  // namespace tma
}  // namespace fvs
