// fvs_tcgen05.cuh -- BF16 GEMM on the 5th-generation tensor cores (tcgen05,
// accumulators in tensor memory), hand-written in inline PTX for sm_103a.
//
//   C[M x N] (+)= A[M x K] . B[N x K]^T      A, B bf16 (K contiguous), C fp32
//
// One CTA computes a 128 x N tile of C over a K range (split-K over
// blockIdx.y accumulates with atomicAdd).  Per K chunk of 64 one thread
// issues TMA loads (cp.async.bulk.tensor.2d) of the A and B tiles, one box of
// 8 elements (16 bytes) x rows per 8-element K slice, which lands in shared
// memory as the canonical no-swizzle K-major layout: 8-row x 16-byte core
// matrices, element (r, k) at (k/8)*LBO + (r/8)*SBO + (r%8)*16 + (k%8)*2
// bytes with SBO = 128 and LBO = rows*16.  The copies complete on an
// mbarrier (expect_tx); then one thread issues
// tcgen05.mma.cta_group::1.kind::f16 with M = 128, K = 16 per instruction,
// and tcgen05.commit arrives on a second mbarrier when the MMAs have
// completed.  Every wait is bounded and a timeout sets an error flag instead
// of hanging.  The accumulator (128 lanes x N fp32 columns of tensor memory)
// is read back with tcgen05.ld: warp w reads lanes 32w..32w+31, i.e. rows
// 32w..32w+31 of the tile.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>

#include "fvs_tma.cuh"

namespace fvs {
namespace tc {

using tma::FenceProxyAsync;
using tma::MbarArriveExpectTx;
using tma::MbarInit;
using tma::MbarWait;
using tma::SmemAddr;
using tma::TmaLoad2D;

constexpr int kTileM = 128;
constexpr int kChunkK = 64;
constexpr int kThreads = 128;

// Shared-memory matrix descriptor (tcgen05): start address, leading- and
// stride-dimension byte offsets (all >> 4), descriptor version 1 at bits
// 46-47, no swizzle (layout type 0 at bits 61-63).
__device__ __forceinline__ uint64_t SmemDesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= uint64_t((addr >> 4) & 0x3FFF);
  d |= uint64_t((lbo >> 4) & 0x3FFF) << 16;
  d |= uint64_t((sbo >> 4) & 0x3FFF) << 32;
  d |= uint64_t(1) << 46;
  return d;
}

// Instruction descriptor of kind::f16: D fp32 (bits 4-5 = 1), A and B bf16
// (bits 7-9 and 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at
// bits 24-28.
__host__ __device__ constexpr uint32_t InstrDescBf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(n >> 3) << 17) | (uint32_t(m >> 4) << 24);
}

__device__ __forceinline__ void TmemAlloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   SmemAddr(dst_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void TmemDealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void Mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                    uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void Commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          SmemAddr(bar))
      : "memory");
}

__device__ __forceinline__ void FenceBeforeSync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void FenceAfterSync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// 16 fp32 columns of this thread's TMEM lane starting at column `col`.
__device__ __forceinline__ void TmemLoad16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace fvs
