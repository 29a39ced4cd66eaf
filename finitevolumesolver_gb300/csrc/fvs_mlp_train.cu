// fvs_mlp_train.cu -- the learned Newton start value: tcgen05 GEMM, training
// (forward, backward, Adam) and batched inference of the 5 -> 64 -> 64 -> 1
// GELU perceptron, all hand-written for sm_103a.
//
// Layout of the network (B = batch rows, a multiple of 128):
//   X   [B][16] bf16   standardised features, columns 5..15 zero
//   Z1  [B][64] fp32 = X W1^T + b1,  H1 = GELU(Z1) (bf16 [B][64] and [64][B])
//   Z2  [B][64] fp32 = H1 W2^T + b2, H2 = GELU(Z2)
//   y   [B]          = H2 . w3 + b3   (CUDA cores)
// Loss: mean squared error against y* = log(p* / max(pL, pR)).
// Backward: dZ2 = (dy w3) * GELU'(Z2); dH1 = dZ2 W2 (tcgen05);
// dW2 = dZ2^T H1 (tcgen05, split over the batch); dZ1 = dH1 * GELU'(Z1);
// dW1 = dZ1^T X (tcgen05).  The M = 64 weight-gradient products run as
// M = 128 tiles whose upper 64 rows are loaded as zeros and not stored.
#include "../../include/fvs_gpu.h"
#include "fvs_internal.h"
#include "fvs_mlp.cuh"
#include "fvs_tcgen05.cuh"

#include <cuda.h>
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

namespace fvs {
namespace mlpk {

constexpr int kH = mlp::kHidden;  // 64
constexpr int kXin = 16;          // padded input width

// ---------------------------------------------------------------------------
// tcgen05 GEMM: C[M x N] (+)= A[M x K] . B[N x K]^T

struct GemmArgs {
  const __nv_bfloat16* A;
  int lda;
  const __nv_bfloat16* B;
  int ldb;
  float* C;
  int ldc;
  int M, K;
  int k_per_cta;  // multiple of 16; blockIdx.y selects the K range
  int atomic;     // 1: atomicAdd into C (split K), 0: store
  int* error;
};

// Operands arrive by TMA: for every 8-element K slice of a chunk, one 2-D
// tensor-map box of 16 bytes x rows lands as `rows` consecutive 16-byte rows,
// i.e. a column of 8 x 16-byte core matrices.  In the canonical K-major
// no-swizzle layout that is SBO = 128 bytes (next 8-row group) and LBO =
// rows * 16 bytes (next K slice).  Rows beyond the tensor are zero-filled.
template <int N>
__global__ void __launch_bounds__(tc::kThreads)
    TcGemmKernel(GemmArgs a, const __grid_constant__ CUtensorMap tmA,
                 const __grid_constant__ CUtensorMap tmB) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full_bar, mma_bar;
  __shared__ uint32_t tmem_base;
  const uint32_t raw = tc::SmemAddr(smem_raw);
  uint8_t* sA = smem_raw + ((1024u - (raw & 1023u)) & 1023u);
  uint8_t* sB = sA + tc::kTileM * tc::kChunkK * 2;
  constexpr uint32_t kCols = N < 32 ? 32 : N;
  constexpr uint32_t kSbo = 128;
  constexpr uint32_t kLboA = tc::kTileM * 16;
  constexpr uint32_t kLboB = N * 16;
  constexpr uint32_t kIdesc = tc::InstrDescBf16(tc::kTileM, N);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * tc::kTileM;
  const int k_begin = blockIdx.y * a.k_per_cta;
  const int k_end = min(a.K, k_begin + a.k_per_cta);
  if (warp == 0) tc::TmemAlloc(&tmem_base, kCols);
  if (tid == 0) {
    tc::MbarInit(&full_bar, 1);
    tc::MbarInit(&mma_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::FenceBeforeSync();
  __syncthreads();
  tc::FenceAfterSync();
  const uint32_t tmem = tmem_base;
  uint32_t phase = 0;
  bool ok = true;       // CTA-uniform: decided with __syncthreads_or
  bool pending = false;  // copies or MMAs issued but not seen complete
  bool first = true;
  for (int kc = k_begin; kc < k_end && ok; kc += tc::kChunkK) {
    const int slices = min(tc::kChunkK, k_end - kc) / 8;
    if (tid == 0) {
      tc::MbarArriveExpectTx(&full_bar, uint32_t(slices) * (kLboA + kLboB));
      for (int sl = 0; sl < slices; ++sl) {
        tc::TmaLoad2D(sA + sl * kLboA, &tmA, kc + 8 * sl, m0, &full_bar);
        tc::TmaLoad2D(sB + sl * kLboB, &tmB, kc + 8 * sl, 0, &full_bar);
      }
    }
    pending = true;
    const bool landed = tc::MbarWait(&full_bar, phase, 1u << 22);
    ok = !__syncthreads_or(landed ? 0 : 1);
    if (!ok) break;
    if (tid == 0) {
      tc::FenceAfterSync();
      const uint32_t abase = tc::SmemAddr(sA), bbase = tc::SmemAddr(sB);
      for (int ks = 0; ks < slices / 2; ++ks) {
        const uint64_t ad = tc::SmemDesc(abase + 2 * ks * kLboA, kLboA, kSbo);
        const uint64_t bd = tc::SmemDesc(bbase + 2 * ks * kLboB, kLboB, kSbo);
        tc::Mma(tmem, ad, bd, kIdesc, (first && ks == 0) ? 0u : 1u);
      }
      tc::Commit(&mma_bar);
    }
    first = false;
    const bool done = tc::MbarWait(&mma_bar, phase, 1u << 22);
    tc::FenceAfterSync();
    ok = !__syncthreads_or(done ? 0 : 1);
    if (ok) {
      phase ^= 1u;
      pending = false;
    }
  }
  if (!ok && pending) {
    // A copy or the tensor core did not signal in time: record it and give
    // the copies and MMAs of this chunk a second bounded chance to drain
    // before shared and tensor memory are released.
    if (tid == 0 && a.error) atomicOr(a.error, 1);
    tc::MbarWait(&full_bar, phase, 1u << 22);
    tc::MbarWait(&mma_bar, phase, 1u << 22);
  }
  if (ok && !first) {
    const int row = m0 + warp * 32 + lane;
#pragma unroll
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      tc::TmemLoad16(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0), v);
      if (row < a.M) {
        float* crow = a.C + int64_t(row) * a.ldc + c0;
        if (a.atomic) {
#pragma unroll
          for (int i = 0; i < 16; ++i) atomicAdd(crow + i, v[i]);
        } else {
#pragma unroll
          for (int i = 0; i < 16; ++i) crow[i] = v[i];
        }
      }
    }
  }
  tc::FenceBeforeSync();
  __syncthreads();
  if (warp == 0) tc::TmemDealloc(tmem, kCols);
}

using tma::EncodeTiled;
using tma::EncodeTiledFn;

// Tensor map of a row-major bf16 matrix [rows][inner] with row pitch `ld`
// elements; boxes of 8 elements x box_rows rows.
cudaError_t MakeOperandMap(CUtensorMap* m, const __nv_bfloat16* base, int inner, int rows, int ld,
                           int box_rows) {
  EncodeTiledFn fn = EncodeTiled();
  if (!fn) return cudaErrorNotSupported;
  const cuuint64_t dims[2] = {cuuint64_t(inner), cuuint64_t(rows)};
  const cuuint64_t strides[1] = {cuuint64_t(ld) * 2};
  const cuuint32_t box[2] = {8u, cuuint32_t(box_rows)};
  const cuuint32_t estr[2] = {1u, 1u};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                        const_cast<__nv_bfloat16*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

template <int N>
cudaError_t LaunchGemm(const GemmArgs& a, int splits, cudaStream_t s) {
  // the operands' rows must start on 16-byte boundaries (TMA global strides)
  if ((a.lda % 8) != 0 || (a.ldb % 8) != 0 || (reinterpret_cast<uintptr_t>(a.A) & 15) != 0 ||
      (reinterpret_cast<uintptr_t>(a.B) & 15) != 0 || (a.K % 16) != 0 || (a.k_per_cta % 16) != 0)
    return cudaErrorInvalidValue;
  alignas(64) CUtensorMap tmA, tmB;
  cudaError_t e = MakeOperandMap(&tmA, a.A, a.K, a.M, a.lda, tc::kTileM);
  if (e == cudaSuccess) e = MakeOperandMap(&tmB, a.B, a.K, N, a.ldb, N);
  if (e != cudaSuccess) return e;
  const size_t smem = 1024 + size_t(tc::kTileM) * tc::kChunkK * 2 + size_t(N) * tc::kChunkK * 2;
  static bool attr_set = false;
  if (!attr_set) {
    e = cudaFuncSetAttribute(TcGemmKernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(smem));
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  dim3 grid(unsigned((a.M + tc::kTileM - 1) / tc::kTileM), unsigned(splits));
  TcGemmKernel<N><<<grid, tc::kThreads, smem, s>>>(a, tmA, tmB);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Elementwise parts

__device__ __forceinline__ float Gelu(float x) { return mlp::Gelu(x); }

__device__ __forceinline__ float GeluGrad(float x) {
  const float k0 = 0.7978845608028654f, k1 = 0.044715f;
  const float t = tanhf(k0 * fmaf(k1 * x * x, x, x));
  return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * k0 * fmaf(3.0f * k1, x * x, 1.0f);
}

// Features and labels of Riemann problems given by primitive states.
__global__ void FeaturesKernel(int64_t n, const double* rhoL, const double* uL, const double* pL,
                               const double* rhoR, const double* uR, const double* pR,
                               const double* pstar, double gamma, float* feat, float* label) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double aL = sqrt(gamma * pL[i] / rhoL[i]);
  const double aR = sqrt(gamma * pR[i] / rhoR[i]);
  float x[mlp::kIn];
  mlp::Features(x, rhoL[i], uL[i], pL[i], aL, rhoR[i], uR[i], pR[i], aR);
#pragma unroll
  for (int k = 0; k < mlp::kIn; ++k) feat[i * mlp::kIn + k] = x[k];
  if (label && pstar) {
    const double pref = pL[i] > pR[i] ? pL[i] : pR[i];
    label[i] = static_cast<float>(log(pstar[i] / pref));
  }
}

// Mean and standard deviation of the raw features (double accumulation).
__global__ void MomentsKernel(int64_t n, const float* feat, double* acc) {
  double s[mlp::kIn] = {0}, q[mlp::kIn] = {0};
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
#pragma unroll
    for (int k = 0; k < mlp::kIn; ++k) {
      const double v = feat[i * mlp::kIn + k];
      s[k] += v;
      q[k] += v * v;
    }
  }
#pragma unroll
  for (int k = 0; k < mlp::kIn; ++k) {
    atomicAdd(acc + k, s[k]);
    atomicAdd(acc + mlp::kIn + k, q[k]);
  }
}

struct Net {
  // fp32 master parameters in the inference blob layout (mlp::kParams floats)
  float* master;
  // Adam moments, same layout
  float* m1;
  float* m2;
  float* grad;
  // inference blob: bf16-rounded weights widened to fp32
  float* blob;
  __nv_bfloat16* W1;   // [64][16]
  __nv_bfloat16* W2;   // [64][64]
  __nv_bfloat16* W2t;  // [64][64] transposed
};

// bf16 copies of the weights and the inference blob from the master weights.
__global__ void PublishKernel(Net net) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= mlp::kParams) return;
  const float w = net.master[i];
  float out = w;
  if (i >= mlp::kOffW1 && i < mlp::kOffB1) {
    const int o = (i - mlp::kOffW1) / mlp::kIn, k = (i - mlp::kOffW1) % mlp::kIn;
    const __nv_bfloat16 b = __float2bfloat16_rn(w);
    net.W1[o * kXin + k] = b;
    out = __bfloat162float(b);
  } else if (i >= mlp::kOffW2 && i < mlp::kOffB2) {
    const int o = (i - mlp::kOffW2) / kH, k = (i - mlp::kOffW2) % kH;
    const __nv_bfloat16 b = __float2bfloat16_rn(w);
    net.W2[o * kH + k] = b;
    net.W2t[k * kH + o] = b;
    out = __bfloat162float(b);
  }
  net.blob[i] = out;
}

struct StepBuffers {
  int batch;
  const float* feat;   // raw features [n][5]
  const float* label;  // [n]
  int64_t n;
  uint64_t seed;
  unsigned long long* step;  // device step counter
  __nv_bfloat16* X;    // [B][16]
  __nv_bfloat16* Xt;   // [16][B]
  float* target;       // [B]
  float* Z1;           // [B][64]
  __nv_bfloat16* H1;   // [B][64]
  __nv_bfloat16* H1t;  // [64][B]
  float* Z2;           // [B][64]
  __nv_bfloat16* D2;   // dZ2 [B][64]
  __nv_bfloat16* D2t;  // dZ2^T [64][B]
  float* dH1;          // [B][64]
  __nv_bfloat16* D1t;  // dZ1^T [64][B]
  float* dW2;          // [64][64]
  float* dW1;          // [64][16]
  float* loss;         // accumulated loss (sum of squared errors)
  int use_given_rows;  // 1: rows are 0..B-1 of feat (gradient check)
};

__device__ __forceinline__ uint64_t Mix(uint64_t x) {
  // SplitMix64 finaliser
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Sample the batch rows, standardise the features, write X and X^T.
__global__ void GatherKernel(StepBuffers b, const float* stats) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= b.batch) return;
  int64_t row;
  if (b.use_given_rows) {
    row = r;
  } else {
    const uint64_t h = Mix(b.seed ^ Mix(*b.step * 0x100000001ull + uint64_t(r)));
    row = int64_t(h % uint64_t(b.n));
  }
  for (int k = 0; k < kXin; ++k) {
    float v = 0.0f;
    if (k < mlp::kIn)
      v = (b.feat[row * mlp::kIn + k] - stats[mlp::kOffMean + k]) * stats[mlp::kOffInvStd + k];
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    b.X[int64_t(r) * kXin + k] = h;
    b.Xt[int64_t(k) * b.batch + r] = h;
  }
  b.target[r] = b.label[row];
}

// Tiles of 32 rows x 64 hidden units per 256-thread block: row-major
// reads and writes are coalesced, the transposed copy goes through shared
// memory so that its writes are coalesced too.
constexpr int kTileRows = 32;

// Z1 += b1, H1 = GELU(Z1) in both layouts.
__global__ void __launch_bounds__(256) Act1Kernel(StepBuffers b, const float* blob) {
  __shared__ __nv_bfloat16 tile[kH][kTileRows + 2];
  const int r0 = blockIdx.x * kTileRows;
  for (int e = threadIdx.x; e < kTileRows * kH; e += blockDim.x) {
    const int r = e / kH, o = e % kH;
    const int64_t i = int64_t(r0 + r) * kH + o;
    const float z = b.Z1[i] + blob[mlp::kOffB1 + o];
    b.Z1[i] = z;
    const __nv_bfloat16 h = __float2bfloat16_rn(Gelu(z));
    b.H1[i] = h;
    tile[o][r] = h;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < kTileRows * kH; e += blockDim.x) {
    const int o = e / kTileRows, r = e % kTileRows;
    b.H1t[int64_t(o) * b.batch + r0 + r] = tile[o][r];
  }
}

// Output layer, loss, and the backward pass down to dZ2 (one thread per row;
// dw3, db2, db3 and the loss are reduced over the warp's 32 rows first).
__global__ void OutKernel(StepBuffers b, const float* blob, float* grad) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = r < b.batch;
  const int64_t row = int64_t(active ? r : 0) * kH;
  float y = blob[mlp::kOffB3];
  if (active) {
#pragma unroll 8
    for (int o = 0; o < kH; ++o) {
      const float z = b.Z2[row + o] + blob[mlp::kOffB2 + o];
      b.Z2[row + o] = z;
      y = fmaf(blob[mlp::kOffW3 + o], Gelu(z), y);
    }
  }
  const float e = active ? y - b.target[r] : 0.0f;
  const float dy = 2.0f * e / float(b.batch);
  float e2 = e * e, g3 = dy;
  for (int s = 16; s > 0; s >>= 1) {
    e2 += __shfl_xor_sync(0xffffffffu, e2, s);
    g3 += __shfl_xor_sync(0xffffffffu, g3, s);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(b.loss, e2);
    atomicAdd(grad + mlp::kOffB3, g3);
  }
#pragma unroll 4
  for (int o = 0; o < kH; ++o) {
    float gw = 0.0f, d2 = 0.0f;
    if (active) {
      const float z = b.Z2[row + o];
      gw = dy * Gelu(z);
      d2 = dy * blob[mlp::kOffW3 + o] * GeluGrad(z);
      const __nv_bfloat16 h = __float2bfloat16_rn(d2);
      b.D2[row + o] = h;
      b.D2t[int64_t(o) * b.batch + r] = h;
    }
    for (int s = 16; s > 0; s >>= 1) {
      gw += __shfl_xor_sync(0xffffffffu, gw, s);
      d2 += __shfl_xor_sync(0xffffffffu, d2, s);
    }
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(grad + mlp::kOffW3 + o, gw);
      atomicAdd(grad + mlp::kOffB2 + o, d2);
    }
  }
}

// dZ1 = dH1 * GELU'(Z1) (transposed, bf16) and db1, per 32-row tile.
__global__ void __launch_bounds__(256) Back1Kernel(StepBuffers b, float* grad) {
  __shared__ float tile[kH][kTileRows + 1];
  const int r0 = blockIdx.x * kTileRows;
  for (int e = threadIdx.x; e < kTileRows * kH; e += blockDim.x) {
    const int r = e / kH, o = e % kH;
    const int64_t i = int64_t(r0 + r) * kH + o;
    tile[o][r] = b.dH1[i] * GeluGrad(b.Z1[i]);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < kTileRows * kH; e += blockDim.x) {
    const int o = e / kTileRows, r = e % kTileRows;
    const float d1 = tile[o][r];
    b.D1t[int64_t(o) * b.batch + r0 + r] = __float2bfloat16_rn(d1);
    // the 32 lanes of a warp hold the 32 rows of one hidden unit
    float v = d1;
    for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
    if ((threadIdx.x & 31) == 0) atomicAdd(grad + mlp::kOffB1 + o, v);
  }
}

// Gather the weight gradients from the GEMM outputs into the blob layout.
__global__ void CollectKernel(StepBuffers b, float* grad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kH * mlp::kIn) {
    const int o = i / mlp::kIn, k = i % mlp::kIn;
    grad[mlp::kOffW1 + i] = b.dW1[o * kXin + k];
  }
  if (i < kH * kH) grad[mlp::kOffW2 + i] = b.dW2[i];
}

// Adam (lr, beta1 0.9, beta2 0.999, eps 1e-8) on the weights and biases.
__global__ void AdamKernel(Net net, float lr, unsigned long long* step) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned long long t = *step + 1;
  if (i >= mlp::kOffW1 && i < mlp::kParams) {
    const float g = net.grad[i];
    const float m = 0.9f * net.m1[i] + 0.1f * g;
    const float v = 0.999f * net.m2[i] + 0.001f * g * g;
    net.m1[i] = m;
    net.m2[i] = v;
    const float mh = m / (1.0f - powf(0.9f, float(t)));
    const float vh = v / (1.0f - powf(0.999f, float(t)));
    net.master[i] -= lr * mh / (sqrtf(vh) + 1e-8f);
  }
}

__global__ void StepCountKernel(unsigned long long* step) { *step += 1; }

// Inference rows: standardised features -> X (bf16 [n][16]).
__global__ void InferGatherKernel(int64_t n, const float* feat, const float* stats,
                                  __nv_bfloat16* X) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= n) return;
  for (int k = 0; k < kXin; ++k) {
    float v = 0.0f;
    if (k < mlp::kIn) v = (feat[r * mlp::kIn + k] - stats[mlp::kOffMean + k]) * stats[mlp::kOffInvStd + k];
    X[r * kXin + k] = __float2bfloat16_rn(v);
  }
}

__global__ void InferAct1Kernel(int64_t n, const float* Z1, const float* blob, __nv_bfloat16* H1) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n * kH) return;
  const int o = static_cast<int>(i % kH);
  H1[i] = __float2bfloat16_rn(Gelu(Z1[i] + blob[mlp::kOffB1 + o]));
}

__global__ void InferOutKernel(int64_t n, const float* Z2, const float* blob, float* y) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= n) return;
  float acc = blob[mlp::kOffB3];
  for (int o = 0; o < kH; ++o) acc = fmaf(blob[mlp::kOffW3 + o], Gelu(Z2[r * kH + o] + blob[mlp::kOffB2 + o]), acc);
  y[r] = acc;
}

}  // namespace mlpk
}  // namespace fvs

// ---------------------------------------------------------------------------
// C ABI

using namespace fvs::mlpk;

struct fvs_mlp {
  Net net{};
  float* buf = nullptr;  // master, m1, m2, grad, blob
  __nv_bfloat16* wbuf = nullptr;
  int* error = nullptr;
  unsigned long long* step = nullptr;
  cudaStream_t stream = nullptr;
  // training scratch (sized for `batch`)
  int batch = 0;
  std::vector<void*> scratch;
  StepBuffers sb{};
  cudaGraphExec_t graph = nullptr;
  const float* graph_feat = nullptr;
  const float* graph_label = nullptr;
  int64_t graph_n = 0;
  float graph_lr = 0.f;
  uint64_t graph_seed = 0;
  // inference scratch
  int64_t infer_cap = 0;
  void* infer_buf = nullptr;
  ~fvs_mlp() {
    if (graph) cudaGraphExecDestroy(graph);
    for (void* p : scratch) cudaFree(p);
    if (infer_buf) cudaFree(infer_buf);
    if (buf) cudaFree(buf);
    if (wbuf) cudaFree(wbuf);
    if (error) cudaFree(error);
    if (step) cudaFree(step);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

int MlpFail(int code, const std::string& msg) {
  fvs::SetLastError(msg);
  return code;
}

int MlpCuda(cudaError_t e, const char* what) {
  fvs::SetLastError(std::string(what) + ": " + cudaGetErrorString(e));
  return FVS_ERR_CUDA;
}

#define MLP_CUDA(call)                                  \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return MlpCuda(e_, #call);   \
  } while (0)

cudaError_t Alloc(fvs_mlp* m, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e == cudaSuccess) {
    m->scratch.push_back(*p);
    e = cudaMemset(*p, 0, bytes);
  }
  return e;
}

int EnsureBatch(fvs_mlp* m, int batch) {
  if (m->batch == batch) return FVS_OK;
  if (m->graph) {
    cudaGraphExecDestroy(m->graph);
    m->graph = nullptr;
  }
  for (void* p : m->scratch) cudaFree(p);
  m->scratch.clear();
  StepBuffers& b = m->sb;
  b = StepBuffers{};
  b.batch = batch;
  const size_t B = size_t(batch);
  MLP_CUDA(Alloc(m, (void**)&b.X, B * kXin * 2));
  MLP_CUDA(Alloc(m, (void**)&b.Xt, B * kXin * 2));
  MLP_CUDA(Alloc(m, (void**)&b.target, B * 4));
  MLP_CUDA(Alloc(m, (void**)&b.Z1, B * kH * 4));
  MLP_CUDA(Alloc(m, (void**)&b.H1, B * kH * 2));
  MLP_CUDA(Alloc(m, (void**)&b.H1t, B * kH * 2));
  MLP_CUDA(Alloc(m, (void**)&b.Z2, B * kH * 4));
  MLP_CUDA(Alloc(m, (void**)&b.D2, B * kH * 2));
  MLP_CUDA(Alloc(m, (void**)&b.D2t, B * kH * 2));
  MLP_CUDA(Alloc(m, (void**)&b.dH1, B * kH * 4));
  MLP_CUDA(Alloc(m, (void**)&b.D1t, B * kH * 2));
  MLP_CUDA(Alloc(m, (void**)&b.dW2, 128 * kH * 4));
  MLP_CUDA(Alloc(m, (void**)&b.dW1, 128 * kXin * 4));
  MLP_CUDA(Alloc(m, (void**)&b.loss, 4));
  b.step = m->step;
  m->batch = batch;
  return FVS_OK;
}

// One training step (forward, backward, and optionally Adam) on the stream.
cudaError_t EnqueueStep(fvs_mlp* m, bool update, float lr) {
  StepBuffers& b = m->sb;
  cudaStream_t s = m->stream;
  const Net& net = m->net;
  const int B = b.batch;
  cudaError_t e = cudaMemsetAsync(net.grad, 0, sizeof(float) * fvs::mlp::kParams, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b.dW2, 0, 128 * kH * 4, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b.dW1, 0, 128 * kXin * 4, s);
  if (e != cudaSuccess) return e;
  GatherKernel<<<(B + 127) / 128, 128, 0, s>>>(b, net.blob);
  GemmArgs g{};
  g.error = m->error;
  // Z1 = X W1^T
  g.A = b.X; g.lda = kXin; g.B = net.W1; g.ldb = kXin; g.C = b.Z1; g.ldc = kH;
  g.M = B; g.K = kXin; g.k_per_cta = kXin; g.atomic = 0;
  if ((e = LaunchGemm<64>(g, 1, s)) != cudaSuccess) return e;
  Act1Kernel<<<B / kTileRows, 256, 0, s>>>(b, net.blob);
  // Z2 = H1 W2^T
  g.A = b.H1; g.lda = kH; g.B = net.W2; g.ldb = kH; g.C = b.Z2; g.ldc = kH;
  g.M = B; g.K = kH; g.k_per_cta = kH; g.atomic = 0;
  if ((e = LaunchGemm<64>(g, 1, s)) != cudaSuccess) return e;
  OutKernel<<<(B + 127) / 128, 128, 0, s>>>(b, net.blob, net.grad);
  // dH1 = dZ2 W2  (B operand W2^T: [in][out])
  g.A = b.D2; g.lda = kH; g.B = net.W2t; g.ldb = kH; g.C = b.dH1; g.ldc = kH;
  g.M = B; g.K = kH; g.k_per_cta = kH; g.atomic = 0;
  if ((e = LaunchGemm<64>(g, 1, s)) != cudaSuccess) return e;
  // dW2 = dZ2^T H1 over the batch (split K)
  const int kper = 256;
  g.A = b.D2t; g.lda = B; g.B = b.H1t; g.ldb = B; g.C = b.dW2; g.ldc = kH;
  g.M = kH; g.K = B; g.k_per_cta = kper; g.atomic = 1;
  if ((e = LaunchGemm<64>(g, (B + kper - 1) / kper, s)) != cudaSuccess) return e;
  Back1Kernel<<<B / kTileRows, 256, 0, s>>>(b, net.grad);
  // dW1 = dZ1^T X
  g.A = b.D1t; g.lda = B; g.B = b.Xt; g.ldb = B; g.C = b.dW1; g.ldc = kXin;
  g.M = kH; g.K = B; g.k_per_cta = kper; g.atomic = 1;
  if ((e = LaunchGemm<16>(g, (B + kper - 1) / kper, s)) != cudaSuccess) return e;
  CollectKernel<<<(kH * kH + 255) / 256, 256, 0, s>>>(b, net.grad);
  if (update) {
    AdamKernel<<<(fvs::mlp::kParams + 255) / 256, 256, 0, s>>>(net, lr, b.step);
    PublishKernel<<<(fvs::mlp::kParams + 255) / 256, 256, 0, s>>>(net);
    StepCountKernel<<<1, 1, 0, s>>>(b.step);
  }
  return cudaGetLastError();
}

uint64_t HostMix(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

}  // namespace

extern "C" {

int fvs_mlp_param_count(void) { return fvs::mlp::kParams; }

int fvs_tc_gemm_bf16(const void* A_dev, int lda, const void* B_dev, int ldb, float* C_dev, int ldc,
                     int M, int N, int K, int splits, int accumulate, void* stream) {
  if (!A_dev || !B_dev || !C_dev || M < 1 || K < 16 || K % 16 != 0 || splits < 1)
    return MlpFail(FVS_ERR_INVALID, "need M >= 1, K a positive multiple of 16, splits >= 1");
  if (N != 16 && N != 32 && N != 64)
    return MlpFail(FVS_ERR_UNSUPPORTED, "N must be 16, 32 or 64");
  if (lda < K || ldb < K || ldc < N || lda % 8 != 0 || ldb % 8 != 0 ||
      (reinterpret_cast<uintptr_t>(A_dev) & 15) != 0 || (reinterpret_cast<uintptr_t>(B_dev) & 15) != 0)
    return MlpFail(FVS_ERR_INVALID, "operands must be 16-byte aligned with lda, ldb >= K (multiples of 8)");
  if (splits > 1 && !accumulate)
    return MlpFail(FVS_ERR_INVALID, "split K needs accumulate = 1");
  const int per = (K / splits + 15) / 16 * 16;
  const int used = (K + per - 1) / per;
  static int* err = nullptr;
  if (!err) {
    MLP_CUDA(cudaMalloc(&err, sizeof(int)));
    MLP_CUDA(cudaMemset(err, 0, sizeof(int)));
  }
  GemmArgs g{};
  g.A = static_cast<const __nv_bfloat16*>(A_dev);
  g.lda = lda;
  g.B = static_cast<const __nv_bfloat16*>(B_dev);
  g.ldb = ldb;
  g.C = C_dev;
  g.ldc = ldc;
  g.M = M;
  g.K = K;
  g.k_per_cta = per;
  g.atomic = accumulate;
  g.error = err;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = N == 16 ? LaunchGemm<16>(g, used, s)
                : N == 32 ? LaunchGemm<32>(g, used, s)
                          : LaunchGemm<64>(g, used, s);
  MLP_CUDA(e);
  int h = 0;
  MLP_CUDA(cudaMemcpyAsync(&h, err, sizeof h, cudaMemcpyDeviceToHost, s));
  MLP_CUDA(cudaStreamSynchronize(s));
  if (h) return MlpFail(FVS_ERR_CUDA, "tensor-core wait timed out");
  return FVS_OK;
}

int fvs_mlp_create(uint64_t seed, fvs_mlp** out) {
  if (!out) return MlpFail(FVS_ERR_INVALID, "NULL argument");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return MlpFail(FVS_ERR_NO_DEVICE, "no CUDA device available");
  }
  fvs_mlp* m = new fvs_mlp();
  const int P = fvs::mlp::kParams;
  cudaError_t e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&m->buf, sizeof(float) * P * 5);
  if (e == cudaSuccess) e = cudaMalloc(&m->wbuf, sizeof(__nv_bfloat16) * (64 * 16 + 2 * 64 * 64));
  if (e == cudaSuccess) e = cudaMalloc(&m->error, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&m->step, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(m->buf, 0, sizeof(float) * P * 5);
  if (e == cudaSuccess) e = cudaMemset(m->wbuf, 0, sizeof(__nv_bfloat16) * (64 * 16 + 2 * 64 * 64));
  if (e == cudaSuccess) e = cudaMemset(m->error, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(m->step, 0, sizeof(unsigned long long));
  if (e != cudaSuccess) {
    delete m;
    return MlpCuda(e, "fvs_mlp_create");
  }
  m->net.master = m->buf;
  m->net.m1 = m->buf + P;
  m->net.m2 = m->buf + 2 * P;
  m->net.grad = m->buf + 3 * P;
  m->net.blob = m->buf + 4 * P;
  m->net.W1 = m->wbuf;
  m->net.W2 = m->wbuf + 64 * 16;
  m->net.W2t = m->wbuf + 64 * 16 + 64 * 64;
  // He-style uniform initialisation on the host (deterministic from seed)
  std::vector<float> h(P, 0.0f);
  for (int k = 0; k < fvs::mlp::kIn; ++k) h[fvs::mlp::kOffInvStd + k] = 1.0f;
  uint64_t st = seed;
  auto uni = [&]() {
    st = HostMix(st);
    return float((st >> 11) * (1.0 / 9007199254740992.0)) * 2.0f - 1.0f;
  };
  const float s1 = std::sqrt(6.0f / fvs::mlp::kIn), s2 = std::sqrt(6.0f / kH);
  for (int i = 0; i < kH * fvs::mlp::kIn; ++i) h[fvs::mlp::kOffW1 + i] = s1 * uni();
  for (int i = 0; i < kH * kH; ++i) h[fvs::mlp::kOffW2 + i] = s2 * uni();
  for (int i = 0; i < kH; ++i) h[fvs::mlp::kOffW3 + i] = 0.5f * s2 * uni();
  e = cudaMemcpy(m->net.master, h.data(), sizeof(float) * P, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    delete m;
    return MlpCuda(e, "fvs_mlp_create upload");
  }
  PublishKernel<<<(P + 255) / 256, 256, 0, m->stream>>>(m->net);
  e = cudaStreamSynchronize(m->stream);
  if (e != cudaSuccess) {
    delete m;
    return MlpCuda(e, "fvs_mlp_create publish");
  }
  *out = m;
  return FVS_OK;
}

int fvs_mlp_destroy(fvs_mlp* m) {
  if (m) {
    cudaStreamSynchronize(m->stream);
    delete m;
  }
  return FVS_OK;
}

int fvs_riemann_features(int64_t n, double gamma, const double* rhoL_dev, const double* uL_dev,
                         const double* pL_dev, const double* rhoR_dev, const double* uR_dev,
                         const double* pR_dev, const double* pstar_dev, float* features_dev,
                         float* labels_dev, void* stream) {
  if (n < 0 || !features_dev) return MlpFail(FVS_ERR_INVALID, "bad arguments");
  if (n == 0) return FVS_OK;
  FeaturesKernel<<<unsigned((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      n, rhoL_dev, uL_dev, pL_dev, rhoR_dev, uR_dev, pR_dev, pstar_dev, gamma, features_dev,
      labels_dev);
  MLP_CUDA(cudaGetLastError());
  return FVS_OK;
}

int fvs_mlp_set_normalization(fvs_mlp* m, const float* features_dev, int64_t n) {
  if (!m || !features_dev || n < 2) return MlpFail(FVS_ERR_INVALID, "bad arguments");
  double* acc = nullptr;
  MLP_CUDA(cudaMallocAsync(&acc, sizeof(double) * 2 * fvs::mlp::kIn, m->stream));
  MLP_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * 2 * fvs::mlp::kIn, m->stream));
  MomentsKernel<<<152 * 4, 256, 0, m->stream>>>(n, features_dev, acc);
  double h[2 * fvs::mlp::kIn];
  MLP_CUDA(cudaMemcpyAsync(h, acc, sizeof h, cudaMemcpyDeviceToHost, m->stream));
  MLP_CUDA(cudaFreeAsync(acc, m->stream));
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  float st[2 * fvs::mlp::kIn];
  for (int k = 0; k < fvs::mlp::kIn; ++k) {
    const double mean = h[k] / double(n);
    const double var = h[fvs::mlp::kIn + k] / double(n) - mean * mean;
    st[k] = float(mean);
    st[fvs::mlp::kIn + k] = float(1.0 / std::sqrt(var > 1e-12 ? var : 1e-12));
  }
  MLP_CUDA(cudaMemcpyAsync(m->net.master + fvs::mlp::kOffMean, st, sizeof st,
                           cudaMemcpyHostToDevice, m->stream));
  PublishKernel<<<(fvs::mlp::kParams + 255) / 256, 256, 0, m->stream>>>(m->net);
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  return FVS_OK;
}

int fvs_mlp_train(fvs_mlp* m, const float* features_dev, const float* labels_dev, int64_t n,
                  int steps, int batch, float lr, uint64_t seed, float* mean_loss) {
  if (!m || !features_dev || !labels_dev || n < 1 || steps < 0)
    return MlpFail(FVS_ERR_INVALID, "bad arguments");
  if (batch < 128 || batch % 256 != 0 || batch > (1 << 20))
    return MlpFail(FVS_ERR_INVALID, "batch must be a multiple of 256 in [256, 2^20]");
  if (int r = EnsureBatch(m, batch)) return r;
  StepBuffers& b = m->sb;
  b.feat = features_dev;
  b.label = labels_dev;
  b.n = n;
  b.seed = seed;
  b.use_given_rows = 0;
  if (!m->graph || m->graph_feat != features_dev || m->graph_label != labels_dev ||
      m->graph_n != n || m->graph_lr != lr || m->graph_seed != seed) {
    if (m->graph) cudaGraphExecDestroy(m->graph);
    m->graph = nullptr;
    cudaGraph_t g;
    MLP_CUDA(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = EnqueueStep(m, true, lr);
    cudaError_t e2 = cudaStreamEndCapture(m->stream, &g);
    if (e != cudaSuccess) return MlpCuda(e, "capture training step");
    if (e2 != cudaSuccess) return MlpCuda(e2, "end capture");
    e = cudaGraphInstantiate(&m->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return MlpCuda(e, "instantiate training graph");
    m->graph_feat = features_dev;
    m->graph_label = labels_dev;
    m->graph_n = n;
    m->graph_lr = lr;
    m->graph_seed = seed;
  }
  MLP_CUDA(cudaMemsetAsync(b.loss, 0, sizeof(float), m->stream));
  for (int i = 0; i < steps; ++i) MLP_CUDA(cudaGraphLaunch(m->graph, m->stream));
  float loss = 0.f;
  int err = 0;
  MLP_CUDA(cudaMemcpyAsync(&loss, b.loss, sizeof loss, cudaMemcpyDeviceToHost, m->stream));
  MLP_CUDA(cudaMemcpyAsync(&err, m->error, sizeof err, cudaMemcpyDeviceToHost, m->stream));
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  if (err) return MlpFail(FVS_ERR_CUDA, "tensor-core wait timed out");
  if (mean_loss) *mean_loss = steps > 0 ? loss / float(int64_t(steps) * batch) : 0.f;
  return FVS_OK;
}

int fvs_mlp_gradients(fvs_mlp* m, const float* features_dev, const float* labels_dev, int batch,
                      float* grads_host, float* loss_host) {
  if (!m || !features_dev || !labels_dev || !grads_host)
    return MlpFail(FVS_ERR_INVALID, "bad arguments");
  if (batch < 128 || batch % 256 != 0) return MlpFail(FVS_ERR_INVALID, "batch multiple of 256");
  if (int r = EnsureBatch(m, batch)) return r;
  StepBuffers& b = m->sb;
  b.feat = features_dev;
  b.label = labels_dev;
  b.n = batch;
  b.use_given_rows = 1;
  MLP_CUDA(cudaMemsetAsync(b.loss, 0, sizeof(float), m->stream));
  MLP_CUDA(EnqueueStep(m, false, 0.f));
  int err = 0;
  MLP_CUDA(cudaMemcpyAsync(grads_host, m->net.grad, sizeof(float) * fvs::mlp::kParams,
                           cudaMemcpyDeviceToHost, m->stream));
  float loss = 0.f;
  MLP_CUDA(cudaMemcpyAsync(&loss, b.loss, sizeof loss, cudaMemcpyDeviceToHost, m->stream));
  MLP_CUDA(cudaMemcpyAsync(&err, m->error, sizeof err, cudaMemcpyDeviceToHost, m->stream));
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  if (err) return MlpFail(FVS_ERR_CUDA, "tensor-core wait timed out");
  if (loss_host) *loss_host = loss / float(batch);
  return FVS_OK;
}

int fvs_mlp_predict(fvs_mlp* m, const float* features_dev, int64_t n, float* y_dev) {
  if (!m || !features_dev || !y_dev || n < 0) return MlpFail(FVS_ERR_INVALID, "bad arguments");
  if (n == 0) return FVS_OK;
  const int64_t npad = (n + 127) / 128 * 128;
  if (npad > m->infer_cap) {
    if (m->infer_buf) cudaFree(m->infer_buf);
    m->infer_buf = nullptr;
    const size_t bytes = size_t(npad) * (kXin * 2 + kH * 4 * 2 + kH * 2);
    MLP_CUDA(cudaMalloc(&m->infer_buf, bytes));
    MLP_CUDA(cudaMemset(m->infer_buf, 0, bytes));
    m->infer_cap = npad;
  }
  uint8_t* p = static_cast<uint8_t*>(m->infer_buf);
  __nv_bfloat16* X = reinterpret_cast<__nv_bfloat16*>(p);
  float* Z1 = reinterpret_cast<float*>(p + size_t(m->infer_cap) * kXin * 2);
  float* Z2 = Z1 + size_t(m->infer_cap) * kH;
  __nv_bfloat16* H1 = reinterpret_cast<__nv_bfloat16*>(Z2 + size_t(m->infer_cap) * kH);
  cudaStream_t s = m->stream;
  InferGatherKernel<<<unsigned((n + 255) / 256), 256, 0, s>>>(n, features_dev, m->net.blob, X);
  GemmArgs g{};
  g.error = m->error;
  g.A = X; g.lda = kXin; g.B = m->net.W1; g.ldb = kXin; g.C = Z1; g.ldc = kH;
  g.M = int(n); g.K = kXin; g.k_per_cta = kXin; g.atomic = 0;
  MLP_CUDA(LaunchGemm<64>(g, 1, s));
  InferAct1Kernel<<<unsigned((n * kH + 255) / 256), 256, 0, s>>>(n, Z1, m->net.blob, H1);
  g.A = H1; g.lda = kH; g.B = m->net.W2; g.ldb = kH; g.C = Z2; g.ldc = kH;
  g.M = int(n); g.K = kH; g.k_per_cta = kH; g.atomic = 0;
  MLP_CUDA(LaunchGemm<64>(g, 1, s));
  InferOutKernel<<<unsigned((n + 255) / 256), 256, 0, s>>>(n, Z2, m->net.blob, y_dev);
  int err = 0;
  MLP_CUDA(cudaMemcpyAsync(&err, m->error, sizeof err, cudaMemcpyDeviceToHost, s));
  MLP_CUDA(cudaStreamSynchronize(s));
  if (err) return MlpFail(FVS_ERR_CUDA, "tensor-core wait timed out");
  return FVS_OK;
}

int fvs_mlp_params(fvs_mlp* m, const float** params_dev) {
  if (!m || !params_dev) return MlpFail(FVS_ERR_INVALID, "NULL argument");
  *params_dev = m->net.blob;
  return FVS_OK;
}

int fvs_mlp_get_master(fvs_mlp* m, float* host) {
  if (!m || !host) return MlpFail(FVS_ERR_INVALID, "NULL argument");
  MLP_CUDA(cudaMemcpy(host, m->net.master, sizeof(float) * fvs::mlp::kParams,
                      cudaMemcpyDeviceToHost));
  return FVS_OK;
}

int fvs_mlp_set_master(fvs_mlp* m, const float* host) {
  if (!m || !host) return MlpFail(FVS_ERR_INVALID, "NULL argument");
  MLP_CUDA(cudaMemcpy(m->net.master, host, sizeof(float) * fvs::mlp::kParams,
                      cudaMemcpyHostToDevice));
  PublishKernel<<<(fvs::mlp::kParams + 255) / 256, 256, 0, m->stream>>>(m->net);
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  return FVS_OK;
}

}  // extern "C"
