// fvs_noalloc.cu -- fvs_compute_stable_dt_noalloc: the patch stable-dt
// reduction without any device allocation.
//
// Some callers cannot let a library allocate device memory: an integrator
// that hands out every byte of device memory through its own arena (the way
// AMReX's arenas own a device-resident MultiFab hierarchy), or an application
// running close to the memory limit.  For them cudaMalloc/cudaFree behind
// their back is a problem: the calls synchronise the whole device, they sit
// outside the arena's budget, and they can fail at run time when the arena
// already holds the memory.  fvs_compute_stable_dt allocates one reduction
// word per call; this variant instead reduces through a fixed array that is
// part of the library image, so it allocates nothing.
//
// Compiled with -fmad=false like the other exact-FP64 kernels: the Einfeldt
// speeds, and therefore the returned dt, are bit-identical to
// fvs_compute_stable_dt's.
#include "../../include/fvs_gpu.h"
#include "fvs_internal.h"
#include "fvs_physics_exact.cuh"

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

namespace {

// Scratch of the two-pass reduction: one partial maximum per block of the
// first pass, and one slot for the final maximum: (8192 + 1) x 8 = 65,544
// bytes.  Every GPU that loads this library holds it until the process exits.
constexpr int kThreads = 256;
constexpr int kMaxBlocks = 8192;
constexpr int64_t kMaxWindows = int64_t(kMaxBlocks) * kThreads;  // 2,097,152
static __device__ __align__(256) double g_noalloc_scratch[kMaxBlocks + 1];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
double* g_scratch_ptr[kMaxDevices] = {};

struct View {
  const double* p;
  fvs::BoxDesc b;
  __device__ __forceinline__ double operator()(int c, int i, int j, int k) const {
    return p[((int64_t(c) * b.n[2] + (k - b.lo[2])) * b.n[1] + (j - b.lo[1])) *
                 int64_t(b.n[0]) +
             (i - b.lo[0])];
  }
};

template <int D>
__device__ __forceinline__ fvs::exact::Complete<D> Load(const View& v, int i, int j,
                                                        int k) {
  fvs::exact::Complete<D> q;
  q.rho = v(0, i, j, k);
#pragma unroll
  for (int d = 0; d < D; ++d) q.m[d] = v(1 + d, i, j, k);
  q.E = v(1 + D, i, j, k);
  q.p = v(2 + D, i, j, k);
  q.c = v(3 + D, i, j, k);
  return q;
}

// Block max of non-negative speeds; a NaN speed counts as 0 (skipped), the
// rule of the allocating entry point's reduction.
__device__ __forceinline__ double BlockMax(double s) {
  __shared__ double warp_max[kThreads / 32];
  s = s > 0.0 ? s : 0.0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double w = __shfl_xor_sync(0xffffffffu, s, o);
    s = w > s ? w : s;
  }
  if ((threadIdx.x & 31) == 0) warp_max[threadIdx.x >> 5] = s;
  __syncthreads();
  double m = 0.0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < kThreads / 32; ++w) m = warp_max[w] > m ? warp_max[w] : m;
  }
  return m;
}

// Pass 1: max face speed max(0, |sL|, |sR|) of the windows of one block
// (the window rule of FluxMethod::ComputeStableDt, FluxMethod.hpp:295-382),
// written to scratch[blockIdx.x].
template <int D>
__global__ void __launch_bounds__(kThreads)
    NoAllocPartialKernel(int w, double gamma, View st, fvs::BoxDesc wbox, int dir,
                         double* scratch) {
  const int64_t nwin = int64_t(wbox.n[0]) * wbox.n[1] * wbox.n[2];
  const int64_t id = int64_t(blockIdx.x) * kThreads + threadIdx.x;
  double s = 0.0;
  if (id < nwin) {
    int c[3];
    c[0] = wbox.lo[0] + static_cast<int>(id % wbox.n[0]);
    c[1] = wbox.lo[1] + static_cast<int>((id / wbox.n[0]) % wbox.n[1]);
    c[2] = wbox.lo[2] + static_cast<int>(id / (int64_t(wbox.n[0]) * wbox.n[1]));
    c[dir] += w - 1;
    const fvs::exact::Complete<D> L = Load<D>(st, c[0], c[1], c[2]);
    c[dir] += 1;
    const fvs::exact::Complete<D> R = Load<D>(st, c[0], c[1], c[2]);
    fvs::exact::Gas eq;
    eq.gamma = gamma;
    eq.gamma_minus_1_inv = 1.0 / (gamma - 1.0);
    double s0, s1;
    fvs::exact::Einfeldt<D>(eq, L, R, dir, s0, s1);
    s = fvs::exact::PMax(fvs::exact::PMax(0.0, fabs(s0)), fabs(s1));
  }
  const double m = BlockMax(s);
  if (threadIdx.x == 0) scratch[blockIdx.x] = m;
}

// Pass 2: max over the nblocks partial maxima -> scratch[kMaxBlocks].
__global__ void __launch_bounds__(kThreads) NoAllocFinalKernel(double* scratch, int nblocks) {
  double s = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += kThreads) {
    const double v = scratch[b];
    s = v > s ? v : s;
  }
  const double m = BlockMax(s);
  if (threadIdx.x == 0) scratch[kMaxBlocks] = m;
}

int Fail(int code, const std::string& msg) {
  fvs::SetLastError(msg);  // reported by fvs_last_error()
  return code;
}

// Resolves the device address of g_noalloc_scratch for the current device,
// once per device (cudaGetSymbolAddress with that device current).
int ScratchForCurrentDevice(double** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return Fail(FVS_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return Fail(FVS_ERR_UNSUPPORTED, "device ordinal beyond the supported 64 devices");
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return Fail(FVS_ERR_CUDA,
                  std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[dev];
  return FVS_OK;
}

}  // namespace

extern "C" int fvs_compute_stable_dt_noalloc(const fvs_method* m, int rank,
                                             const double* states_dev, fvs_box cell_box,
                                             double dx, int dir, int window_rule,
                                             double* dt_out, void* stream) {
  // the allocating entry point's checks, in its order, so that both return
  // the same status for the same arguments
  if (int r = fvs::CheckMethod(m, rank)) return r;
  if (dir < 0 || dir >= rank) return Fail(FVS_ERR_INVALID, "direction out of range");
  fvs::BoxDesc cb;
  for (int d = 0; d < 3; ++d) {
    if (cell_box.hi[d] < cell_box.lo[d]) return Fail(FVS_ERR_INVALID, "invalid box");
    cb.lo[d] = cell_box.lo[d];
    cb.n[d] = cell_box.hi[d] - cell_box.lo[d];
  }
  if (!dt_out) return Fail(FVS_ERR_INVALID, "dt_out is NULL");
  if (window_rule != 0 && window_rule != 1)
    return Fail(FVS_ERR_INVALID, "window_rule must be 0 or 1");
  if (int r = fvs::CheckDevice()) return r;
  if (m->flux_method != FVS_MUSCL_HLLE && m->flux_method != FVS_HLLE)
    return Fail(FVS_ERR_UNSUPPORTED, "the allocation-free stable dt covers the HLLE methods "
                                     "(FVS_MUSCL_HLLE, FVS_HLLE)");
  const int w = (m->flux_method == FVS_HLLE) ? 1 : 2;
  fvs::BoxDesc wbox = cb;
  wbox.n[dir] -= (window_rule == 0) ? 2 * w : 2 * w - 1;
  const int64_t nwin =
      wbox.n[dir] <= 0 ? 0 : int64_t(wbox.n[0]) * wbox.n[1] * wbox.n[2];
  if (nwin > kMaxWindows)
    return Fail(FVS_ERR_INVALID,
                "fvs_compute_stable_dt_noalloc: " + std::to_string(nwin) +
                    " stencil windows exceed the maximum of " +
                    std::to_string(kMaxWindows) +
                    " (8192 blocks x 256 threads of static scratch); split the patch "
                    "or call fvs_compute_stable_dt");
  if (nwin == 0) {
    *dt_out = INFINITY;
    return FVS_OK;
  }
  if (!states_dev) return Fail(FVS_ERR_INVALID, "NULL data pointer");
  double* scratch = nullptr;
  if (int r = ScratchForCurrentDevice(&scratch)) return r;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nblocks = static_cast<int>((nwin + kThreads - 1) / kThreads);
  const View sv{states_dev, cb};
  switch (rank) {
  case 1:
    NoAllocPartialKernel<1><<<nblocks, kThreads, 0, st>>>(w, m->gamma, sv, wbox, dir, scratch);
    break;
  case 2:
    NoAllocPartialKernel<2><<<nblocks, kThreads, 0, st>>>(w, m->gamma, sv, wbox, dir, scratch);
    break;
  default:
    NoAllocPartialKernel<3><<<nblocks, kThreads, 0, st>>>(w, m->gamma, sv, wbox, dir, scratch);
    break;
  }
  NoAllocFinalKernel<<<1, kThreads, 0, st>>>(scratch, nblocks);
  cudaError_t e = cudaGetLastError();
  double smax = 0.0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&smax, scratch + kMaxBlocks, sizeof smax, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess)
    return Fail(FVS_ERR_CUDA,
                std::string("fvs_compute_stable_dt_noalloc: ") + cudaGetErrorString(e));
  *dt_out = (smax > 0.0) ? dx / smax : INFINITY;
  return FVS_OK;
}
