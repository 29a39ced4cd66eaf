// fvs_stable.cuh -- stable-dt pass of a uniform grid over all directions,
// generic over a physics policy (fast FP64 and mixed flavours).
//
// DimensionalSplitLevelIntegrator::ComputeStableDt takes the minimum over
// directions of FluxMethodAdapter::ComputeStableDt
// (include/fub/solver/DimensionalSplitLevelIntegrator.hpp:204-219); each face
// contributes dx / max(0, |sL|, |sR|) with Einfeldt speeds
// (include/fub/flux_method/HllMethod.hpp:337-347).  The kernel writes the max
// face speed per direction; dt = dx / speed is formed once on the host/device.
#pragma once

#include "fvs_internal.h"
#include "fvs_sweep.cuh"

namespace fvs {

// Whether face f (between cells f-1 and f, 0 <= f <= n) of a direction of n
// cells enters the reference's dt: MFIter tiles of 8 cells grown by 2 ghost
// layers at the box boundary, windows of 2w cells inside each tile, the
// window's middle pair is the face (FluxMethodAdapter.hpp:85-96,
// FluxMethod.hpp:341-382).
__device__ __forceinline__ bool ReferenceTileFaceT(int f, int n, int w) {
  const int G = 2;
  for (int T = (f / 8) - 1; T <= f / 8; ++T) {
    if (T < 0) continue;
    const int t0 = T * 8;
    if (t0 >= n) continue;
    const int t1 = min(n, t0 + 8);
    const int a = (t0 == 0) ? -G : t0;
    const int b = (t1 == n) ? n + G : t1;
    if (f >= a + w && f < b - w + 1) return true;
  }
  return false;
}

template <int D, template <int> class PT>
__global__ void __launch_bounds__(256) StableDtKernelT(StableDtArgs a) {
  using P = PT<D>;
  using R = typename P::Real;
  constexpr int K = D + 2;
  const int nx = a.n[0], ny = a.n[1], nz = a.n[2];
  const int64_t cs = int64_t(nx) * ny * nz;
  const int64_t cell = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (a.ctrl && (a.ctrl->abort || a.ctrl->done)) return;
  const typename P::Gas eq = P::MakeGas(a.gamma);
  double smax[3] = {0.0, 0.0, 0.0};
  if (cell < cs) {
    const int i = static_cast<int>(cell % nx);
    const int j = static_cast<int>((cell / nx) % ny);
    const int k = static_cast<int>(cell / (int64_t(nx) * ny));
    const int idx[3] = {i, j, k};
    double ud[K];
    R u[K];
#pragma unroll
    for (int c = 0; c < K; ++c) ud[c] = __ldg(a.in + c * cs + cell);
    P::ToCell(u, ud);
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const typename P::Wave w = P::MakeWave(eq, u, d);
      const int nd = a.n[d];
      const int faces = (idx[d] == nd - 1) ? 2 : 1;
      for (int fi = 0; fi < faces; ++fi) {
        const int f = idx[d] + fi;
        if (a.rule == 1 && d > 0 && !ReferenceTileFaceT(f, nd, a.width)) continue;
        if (fi == 1 && a.bc[d] == 0) continue;  // periodic: face n == face 0
        const int other = BcIndex(fi == 0 ? f - 1 : f, nd, a.bc[d]);
        int oidx[3] = {i, j, k};
        oidx[d] = other;
        const int64_t ocell = (int64_t(oidx[2]) * ny + oidx[1]) * int64_t(nx) + oidx[0];
        double vd[K];
        R v[K];
#pragma unroll
        for (int c = 0; c < K; ++c) vd[c] = __ldg(a.in + c * cs + ocell);
        P::ToCell(v, vd);
        const typename P::Wave wo = P::MakeWave(eq, v, d);
        const double s = static_cast<double>((fi == 0) ? P::FaceMaxSpeed(eq, wo, w)
                                                       : P::FaceMaxSpeed(eq, w, wo));
        smax[d] = s > smax[d] ? s : smax[d];
      }
    }
  }
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const double m = WarpMax(smax[d]);
    if ((threadIdx.x & 31) == 0 && m > 0.0) AtomicMaxPositive(a.smax_out + d, m);
  }
}

template <template <int> class PT>
cudaError_t LaunchStableDtT(const StableDtArgs& a, cudaStream_t s) {
  const int64_t cells = int64_t(a.n[0]) * a.n[1] * a.n[2];
  const int block = 256;
  const unsigned grid = static_cast<unsigned>((cells + block - 1) / block);
  switch (a.rank) {
  case 1:
    StableDtKernelT<1, PT><<<grid, block, 0, s>>>(a);
    break;
  case 2:
    StableDtKernelT<2, PT><<<grid, block, 0, s>>>(a);
    break;
  default:
    StableDtKernelT<3, PT><<<grid, block, 0, s>>>(a);
    break;
  }
  return cudaGetLastError();
}

}  // namespace fvs
