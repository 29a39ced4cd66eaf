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

#include <algorithm>
#include <type_traits>

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
  if (!BlockAll(!(a.ctrl && (a.ctrl->abort || a.ctrl->done)))) return;
  const typename P::Gas eq = P::MakeGas(a.gamma);
  R smr[3] = {R(0), R(0), R(0)};  // in the policy's precision (no FP64 work per face)
  // grid-stride over cells; one atomic per block and direction at the end
  for (int64_t cell = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; cell < cs;
       cell += int64_t(gridDim.x) * blockDim.x) {
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
        const int og = fi == 0 ? f - 1 : f;
        const int other = BcIndex(og, nd, a.bc[d]);
        int oidx[3] = {i, j, k};
        oidx[d] = other;
        const int64_t ocell = (int64_t(oidx[2]) * ny + oidx[1]) * int64_t(nx) + oidx[0];
        double vd[K];
        R v[K];
#pragma unroll
        for (int c = 0; c < K; ++c) vd[c] = __ldg(a.in + c * cs + ocell);
        if (BcFlip(og, nd, a.bc[d])) vd[1 + d] = -vd[1 + d];
        P::ToCell(v, vd);
        const typename P::Wave wo = P::MakeWave(eq, v, d);
        const R s = (fi == 0) ? P::FaceMaxSpeed(eq, wo, w) : P::FaceMaxSpeed(eq, w, wo);
        smr[d] = s > smr[d] ? s : smr[d];
      }
    }
  }
  double smax[D];
#pragma unroll
  for (int d = 0; d < D; ++d) smax[d] = static_cast<double>(smr[d]);
  BlockMaxAtomic<D>(a.smax_out, smax);
}

// The waves of one cell in the three directions: a policy with a shared
// preparation (MakeWaves) computes the direction-free part once, any other
// policy calls MakeWave per direction.
template <class P, class = void> struct WavesOf {
  static __device__ __forceinline__ void Get(const typename P::Gas& eq,
                                             const typename P::Real* u,
                                             typename P::Wave* w) {
#pragma unroll
    for (int d = 0; d < 3; ++d) w[d] = P::MakeWave(eq, u, d);
  }
};
template <class P> struct WavesOf<P, std::void_t<decltype(&P::MakeWaves)>> {
  static __device__ __forceinline__ void Get(const typename P::Gas& eq,
                                             const typename P::Real* u,
                                             typename P::Wave* w) {
    P::MakeWaves(eq, u, w);
  }
};

// Stable dt of a 3-D grid with every cell loaded and its waves computed once
// (the faces and their speeds are those of StableDtKernelT).  A block of 8
// warps covers 8 consecutive y rows of one 31-cell x range and marches along
// z over `seg` planes: lane 0 of a warp holds the left neighbour of the
// warp's first cell (x faces by a shuffle), the previous plane's z waves stay
// in registers, and the y waves pass from each warp to the next through
// shared memory (double-buffered, one barrier per plane); only the block's
// first warp loads the row below the block.  One atomic per block and
// direction.  Every block is full (rows past ny compute a clamped row and
// take no faces), so all its threads reach every barrier.
constexpr int kDtRows = 8;

template <template <int> class PT>
__global__ void __launch_bounds__(32 * kDtRows) StableDtMarch3Kernel(StableDtArgs a, int seg) {
  using P = PT<3>;
  using R = typename P::Real;
  using W = typename P::Wave;
  constexpr int K = 5;
  __shared__ W ywave[2][kDtRows][32];
  const int nx = a.n[0], ny = a.n[1], nz = a.n[2];
  const int64_t cs = int64_t(nx) * ny * nz;
  if (!BlockAll(!(a.ctrl && (a.ctrl->abort || a.ctrl->done)))) return;
  const typename P::Gas eq = P::MakeGas(a.gamma);
  R smr[3] = {R(0), R(0), R(0)};  // in the policy's precision (no FP64 work per face)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int xw = (nx + 30) / 31;
  const int jblocks = (ny + kDtRows - 1) / kDtRows;
  const int wx = static_cast<int>(blockIdx.x % xw);
  const int jb = static_cast<int>((blockIdx.x / xw) % jblocks);
  // planes [k_lo, k_hi) only when k_hi > 0 (an uploaded slab)
  const int k0 = a.k_lo + static_cast<int>(blockIdx.x / (int64_t(xw) * jblocks)) * seg;
  const int k1 = min(a.k_hi > 0 ? a.k_hi : nz, k0 + seg);
  const int j = jb * kDtRows + warp;
  const bool jvalid = j < ny;
  const int jc = jvalid ? j : ny - 1;
  const int i = wx * 31 + lane - 1;
  const bool own = jvalid && lane >= 1 && i < nx;
  const int ic = BcIndex(i, nx, a.bc[0]);  // lane 0: the left neighbour
  const int jbelow = BcIndex(jb * kDtRows - 1, ny, a.bc[1]);
  auto fetch = [&](int jj, int kk, double* ud) {
    const int64_t off = (int64_t(kk) * ny + jj) * nx + ic;
#pragma unroll
    for (int c = 0; c < K; ++c) ud[c] = __ldg(a.in + c * cs + off);
  };
  auto load = [&](int jj, int kk, R* u) {
    double ud[K];
    fetch(jj, kk, ud);
    P::ToCell(u, ud);
  };
  auto take = [&](R& m, R v) { m = v > m ? v : m; };
  const bool ytile = !(a.rule == 1 && !ReferenceTileFaceT(j, ny, a.width));
  const bool ytop = j == ny - 1 && a.bc[1] != 0 &&
                    !(a.rule == 1 && !ReferenceTileFaceT(ny, ny, a.width));
  W wz_prev;
  {
    R u[K];
    load(jc, BcIndex(k0 - 1, nz, a.bc[2]), u);
    wz_prev = P::MakeWave(eq, u, 2);
  }
  // the next plane's cell, and for warp 0 the cell of the row below the
  // block, are loaded one plane before their use
  double un[K], vn[K] = {};
  fetch(jc, k0, un);
  if (warp == 0) fetch(jbelow, k0, vn);
  for (int k = k0; k < k1; ++k) {
    double ud[K], vd[K];
#pragma unroll
    for (int c = 0; c < K; ++c) {
      ud[c] = un[c];
      vd[c] = vn[c];
    }
    if (k + 1 < k1) {
      fetch(jc, k + 1, un);
      if (warp == 0) fetch(jbelow, k + 1, vn);
    }
    R u[K];
    P::ToCell(u, ud);
    W w[3];
    WavesOf<P>::Get(eq, u, w);
    ywave[k & 1][warp][lane] = w[1];
    W wy_below;
    if (warp == 0) {  // the row below the block
      R v[K];
      P::ToCell(v, vd);
      wy_below = P::MakeWave(eq, v, 1);
    }
    const W wl = ShflUp(w[0], 1);
    __syncthreads();
    if (warp > 0) wy_below = ywave[k & 1][warp - 1][lane];
    if (own) {
      // x: face i (i-1, i); face nx of a transmissive row (nx-1, nx-1)
      take(smr[0], P::FaceMaxSpeed(eq, wl, w[0]));
      if (i == nx - 1 && a.bc[0] != 0) take(smr[0], P::FaceMaxSpeed(eq, w[0], w[0]));
      // y: face j (j-1, j); face ny of a transmissive column
      if (ytile) take(smr[1], P::FaceMaxSpeed(eq, wy_below, w[1]));
      if (ytop) take(smr[1], P::FaceMaxSpeed(eq, w[1], w[1]));
      // z: face k (k-1, k); face nz of a transmissive column
      if (!(a.rule == 1 && !ReferenceTileFaceT(k, nz, a.width)))
        take(smr[2], P::FaceMaxSpeed(eq, wz_prev, w[2]));
      if (k == nz - 1 && a.bc[2] != 0 && !(a.rule == 1 && !ReferenceTileFaceT(nz, nz, a.width)))
        take(smr[2], P::FaceMaxSpeed(eq, w[2], w[2]));
    }
    wz_prev = w[2];
  }
  const double smax[3] = {static_cast<double>(smr[0]), static_cast<double>(smr[1]),
                          static_cast<double>(smr[2])};
  BlockMaxAtomic<3>(a.smax_out, smax);
}

// StableDtMarch3Kernel with the CFL speeds screened in FP32 (EinfeldtCfl
// policies, 1 < gamma <= 2): the same blocks, marching and faces; the FP32
// waves pass between lanes (x), warps (y, shared memory) and planes (z), and
// a direction's exact speeds are evaluated only by warps holding a face of
// that direction whose FP32 speed plus error bound reaches the direction's
// threshold (the lane's own maximum and the pass's maximum published so far,
// every kCflSyncRows planes).  The exact waves of a face's other cell come
// from a shuffle (x) or a reload of its state (y, z; L1 hits).  Cells outside
// the bound's range carry h = inf, so their faces are always evaluated.  The
// per-direction maxima are the same numbers as the unscreened kernel's, bit
// for bit; the max slots must start at zero (or at an exact speed of the same
// state).
template <template <int> class PT>
__global__ void __launch_bounds__(32 * kDtRows) StableDtScreen3Kernel(StableDtArgs a, int seg) {
  using P = PT<3>;
  using R = typename P::Real;
  using W = typename P::Wave;
  using V = fast::Wave<float>;
  constexpr int K = 5;
  constexpr unsigned kAll = 0xffffffffu;
  __shared__ V ycell[2][kDtRows][32];
  const int nx = a.n[0], ny = a.n[1], nz = a.n[2];
  const int64_t cs = int64_t(nx) * ny * nz;
  if (!BlockAll(!(a.ctrl && (a.ctrl->abort || a.ctrl->done)))) return;
  const typename P::Gas eq = P::MakeGas(a.gamma);
  fast::Gas<float> g32;
  g32.gamma = static_cast<float>(a.gamma);
  g32.gm1 = static_cast<float>(a.gamma - 1.0);
  R smr[3] = {R(0), R(0), R(0)};
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int xw = (nx + 30) / 31;
  const int jblocks = (ny + kDtRows - 1) / kDtRows;
  const int wx = static_cast<int>(blockIdx.x % xw);
  const int jb = static_cast<int>((blockIdx.x / xw) % jblocks);
  // planes [k_lo, k_hi) only when k_hi > 0 (an uploaded slab)
  const int k0 = a.k_lo + static_cast<int>(blockIdx.x / (int64_t(xw) * jblocks)) * seg;
  const int k1 = min(a.k_hi > 0 ? a.k_hi : nz, k0 + seg);
  const int j = jb * kDtRows + warp;
  const bool jvalid = j < ny;
  const int jc = jvalid ? j : ny - 1;
  const int i = wx * 31 + lane - 1;
  const bool own = jvalid && lane >= 1 && i < nx;
  const int ic = BcIndex(i, nx, a.bc[0]);  // lane 0: the left neighbour
  const int jbelow = BcIndex(jb * kDtRows - 1, ny, a.bc[1]);
  const int jn = warp > 0 ? j - 1 : jbelow;  // the row below this warp's (own lanes)
  auto fetch = [&](int jj, int kk, double* ud) {
    const int64_t off = (int64_t(kk) * ny + jj) * nx + ic;
#pragma unroll
    for (int c = 0; c < K; ++c) ud[c] = __ldg(a.in + c * cs + off);
  };
  auto load = [&](int jj, int kk, R* u) {
    double ud[K];
    fetch(jj, kk, ud);
    P::ToCell(u, ud);
  };
  // FP32 waves of a cell in the three directions; h = inf outside the range
  auto screen_waves = [&](const R* u, V* v) {
    float c32[K];
#pragma unroll
    for (int c = 0; c < K; ++c) c32[c] = CflToF32(u[c]);
    fast::MakeWaves<3, float>(g32, c32, v);
    const bool ok = CflInRange<3>(c32) && v[0].a > 0.0f;
#pragma unroll
    for (int d = 0; d < 3; ++d) v[d].h = ok ? v[d].h : __int_as_float(0x7f800000);
  };
  auto bound = [&](const V& l, const V& r) {
    const float s32 = fast::FaceMaxSpeed<float>(g32, l, r);
    const float sh = fast::Math<float>::Sqrt(fmaxf(l.h, r.h));
    return fmaf(s32, kCflRel, fmaf(kCflScale, sh, kCflAbs));
  };
  auto take = [&](R& m, R v) { m = v > m ? v : m; };
  const bool ytile = !(a.rule == 1 && !ReferenceTileFaceT(j, ny, a.width));
  const bool ytop = j == ny - 1 && a.bc[1] != 0 &&
                    !(a.rule == 1 && !ReferenceTileFaceT(ny, ny, a.width));
  float thr[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) thr[d] = CflFloatBelow(CflSync(a.smax_out + d, 0.0, kAll));
  V vz_prev;
  {
    R u[K];
    load(jc, BcIndex(k0 - 1, nz, a.bc[2]), u);
    V v[3];
    screen_waves(u, v);
    vz_prev = v[2];
  }
  // the next plane's cell, and for warp 0 the cell of the row below the
  // block, are loaded one plane before their use
  double un[K], vn[K] = {};
  fetch(jc, k0, un);
  if (warp == 0) fetch(jbelow, k0, vn);
  for (int k = k0; k < k1; ++k) {
    double ud[K], vd[K];
#pragma unroll
    for (int c = 0; c < K; ++c) {
      ud[c] = un[c];
      vd[c] = vn[c];
    }
    if (k + 1 < k1) {
      fetch(jc, k + 1, un);
      if (warp == 0) fetch(jbelow, k + 1, vn);
    }
    R u[K];
    P::ToCell(u, ud);
    V v[3];
    screen_waves(u, v);
    ycell[k & 1][warp][lane] = v[1];
    V vy_below;
    if (warp == 0) {  // the row below the block
      R ub[K];
      P::ToCell(ub, vd);
      V vb[3];
      screen_waves(ub, vb);
      vy_below = vb[1];
    }
    const V vl = ShflUp(v[0], 1);
    __syncthreads();
    if (warp > 0) vy_below = ycell[k & 1][warp - 1][lane];
    const bool zface = !(a.rule == 1 && !ReferenceTileFaceT(k, nz, a.width));
    const bool ztop = k == nz - 1 && a.bc[2] != 0 &&
                      !(a.rule == 1 && !ReferenceTileFaceT(nz, nz, a.width));
    const bool xtop = i == nx - 1 && a.bc[0] != 0;
    bool need[3] = {false, false, false};
    if (own) {
      need[0] = !(bound(vl, v[0]) < thr[0]) || (xtop && !(bound(v[0], v[0]) < thr[0]));
      need[1] = (ytile && !(bound(vy_below, v[1]) < thr[1])) ||
                (ytop && !(bound(v[1], v[1]) < thr[1]));
      need[2] = (zface && !(bound(vz_prev, v[2]) < thr[2])) ||
                (ztop && !(bound(v[2], v[2]) < thr[2]));
    }
    const bool any_x = __any_sync(kAll, need[0]);
    const bool any_y = __any_sync(kAll, need[1]);
    const bool any_z = __any_sync(kAll, need[2]);
    if (any_x || any_y || any_z) {
      // exact speeds of the warp's faces in the directions that need them
      W w[3];
      WavesOf<P>::Get(eq, u, w);
      if (any_x) {
        const W wl = ShflUp(w[0], 1);
        if (own) {
          take(smr[0], P::FaceMaxSpeed(eq, wl, w[0]));
          if (xtop) take(smr[0], P::FaceMaxSpeed(eq, w[0], w[0]));
        }
      }
      if (any_y && own) {
        R ub[K];
        load(jn, k, ub);
        if (ytile) take(smr[1], P::FaceMaxSpeed(eq, P::MakeWave(eq, ub, 1), w[1]));
        if (ytop) take(smr[1], P::FaceMaxSpeed(eq, w[1], w[1]));
      }
      if (any_z && own) {
        R uz[K];
        load(jc, BcIndex(k - 1, nz, a.bc[2]), uz);
        if (zface) take(smr[2], P::FaceMaxSpeed(eq, P::MakeWave(eq, uz, 2), w[2]));
        if (ztop) take(smr[2], P::FaceMaxSpeed(eq, w[2], w[2]));
      }
#pragma unroll
      for (int d = 0; d < 3; ++d) thr[d] = fmaxf(thr[d], CflFloatBelow(static_cast<double>(smr[d])));
    }
    if (((k - k0) % kCflSyncRows) == kCflSyncRows - 1) {
#pragma unroll
      for (int d = 0; d < 3; ++d)
        thr[d] = fmaxf(thr[d], CflFloatBelow(CflSync(a.smax_out + d,
                                                     static_cast<double>(smr[d]), kAll)));
    }
    vz_prev = v[2];
  }
  const double smax[3] = {static_cast<double>(smr[0]), static_cast<double>(smr[1]),
                          static_cast<double>(smr[2])};
  BlockMaxAtomic<3>(a.smax_out, smax);
}

template <template <int> class PT>
cudaError_t LaunchStableDtT(const StableDtArgs& a, cudaStream_t s) {
  const int64_t cells = int64_t(a.n[0]) * a.n[1] * a.n[2];
  const int block = 256;
  const bool reflective = a.bc[0] == 2 || a.bc[1] == 2 || a.bc[2] == 2;
  if (a.rank == 3 && !reflective) {
    // blocks of kDtRows x rows; enough blocks for about two waves of the GPU,
    // the planes split accordingly; every block full (see the kernel)
    const int planes = a.k_hi > 0 ? a.k_hi - a.k_lo : a.n[2];
    const int64_t tiles = int64_t((a.n[0] + 30) / 31) * ((a.n[1] + kDtRows - 1) / kDtRows);
    const int64_t want = int64_t(GridStrideBlocks(int64_t(1) << 40, 32 * kDtRows, 8)) * 2;
    const int64_t zseg =
        std::max<int64_t>(1, std::min<int64_t>(planes, (want + tiles - 1) / tiles));
    const int seg = static_cast<int>((planes + zseg - 1) / zseg);
    const unsigned grid = static_cast<unsigned>(tiles * ((planes + seg - 1) / seg));
    if constexpr (EinfeldtCfl<PT<3>>::value) {
      if (a.gamma > 1.0 && a.gamma <= 2.0 && a.smax_out) {
        StableDtScreen3Kernel<PT><<<grid, 32 * kDtRows, 0, s>>>(a, seg);
        return cudaGetLastError();
      }
    }
    StableDtMarch3Kernel<PT><<<grid, 32 * kDtRows, 0, s>>>(a, seg);
    return cudaGetLastError();
  }
  // ranks 1 and 2, and 3-D grids with a reflective direction (the cell-wise
  // kernel reflects the ghost states of the boundary faces); no plane ranges
  if (a.k_hi > 0) return cudaErrorNotSupported;
  const unsigned grid = GridStrideBlocks(cells, block, 8);
  if (a.rank == 1)
    StableDtKernelT<1, PT><<<grid, block, 0, s>>>(a);
  else if (a.rank == 2)
    StableDtKernelT<2, PT><<<grid, block, 0, s>>>(a);
  else
    StableDtKernelT<3, PT><<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace fvs
