// fvs_kernels_exact.cu -- FP64 kernels with the reference's exact arithmetic.
//
// Compiled with -fmad=false (see build.py): no FMA contraction, IEEE
// division and sqrt, so every result is bit-identical to the reference's
// x86-64 build of the same formulas.
#include "fvs_hllem.cuh"
#include "fvs_internal.h"
#include "fvs_recon_hllem.cuh"
#include "fvs_physics_exact.cuh"
#include "fvs_policy_exact.cuh"
#include "fvs_stable.cuh"
#include "fvs_sweep.cuh"

namespace fvs {

cudaError_t LaunchSweepExact(const SweepArgs& a, cudaStream_t s) {
  switch (a.rank) {
  case 1:
    return LaunchSweepT<1, ExactPolicy>(a, s);
  case 2:
    return LaunchSweepT<2, ExactPolicy>(a, s);
  default:
    return LaunchSweepT<3, ExactPolicy>(a, s);
  }
}

// HLLEM sweeps: the marching sweep with Hllem<PerfectGas, Larrouturou> as
// the face flux and its stable-dt speed as the CFL check (fvs_hllem.cuh),
// after one of four reconstructions: none (first order), MUSCL-Hancock of
// the conservative variables, the characteristic or the primitive
// reconstruction of the perfect gas (fvs_recon_hllem.cuh).
template <int D> struct HllemWave {
  exact::Complete<D> q;
  int dir;
};

enum HllemRecon : int { kReconNone = 0, kReconCons = 1, kReconChar = 2, kReconPrim = 3 };

template <int D, int kRecon> struct HllemPolicyT {
  using Real = double;
  static constexpr bool kWarpX = false;
  static constexpr int kMinBlocks = 1;
  static constexpr bool kHllemCfl = true;  // CFL speeds screened in FP32 (HllemScreen)
  using Gas = exact::Gas;
  using Rec = exact::Complete<D>;
  using Wave = HllemWave<D>;
  using Stats = NoStats;
  static __device__ __forceinline__ Gas MakeGas(double gamma) {
    return ExactPolicy<D>::MakeGas(gamma);
  }
  static __device__ __forceinline__ Gas MakeGasFor(const SweepArgs& a) { return MakeGas(a.gamma); }
  static __device__ __forceinline__ void ToCell(double* c, const double* u) {
#pragma unroll
    for (int k = 0; k < D + 2; ++k) c[k] = u[k];
  }
  static __device__ __forceinline__ void Predict(const Gas& eq, Rec& recL, Rec& recR,
                                                 const double* q0, const double* q1,
                                                 const double* q2, int limiter,
                                                 double lambda_half, int dir) {
    if constexpr (kRecon == kReconCons) {
      exact::MusclPredictBoth<D>(eq, recL, recR, q0, q1, q2, limiter, lambda_half, dir);
    } else if constexpr (kRecon == kReconChar || kRecon == kReconPrim) {
      // dt/dx: lambda_half is (0.5 dt)/dx, so doubling it is exact
      const double lambda = 2.0 * lambda_half;
      exact::Complete<D> s0, s1, s2;
      exact::CompleteFromCons<D>(eq, s0, q0);
      exact::CompleteFromCons<D>(eq, s1, q1);
      exact::CompleteFromCons<D>(eq, s2, q2);
      if constexpr (kRecon == kReconChar)
        exact::CharPredictBoth<D>(eq, recL, recR, s0, s1, s2, lambda, dir);
      else
        exact::PrimPredictBoth<D>(eq, recL, recR, s0, s1, s2, lambda, dir);
    } else {
      exact::CompleteFromCons<D>(eq, recL, q1);
      recR = recL;
    }
  }
  static __device__ __forceinline__ Wave MakeWave(const Gas& eq, const double* u, int dir) {
    Wave w;
    exact::CompleteFromCons<D>(eq, w.q, u);
    w.dir = dir;
    return w;
  }
  static __device__ __forceinline__ double FaceMaxSpeed(const Gas& eq, const Wave& wL,
                                                        const Wave& wR) {
    return exact::HllemMaxSpeed<D>(eq, wL.q, wR.q, wL.dir);
  }
  static __device__ __forceinline__ void FluxOnly(const Gas& eq, double* F, const Rec& L,
                                                  const Rec& R, int dir) {
    exact::HllemFlux<D>(eq, F, L, R, dir);
  }
  static __device__ __forceinline__ double Face(const Gas& eq, double* F, const Rec& L,
                                                const Rec& R, const Wave& wL, const Wave& wR,
                                                int dir, Stats&) {
    exact::HllemFlux<D>(eq, F, L, R, dir);
    return exact::HllemMaxSpeed<D>(eq, wL.q, wR.q, dir);
  }
};

template <int D> struct HllemPolicy : HllemPolicyT<D, kReconNone> {};
template <int D> struct MusclHllemPolicy : HllemPolicyT<D, kReconCons> {};
template <int D> struct CharHllemPolicy : HllemPolicyT<D, kReconChar> {};
template <int D> struct PrimHllemPolicy : HllemPolicyT<D, kReconPrim> {};

template <template <int> class PT>
cudaError_t LaunchSweepRanks(const SweepArgs& a, cudaStream_t s) {
  switch (a.rank) {
  case 1:
    return LaunchSweepT<1, PT>(a, s);
  case 2:
    return LaunchSweepT<2, PT>(a, s);
  default:
    return LaunchSweepT<3, PT>(a, s);
  }
}

cudaError_t LaunchSweepHllem(const SweepArgs& a, int recon, cudaStream_t s) {
  switch (recon) {
  case kReconCons:
    return LaunchSweepRanks<MusclHllemPolicy>(a, s);
  case kReconChar:
    return LaunchSweepRanks<CharHllemPolicy>(a, s);
  case kReconPrim:
    return LaunchSweepRanks<PrimHllemPolicy>(a, s);
  default:
    return LaunchSweepRanks<HllemPolicy>(a, s);
  }
}

cudaError_t LaunchStableDtHllem(const StableDtArgs& a, cudaStream_t s) {
  return LaunchStableDtT<HllemPolicy>(a, s);
}

// ---------------------------------------------------------------------------
// Stable dt of a uniform grid over all directions.

// Whether face f (between cells f-1 and f, 0 <= f <= n) of a direction of n
// cells enters the reference's dt: MFIter tiles of 8 cells grown by 2 ghost
// layers at the box boundary, windows of 2w cells inside each tile, the
// window's middle pair is the face (FluxMethodAdapter.hpp:85-96,
// FluxMethod.hpp:341-382).
__device__ __forceinline__ bool ReferenceTileFace(int f, int n, int w) {
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

template <int D>
__global__ void __launch_bounds__(256) StableDtKernel(StableDtArgs a) {
  constexpr int K = D + 2;
  const int nx = a.n[0], ny = a.n[1], nz = a.n[2];
  const int64_t cs = int64_t(nx) * ny * nz;
  if (!BlockAll(!(a.ctrl && (a.ctrl->abort || a.ctrl->done)))) return;
  const exact::Gas eq = ExactPolicy<1>::MakeGas(a.gamma);
  double smax[3] = {0.0, 0.0, 0.0};
  // grid-stride over cells; one atomic per block and direction at the end
  for (int64_t cell = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; cell < cs;
       cell += int64_t(gridDim.x) * blockDim.x) {
    const int i = static_cast<int>(cell % nx);
    const int j = static_cast<int>((cell / nx) % ny);
    const int k = static_cast<int>(cell / (int64_t(nx) * ny));
    const int idx[3] = {i, j, k};
    double u[K];
#pragma unroll
    for (int c = 0; c < K; ++c) u[c] = __ldg(a.in + c * cs + cell);
    exact::Complete<D> q;
    exact::CompleteFromCons<D>(eq, q, u);
    const double sq = sqrt(q.rho);
    const double h = (q.E + q.p) / q.rho;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      exact::CellWave w;
      w.sq = sq;
      w.u = q.m[d] / q.rho;
      w.h = h;
      w.a = q.c;
      const int nd = a.n[d];
      // face idx[d] (between idx[d]-1 and idx[d]); the thread of the last
      // cell also takes face n (its upper boundary face).
      const int faces = (idx[d] == nd - 1) ? 2 : 1;
      for (int fi = 0; fi < faces; ++fi) {
        const int f = idx[d] + fi;
        if (a.rule == 1 && d > 0 && !ReferenceTileFace(f, nd, a.width)) continue;
        if (fi == 1 && a.bc[d] == 0) continue;  // periodic: face n == face 0
        const int og = fi == 0 ? f - 1 : f;
        const int other = BcIndex(og, nd, a.bc[d]);
        int oidx[3] = {i, j, k};
        oidx[d] = other;
        const int64_t ocell =
            (int64_t(oidx[2]) * ny + oidx[1]) * int64_t(nx) + oidx[0];
        double v[K];
#pragma unroll
        for (int c = 0; c < K; ++c) v[c] = __ldg(a.in + c * cs + ocell);
        if (BcFlip(og, nd, a.bc[d])) v[1 + d] = -v[1 + d];
        const exact::CellWave wo = exact::MakeCellWave<D>(eq, v, d);
        const double s = (fi == 0) ? exact::FaceMaxSpeed(eq, wo, w)
                                   : exact::FaceMaxSpeed(eq, w, wo);
        smax[d] = s > smax[d] ? s : smax[d];
      }
    }
  }
  BlockMaxAtomic<D>(a.smax_out, smax);
}

cudaError_t LaunchStableDtExact(const StableDtArgs& a, cudaStream_t s) {
  // 3-D: the marching pass (each cell completed once), with the same face
  // speeds as StableDtKernel
  if (a.rank == 3) return LaunchStableDtT<ExactPolicy>(a, s);
  const int64_t cells = int64_t(a.n[0]) * a.n[1] * a.n[2];
  const int block = 256;
  const unsigned grid = GridStrideBlocks(cells, block, 8);
  switch (a.rank) {
  case 1:
    StableDtKernel<1><<<grid, block, 0, s>>>(a);
    break;
  case 2:
    StableDtKernel<2><<<grid, block, 0, s>>>(a);
    break;
  default:
    StableDtKernel<3><<<grid, block, 0, s>>>(a);
    break;
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Patch-level kernels over FArrayBox-layout box views (component-major,
// x fastest).  These are the drop-in replacements of the reference's
// patch-level FluxMethod / HyperbolicPatchIntegrator calls.

struct View {
  const double* p;
  BoxDesc b;
  __device__ __forceinline__ int64_t Index(int c, int i, int j, int k) const {
    return ((int64_t(c) * b.n[2] + (k - b.lo[2])) * b.n[1] + (j - b.lo[1])) *
               int64_t(b.n[0]) +
           (i - b.lo[0]);
  }
  __device__ __forceinline__ double operator()(int c, int i, int j, int k) const {
    return p[Index(c, i, j, k)];
  }
};

template <int D>
__device__ __forceinline__ exact::Complete<D> LoadComplete(const View& v, int i,
                                                           int j, int k) {
  exact::Complete<D> q;
  q.rho = v(0, i, j, k);
#pragma unroll
  for (int d = 0; d < D; ++d) q.m[d] = v(1 + d, i, j, k);
  q.E = v(1 + D, i, j, k);
  q.p = v(2 + D, i, j, k);
  q.c = v(3 + D, i, j, k);
  return q;
}

__device__ __forceinline__ void Unflatten(int64_t id, const BoxDesc& b, int* ijk) {
  ijk[0] = b.lo[0] + static_cast<int>(id % b.n[0]);
  ijk[1] = b.lo[1] + static_cast<int>((id / b.n[0]) % b.n[1]);
  ijk[2] = b.lo[2] + static_cast<int>(id / (int64_t(b.n[0]) * b.n[1]));
}

// FluxMethod<Base>::ComputeNumericFluxes (FluxMethod.hpp:200-215): face f
// takes the 2w cells f-w .. f+w-1 along dir.
template <int D>
__global__ void PatchFluxKernel(int method, int limiter, double gamma,
                                double* fluxes, BoxDesc fbox, View st,
                                double dt, double dx, int dir) {
  constexpr int K = D + 2;
  const int64_t nface = int64_t(fbox.n[0]) * fbox.n[1] * fbox.n[2];
  const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (id >= nface) return;
  int f[3];
  Unflatten(id, fbox, f);
  const exact::Gas eq = ExactPolicy<1>::MakeGas(gamma);
  double nf[K];
  if (method == 1 || method == 4) {  // HLLE / HLLEM, stencil width 1
    int c0[3] = {f[0], f[1], f[2]};
    c0[dir] -= 1;
    const exact::Complete<D> L = LoadComplete<D>(st, c0[0], c0[1], c0[2]);
    const exact::Complete<D> R = LoadComplete<D>(st, f[0], f[1], f[2]);
    if (method == 1)
      exact::HllFlux<D>(eq, nf, L, R, dir);
    else
      exact::HllemFlux<D>(eq, nf, L, R, dir);
  } else if (method == 6 || method == 7) {
    // characteristic / primitive reconstruction + HLLEM, stencil width 2
    // (MusclHancockCharacteristicMethod.hpp:303-317,
    // MusclHancockPrimMethod.hpp:59-182), from the stored complete states
    const double lambda = dt / dx;
    exact::Complete<D> q[4];
    for (int s = 0; s < 4; ++s) {
      int c[3] = {f[0], f[1], f[2]};
      c[dir] += s - 2;
      q[s] = LoadComplete<D>(st, c[0], c[1], c[2]);
    }
    exact::Complete<D> a0, b0, a1, b1;
    if (method == 6) {
      exact::CharPredictBoth<D>(eq, a0, b0, q[0], q[1], q[2], lambda, dir);
      exact::CharPredictBoth<D>(eq, a1, b1, q[1], q[2], q[3], lambda, dir);
    } else {
      exact::PrimPredictBoth<D>(eq, a0, b0, q[0], q[1], q[2], lambda, dir);
      exact::PrimPredictBoth<D>(eq, a1, b1, q[1], q[2], q[3], lambda, dir);
    }
    exact::HllemFlux<D>(eq, nf, b0, a1, dir);
  } else {  // MUSCL-Hancock (conservative) + HLLE / HLLEM, stencil width 2
    double u[4][K];
    for (int s = 0; s < 4; ++s) {
      int c[3] = {f[0], f[1], f[2]};
      c[dir] += s - 2;
#pragma unroll
      for (int q = 0; q < K; ++q) u[s][q] = st(q, c[0], c[1], c[2]);
    }
    exact::Complete<D> a0, b0, a1, b1;
    const double lambda_half = 0.5 * dt / dx;
    exact::MusclPredictBoth<D>(eq, a0, b0, u[0], u[1], u[2], limiter,
                               lambda_half, dir);
    exact::MusclPredictBoth<D>(eq, a1, b1, u[1], u[2], u[3], limiter,
                               lambda_half, dir);
    if (method == 5)
      exact::HllemFlux<D>(eq, nf, b0, a1, dir);
    else
      exact::HllFlux<D>(eq, nf, b0, a1, dir);
  }
  View fv{fluxes, fbox};
#pragma unroll
  for (int q = 0; q < K; ++q) fluxes[fv.Index(q, f[0], f[1], f[2])] = nf[q];
}

cudaError_t LaunchPatchFluxesExact(int method, int limiter, int rank,
                                   double gamma, double* fluxes, BoxDesc fbox,
                                   const double* states, BoxDesc cbox,
                                   double dt, double dx, int dir,
                                   cudaStream_t s) {
  const int64_t nface = int64_t(fbox.n[0]) * fbox.n[1] * fbox.n[2];
  if (nface == 0) return cudaSuccess;
  const int block = 128;
  const unsigned grid = static_cast<unsigned>((nface + block - 1) / block);
  View st{states, cbox};
  switch (rank) {
  case 1:
    PatchFluxKernel<1><<<grid, block, 0, s>>>(method, limiter, gamma, fluxes,
                                              fbox, st, dt, dx, dir);
    break;
  case 2:
    PatchFluxKernel<2><<<grid, block, 0, s>>>(method, limiter, gamma, fluxes,
                                              fbox, st, dt, dx, dir);
    break;
  default:
    PatchFluxKernel<3><<<grid, block, 0, s>>>(method, limiter, gamma, fluxes,
                                              fbox, st, dt, dx, dir);
    break;
  }
  return cudaGetLastError();
}

// FluxMethod<Base>::ComputeStableDt over windows of 2w cells; window_rule 0
// is the sequential tag (FluxMethod.hpp:295-314), 1 the simd tag
// (FluxMethod.hpp:341-382).  Writes the max face speed; dt = dx / speed.
template <int D>
__global__ void PatchStableDtKernel(int w, int hllem, double gamma, View st, BoxDesc wbox,
                                    int dir, unsigned long long* smax_out) {
  const int64_t nwin = int64_t(wbox.n[0]) * wbox.n[1] * wbox.n[2];
  const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  double s = 0.0;
  if (id < nwin) {
    int c[3];
    Unflatten(id, wbox, c);
    c[dir] += w - 1;
    const exact::Complete<D> L = LoadComplete<D>(st, c[0], c[1], c[2]);
    c[dir] += 1;
    const exact::Complete<D> R = LoadComplete<D>(st, c[0], c[1], c[2]);
    const exact::Gas eq = ExactPolicy<1>::MakeGas(gamma);
    if (hllem) {
      s = exact::HllemMaxSpeed<D>(eq, L, R, dir);
    } else {
      double s0, s1;
      exact::Einfeldt<D>(eq, L, R, dir, s0, s1);
      s = exact::PMax(exact::PMax(0.0, fabs(s0)), fabs(s1));
    }
  }
  s = WarpMax(s);
  if ((threadIdx.x & 31) == 0 && s > 0.0) AtomicMaxPositive(smax_out, s);
}

cudaError_t LaunchPatchStableDtExact(int method, int rank, double gamma,
                                     const double* states, BoxDesc cbox,
                                     int window_rule, int dir,
                                     unsigned long long* smax, cudaStream_t s) {
  const int w = (method == 1 || method == 4) ? 1 : 2;
  const int hllem = (method >= 4) ? 1 : 0;
  BoxDesc wbox = cbox;
  wbox.n[dir] -= (window_rule == 0) ? 2 * w : 2 * w - 1;
  if (wbox.n[dir] <= 0) return cudaSuccess;
  const int64_t nwin = int64_t(wbox.n[0]) * wbox.n[1] * wbox.n[2];
  const int block = 128;
  const unsigned grid = static_cast<unsigned>((nwin + block - 1) / block);
  View st{states, cbox};
  switch (rank) {
  case 1:
    PatchStableDtKernel<1><<<grid, block, 0, s>>>(w, hllem, gamma, st, wbox, dir, smax);
    break;
  case 2:
    PatchStableDtKernel<2><<<grid, block, 0, s>>>(w, hllem, gamma, st, wbox, dir, smax);
    break;
  default:
    PatchStableDtKernel<3><<<grid, block, 0, s>>>(w, hllem, gamma, st, wbox, dir, smax);
    break;
  }
  return cudaGetLastError();
}

// HyperbolicPatchIntegrator::UpdateConservatively
// (src/HyperbolicPatchIntegrator.cpp:88-105): next = prev + dt/dx (F_L - F_R).
__global__ void PatchUpdateKernel(double* next, BoxDesc nbox, BoxDesc region, View prev,
                                  View flux, int ncomp, double dt_dx, int dir) {
  const int64_t ncell = int64_t(region.n[0]) * region.n[1] * region.n[2];
  const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (id >= ncell) return;
  int c[3];
  Unflatten(id, region, c);
  int r[3] = {c[0], c[1], c[2]};
  r[dir] += 1;
  View nv{next, nbox};
  for (int q = 0; q < ncomp; ++q) {
    const double U_prev = prev(q, c[0], c[1], c[2]);
    const double f_left = flux(q, c[0], c[1], c[2]);
    const double f_right = flux(q, r[0], r[1], r[2]);
    next[nv.Index(q, c[0], c[1], c[2])] = U_prev + dt_dx * (f_left - f_right);
  }
}

cudaError_t LaunchPatchUpdate(double* next, BoxDesc nbox, BoxDesc region, const double* prev,
                              BoxDesc pbox, const double* fluxes, BoxDesc fbox,
                              int ncomp, double dt, double dx, int dir,
                              cudaStream_t s) {
  const int64_t ncell = int64_t(region.n[0]) * region.n[1] * region.n[2];
  if (ncell == 0) return cudaSuccess;
  const double dt_dx = dt / dx;
  const int block = 256;
  const unsigned grid = static_cast<unsigned>((ncell + block - 1) / block);
  PatchUpdateKernel<<<grid, block, 0, s>>>(next, nbox, region, View{prev, pbox},
                                           View{fluxes, fbox}, ncomp, dt_dx, dir);
  return cudaGetLastError();
}

// Reconstruction::CompleteFromCons over a region (include/fub/AMReX/
// Reconstruction.hpp:44-60 -> PerfectGas.cpp:96-124).
template <int D>
__global__ void PatchCompleteKernel(double gamma, double* complete,
                                    BoxDesc qbox, View cons, BoxDesc region) {
  constexpr int K = D + 2;
  const int64_t ncell = int64_t(region.n[0]) * region.n[1] * region.n[2];
  const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (id >= ncell) return;
  int c[3];
  Unflatten(id, region, c);
  double u[K];
#pragma unroll
  for (int q = 0; q < K; ++q) u[q] = cons(q, c[0], c[1], c[2]);
  const exact::Gas eq = ExactPolicy<1>::MakeGas(gamma);
  exact::Complete<D> s;
  exact::CompleteFromCons<D>(eq, s, u);
  View qv{complete, qbox};
  complete[qv.Index(0, c[0], c[1], c[2])] = s.rho;
#pragma unroll
  for (int d = 0; d < D; ++d) complete[qv.Index(1 + d, c[0], c[1], c[2])] = s.m[d];
  complete[qv.Index(1 + D, c[0], c[1], c[2])] = s.E;
  complete[qv.Index(2 + D, c[0], c[1], c[2])] = s.p;
  complete[qv.Index(3 + D, c[0], c[1], c[2])] = s.c;
}

cudaError_t LaunchPatchCompleteFromCons(int rank, double gamma, double* complete,
                                        BoxDesc qbox, const double* cons,
                                        BoxDesc ubox, BoxDesc region,
                                        cudaStream_t s) {
  const int64_t ncell = int64_t(region.n[0]) * region.n[1] * region.n[2];
  if (ncell == 0) return cudaSuccess;
  const int block = 256;
  const unsigned grid = static_cast<unsigned>((ncell + block - 1) / block);
  View cv{cons, ubox};
  switch (rank) {
  case 1:
    PatchCompleteKernel<1><<<grid, block, 0, s>>>(gamma, complete, qbox, cv, region);
    break;
  case 2:
    PatchCompleteKernel<2><<<grid, block, 0, s>>>(gamma, complete, qbox, cv, region);
    break;
  default:
    PatchCompleteKernel<3><<<grid, block, 0, s>>>(gamma, complete, qbox, cv, region);
    break;
  }
  return cudaGetLastError();
}

}  // namespace fvs
