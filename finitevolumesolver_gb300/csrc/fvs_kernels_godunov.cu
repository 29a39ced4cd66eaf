// fvs_kernels_godunov.cu -- Godunov (exact Riemann solver) fluxes: the fused
// uniform-grid sweep, the stable-dt pass, the patch-level calls and a batch
// star-state solver.  Compiled with -fmad=false (reference operation order;
// only pow differs from the CPU by a few ulps).
#include "../../include/fvs_gpu.h"
#include "fvs_internal.h"
#include "fvs_riemann.cuh"
#include "fvs_stable.cuh"
#include "fvs_sweep.cuh"

namespace fvs {

struct GodunovGas {
  exact::Gas eq;
  riemann::Options opt;
};

__device__ __forceinline__ GodunovGas MakeGodunovGas(double gamma, int guess, int max_it,
                                                     double tol, const float* mlp) {
  GodunovGas g;
  g.eq.gamma = gamma;
  g.eq.gamma_minus_1_inv = 1.0 / (gamma - 1.0);
  g.opt.guess = guess;
  g.opt.max_iterations = max_it;
  g.opt.tol = tol;
  g.opt.mlp = mlp;
  g.opt.root_n = riemann::RootOrder(gamma);
  return g;
}

// Godunov<PerfectGas, ExactRiemannSolver> (first order, stencil width 1) and
// MusclHancock<PerfectGas, Godunov<ExactRiemannSolver>, Limiter> (MUSCL).
// The face state pair of first-order Godunov is the pair of cell states, so
// one exact solve gives both the flux and the CFL speed of the face (the
// reference solves the same problem twice: GodunovMethod.hpp:129-183).  The
// MUSCL variant solves the predicted states for the flux and the cell states
// for the CFL check, as the reference does.
template <int D, bool kMuscl> struct GodunovPolicyT {
  using Real = double;
  static constexpr bool kWarpX = false;
  static constexpr int kMinBlocks = 1;
  using Gas = GodunovGas;
  using Rec = exact::Complete<D>;
  using Wave = exact::Complete<D>;
  using Stats = NewtonStats;
  static __device__ __forceinline__ Gas MakeGasFor(const SweepArgs& a) {
    return MakeGodunovGas(a.gamma, a.guess, a.max_iterations, a.tolerance, a.mlp);
  }
  static __device__ __forceinline__ void ToCell(double* c, const double* u) {
#pragma unroll
    for (int k = 0; k < D + 2; ++k) c[k] = u[k];
  }
  static __device__ __forceinline__ void Predict(const Gas& g, Rec& recL, Rec& recR,
                                                 const double* q0, const double* q1,
                                                 const double* q2, int limiter,
                                                 double lambda_half, int dir) {
    if constexpr (kMuscl) {
      exact::MusclPredictBoth<D>(g.eq, recL, recR, q0, q1, q2, limiter, lambda_half, dir);
    } else {
      riemann::CompleteFromConsFast<D>(g.eq, recL, q1);
      recR = recL;
    }
  }
  static __device__ __forceinline__ Wave MakeWave(const Gas& g, const double* u, int) {
    Wave w;
    riemann::CompleteFromConsFast<D>(g.eq, w, u);
    return w;
  }
  static __device__ __forceinline__ double Face(const Gas& g, double* F, const Rec& L,
                                                const Rec& R, const Wave& wL, const Wave& wR,
                                                int dir, Stats& st) {
    const riemann::Star s = riemann::GodunovFlux<D>(g.eq, F, L, R, dir, g.opt);
    st.iterations += s.iterations;
    st.failures += s.converged ? 0 : 1;
    st.fallbacks += s.fallback;
    if constexpr (kMuscl) {
      const riemann::Star c = riemann::ComputeMiddleState<D>(g.eq, wL, wR, dir, g.opt);
      st.iterations += c.iterations;
      st.failures += c.converged ? 0 : 1;
      st.fallbacks += c.fallback;
      return riemann::SignalMaxSpeed<D>(g.eq, wL, wR, dir, c.p);
    } else {
      return riemann::SignalMaxSpeed<D>(g.eq, L, R, dir, s.p);
    }
  }
};

template <int D> struct GodunovPolicy : GodunovPolicyT<D, false> {};
template <int D> struct MusclGodunovPolicy : GodunovPolicyT<D, true> {};

cudaError_t LaunchSweepGodunov(const SweepArgs& a, bool muscl, cudaStream_t s) {
  switch (a.rank) {
  case 1:
    return muscl ? LaunchSweepT<1, MusclGodunovPolicy>(a, s) : LaunchSweepT<1, GodunovPolicy>(a, s);
  case 2:
    return muscl ? LaunchSweepT<2, MusclGodunovPolicy>(a, s) : LaunchSweepT<2, GodunovPolicy>(a, s);
  default:
    return muscl ? LaunchSweepT<3, MusclGodunovPolicy>(a, s) : LaunchSweepT<3, GodunovPolicy>(a, s);
  }
}

// Stable dt over all directions with the exact solver's signal speeds.
template <int D>
__global__ void __launch_bounds__(256) GodunovStableDtKernel(StableDtArgs a, int guess, int max_it,
                                                             double tol, const float* mlp) {
  constexpr int K = D + 2;
  const int nx = a.n[0], ny = a.n[1], nz = a.n[2];
  const int64_t cs = int64_t(nx) * ny * nz;
  if (!BlockAll(!(a.ctrl && (a.ctrl->abort || a.ctrl->done)))) return;
  const GodunovGas g = MakeGodunovGas(a.gamma, guess, max_it, tol, mlp);
  double smax[3] = {0.0, 0.0, 0.0};
  // grid-stride over cells; one atomic per block and direction at the end
  for (int64_t cell = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; cell < cs;
       cell += int64_t(gridDim.x) * blockDim.x) {
    const int idx[3] = {static_cast<int>(cell % nx), static_cast<int>((cell / nx) % ny),
                        static_cast<int>(cell / (int64_t(nx) * ny))};
    double u[K];
#pragma unroll
    for (int c = 0; c < K; ++c) u[c] = __ldg(a.in + c * cs + cell);
    exact::Complete<D> q;
    exact::CompleteFromCons<D>(g.eq, q, u);
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const int nd = a.n[d];
      const int faces = (idx[d] == nd - 1) ? 2 : 1;
      for (int fi = 0; fi < faces; ++fi) {
        const int f = idx[d] + fi;
        if (a.rule == 1 && d > 0 && !ReferenceTileFaceT(f, nd, a.width)) continue;
        if (fi == 1 && a.bc[d] == 0) continue;
        int oidx[3] = {idx[0], idx[1], idx[2]};
        const int og = fi == 0 ? f - 1 : f;
        oidx[d] = BcIndex(og, nd, a.bc[d]);
        const int64_t ocell = (int64_t(oidx[2]) * ny + oidx[1]) * int64_t(nx) + oidx[0];
        double v[K];
#pragma unroll
        for (int c = 0; c < K; ++c) v[c] = __ldg(a.in + c * cs + ocell);
        if (BcFlip(og, nd, a.bc[d])) v[1 + d] = -v[1 + d];
        exact::Complete<D> o;
        exact::CompleteFromCons<D>(g.eq, o, v);
        const exact::Complete<D>& L = (fi == 0) ? o : q;
        const exact::Complete<D>& R = (fi == 0) ? q : o;
        const riemann::Star st = riemann::ComputeMiddleState<D>(g.eq, L, R, d, g.opt);
        const double sp = riemann::SignalMaxSpeed<D>(g.eq, L, R, d, st.p);
        smax[d] = sp > smax[d] ? sp : smax[d];
      }
    }
  }
  BlockMaxAtomic<D>(a.smax_out, smax);
}

cudaError_t LaunchStableDtGodunov(const StableDtArgs& a, int guess, int max_it, double tol,
                                  const float* mlp, cudaStream_t s) {
  const int64_t cells = int64_t(a.n[0]) * a.n[1] * a.n[2];
  const int block = 256;
  const unsigned grid = GridStrideBlocks(cells, block, 8);
  switch (a.rank) {
  case 1:
    GodunovStableDtKernel<1><<<grid, block, 0, s>>>(a, guess, max_it, tol, mlp);
    break;
  case 2:
    GodunovStableDtKernel<2><<<grid, block, 0, s>>>(a, guess, max_it, tol, mlp);
    break;
  default:
    GodunovStableDtKernel<3><<<grid, block, 0, s>>>(a, guess, max_it, tol, mlp);
    break;
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Patch-level Godunov fluxes and stable dt over FArrayBox-layout views.

namespace {

struct GView {
  const double* p;
  BoxDesc b;
  __device__ __forceinline__ int64_t Index(int c, int i, int j, int k) const {
    return ((int64_t(c) * b.n[2] + (k - b.lo[2])) * b.n[1] + (j - b.lo[1])) * int64_t(b.n[0]) +
           (i - b.lo[0]);
  }
  __device__ __forceinline__ double operator()(int c, int i, int j, int k) const {
    return p[Index(c, i, j, k)];
  }
};

template <int D>
__device__ __forceinline__ exact::Complete<D> LoadC(const GView& v, const int* c) {
  exact::Complete<D> q;
  q.rho = v(0, c[0], c[1], c[2]);
#pragma unroll
  for (int d = 0; d < D; ++d) q.m[d] = v(1 + d, c[0], c[1], c[2]);
  q.E = v(1 + D, c[0], c[1], c[2]);
  q.p = v(2 + D, c[0], c[1], c[2]);
  q.c = v(3 + D, c[0], c[1], c[2]);
  return q;
}

__device__ __forceinline__ void Unflat(int64_t id, const BoxDesc& b, int* ijk) {
  ijk[0] = b.lo[0] + static_cast<int>(id % b.n[0]);
  ijk[1] = b.lo[1] + static_cast<int>((id / b.n[0]) % b.n[1]);
  ijk[2] = b.lo[2] + static_cast<int>(id / (int64_t(b.n[0]) * b.n[1]));
}

template <int D>
__global__ void PatchGodunovFluxKernel(bool muscl, int limiter, GodunovGas g, double* fluxes,
                                       BoxDesc fbox, GView st, double dt, double dx, int dir,
                                       unsigned long long* stats) {
  constexpr int K = D + 2;
  const int64_t nface = int64_t(fbox.n[0]) * fbox.n[1] * fbox.n[2];
  const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  NewtonStats ns;
  if (id < nface) {
    int f[3];
    Unflat(id, fbox, f);
    double nf[K];
    riemann::Star s;
    if (!muscl) {
      int c0[3] = {f[0], f[1], f[2]};
      c0[dir] -= 1;
      s = riemann::GodunovFlux<D>(g.eq, nf, LoadC<D>(st, c0), LoadC<D>(st, f), dir, g.opt);
    } else {
      double u[4][K];
      for (int q = 0; q < 4; ++q) {
        int c[3] = {f[0], f[1], f[2]};
        c[dir] += q - 2;
#pragma unroll
        for (int k = 0; k < K; ++k) u[q][k] = st(k, c[0], c[1], c[2]);
      }
      const double lambda_half = 0.5 * dt / dx;
      exact::Complete<D> a0, b0, a1, b1;
      exact::MusclPredictBoth<D>(g.eq, a0, b0, u[0], u[1], u[2], limiter, lambda_half, dir);
      exact::MusclPredictBoth<D>(g.eq, a1, b1, u[1], u[2], u[3], limiter, lambda_half, dir);
      s = riemann::GodunovFlux<D>(g.eq, nf, b0, a1, dir, g.opt);
    }
    ns.iterations = s.iterations;
    ns.failures = s.converged ? 0 : 1;
    ns.fallbacks = s.fallback;
    GView fv{fluxes, fbox};
#pragma unroll
    for (int k = 0; k < K; ++k) fluxes[fv.Index(k, f[0], f[1], f[2])] = nf[k];
  }
  ns.Flush(stats);
}

template <int D>
__global__ void PatchGodunovDtKernel(int w, GodunovGas g, GView st, BoxDesc wbox, int dir,
                                     unsigned long long* smax_out) {
  const int64_t nwin = int64_t(wbox.n[0]) * wbox.n[1] * wbox.n[2];
  const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  double s = 0.0;
  if (id < nwin) {
    int c[3];
    Unflat(id, wbox, c);
    c[dir] += w - 1;
    const exact::Complete<D> L = LoadC<D>(st, c);
    c[dir] += 1;
    const exact::Complete<D> R = LoadC<D>(st, c);
    const riemann::Star m = riemann::ComputeMiddleState<D>(g.eq, L, R, dir, g.opt);
    s = riemann::SignalMaxSpeed<D>(g.eq, L, R, dir, m.p);
  }
  s = WarpMax(s);
  if ((threadIdx.x & 31) == 0 && s > 0.0) AtomicMaxPositive(smax_out, s);
}

template <int D>
__global__ void ExactStarKernel(int64_t n, GodunovGas g, const double* rhoL, const double* uL,
                                const double* pL, const double* rhoR, const double* uR,
                                const double* pR, double* pstar, double* ustar, int* iters,
                                int* converged) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  exact::Complete<1> L, R;
  L.rho = rhoL[i];
  L.m[0] = rhoL[i] * uL[i];
  L.p = pL[i];
  L.E = pL[i] * g.eq.gamma_minus_1_inv + 0.5 * L.m[0] * L.m[0] / L.rho;
  L.c = sqrt(g.eq.gamma * L.p / L.rho);
  R.rho = rhoR[i];
  R.m[0] = rhoR[i] * uR[i];
  R.p = pR[i];
  R.E = pR[i] * g.eq.gamma_minus_1_inv + 0.5 * R.m[0] * R.m[0] / R.rho;
  R.c = sqrt(g.eq.gamma * R.p / R.rho);
  const riemann::Star st = riemann::ComputeMiddleState<1>(g.eq, L, R, 0, g.opt);
  if (pstar) pstar[i] = st.p;
  if (ustar) ustar[i] = st.u;
  if (iters) iters[i] = st.iterations;
  if (converged) converged[i] = st.converged ? (st.fallback ? 2 : 1) : 0;
}

}  // namespace

cudaError_t LaunchPatchGodunovFluxes(bool muscl, int limiter, int rank, double gamma, int guess,
                                     int max_it, double tol, const float* mlp, double* fluxes,
                                     BoxDesc fbox, const double* states, BoxDesc cbox, double dt,
                                     double dx, int dir, unsigned long long* stats,
                                     cudaStream_t s) {
  const int64_t nface = int64_t(fbox.n[0]) * fbox.n[1] * fbox.n[2];
  if (nface == 0) return cudaSuccess;
  const int block = 128;
  const unsigned grid = static_cast<unsigned>((nface + block - 1) / block);
  const GodunovGas g{{gamma, 1.0 / (gamma - 1.0)}, {guess, max_it, tol, mlp}};
  const GView st{states, cbox};
  switch (rank) {
  case 1:
    PatchGodunovFluxKernel<1><<<grid, block, 0, s>>>(muscl, limiter, g, fluxes, fbox, st, dt, dx,
                                                     dir, stats);
    break;
  case 2:
    PatchGodunovFluxKernel<2><<<grid, block, 0, s>>>(muscl, limiter, g, fluxes, fbox, st, dt, dx,
                                                     dir, stats);
    break;
  default:
    PatchGodunovFluxKernel<3><<<grid, block, 0, s>>>(muscl, limiter, g, fluxes, fbox, st, dt, dx,
                                                     dir, stats);
    break;
  }
  return cudaGetLastError();
}

cudaError_t LaunchPatchGodunovStableDt(bool muscl, int rank, double gamma, int guess, int max_it,
                                       double tol, const float* mlp, const double* states,
                                       BoxDesc cbox, int window_rule, int dir,
                                       unsigned long long* smax, cudaStream_t s) {
  const int w = muscl ? 2 : 1;
  BoxDesc wbox = cbox;
  wbox.n[dir] -= (window_rule == 0) ? 2 * w : 2 * w - 1;
  if (wbox.n[dir] <= 0) return cudaSuccess;
  const int64_t nwin = int64_t(wbox.n[0]) * wbox.n[1] * wbox.n[2];
  const int block = 128;
  const unsigned grid = static_cast<unsigned>((nwin + block - 1) / block);
  const GodunovGas g{{gamma, 1.0 / (gamma - 1.0)}, {guess, max_it, tol, mlp}};
  const GView st{states, cbox};
  switch (rank) {
  case 1:
    PatchGodunovDtKernel<1><<<grid, block, 0, s>>>(w, g, st, wbox, dir, smax);
    break;
  case 2:
    PatchGodunovDtKernel<2><<<grid, block, 0, s>>>(w, g, st, wbox, dir, smax);
    break;
  default:
    PatchGodunovDtKernel<3><<<grid, block, 0, s>>>(w, g, st, wbox, dir, smax);
    break;
  }
  return cudaGetLastError();
}

cudaError_t LaunchExactStar(int64_t n, double gamma, int guess, int max_it, double tol,
                            const float* mlp, const double* rhoL, const double* uL,
                            const double* pL, const double* rhoR, const double* uR,
                            const double* pR, double* pstar, double* ustar, int* iters,
                            int* converged, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int block = 128;
  const unsigned grid = static_cast<unsigned>((n + block - 1) / block);
  const GodunovGas g{{gamma, 1.0 / (gamma - 1.0)}, {guess, max_it, tol, mlp}};
  ExactStarKernel<1><<<grid, block, 0, s>>>(n, g, rhoL, uL, pL, rhoR, uR, pR, pstar, ustar, iters,
                                            converged);
  return cudaGetLastError();
}

}  // namespace fvs
