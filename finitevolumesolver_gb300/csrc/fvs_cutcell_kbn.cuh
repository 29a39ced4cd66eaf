// fvs_cutcell_kbn.cuh -- the KBN h-box cut-cell physics and kernels (2-D),
// generic over the arithmetic type T of the reconstruction, fluxes and wave
// speeds:
//   T = double in a -fmad=false translation unit: the exact flavour, bit for
//     bit the CPU oracle's restatement of the reference;
//   T = double with FMA contraction and the refined reciprocals and
//     reciprocal square roots of fvs_physics_fast.cuh (math policy CcFast):
//     the fast FP64 flavour, within 1e-12 of the exact one;
//   T = float: the mixed flavour -- masked MUSCL-Hancock, HLL/Einfeldt,
//     boundary (wall) states and CFL speeds in FP32; the state, the face
//     fractions, the h-box flux combination and the cut-cell update in FP64.
//
// Reference (maikel/FiniteVolumeSolver):
//   KbnCutCellMethod           include/fub/cutcell_method/KbnStabilisation.hpp:188-450
//   ComputeStableFluxes_Row    src/cutcell_method/KbnStabilisation.cpp:55-105
//   UpdateConservatively_Row   src/AMReX/cutcell/TimeIntegrator.cpp:65-221
//   masked MusclHancock / Hll / Einfeldt / Flux / CompleteFromCons
//       include/fub/flux_method/MusclHancockMethod.hpp:487-571,
//       include/fub/flux_method/HllMethod.hpp:295-365,
//       src/equations/perfect_gas/EinfeldtSignalVelocities.hpp:99-142,
//       src/equations/PerfectGas.cpp:79-93, 126-144
//   HllBase::SolveRiemannProblem (boundary solver)  include/fub/flux_method/HllMethod.hpp:161-184
//   MakeRotation, Reflect      include/fub/ext/Eigen.hpp:104-115, src/equations/PerfectGas.cpp:240-252
#pragma once

#include "fvs_convert.cuh"
#include "fvs_cutcell.h"
#include "fvs_internal.h"
#include "fvs_physics_exact.cuh"
#include "fvs_sweep.cuh"

namespace fvs {
namespace cc {

// Arithmetic of the physics below: IEEE quotients and square roots (CcIeee:
// the exact flavour, and FP32 for the mixed one) or the fast FP64 flavour's
// (CcFast: quotients as products with a reciprocal refined from the
// rcp.approx seed, square roots as a times its refined reciprocal square
// root; each within 2 ulp; the square root of a non-positive number is 0).
// The policy is a template argument of every kernel and launcher, so the
// exact and the fast FP64 instantiations, compiled with different flags in
// different translation units, never share a symbol.
struct CcIeee {
  static constexpr bool kFast = false;
  template <class T> static __device__ __forceinline__ T Div(T a, T b) { return a / b; }
  template <class T> static __device__ __forceinline__ T Sqrt(T a) { return sqrt(a); }
};
struct CcFast {
  static constexpr bool kFast = true;
  static __device__ __forceinline__ double Div(double a, double b) {
    return fast::Math<double>::Div(a, b);
  }
  static __device__ __forceinline__ double Rcp(double a) { return fast::Math<double>::Rcp(a); }
  static __device__ __forceinline__ double Sqrt(double a) { return fast::Math<double>::Sqrt(a); }
};

template <class T, class M = CcIeee> struct GasT {
  T gamma;
  T gamma_minus_1_inv;
  T gm1;  // gamma - 1 (fast flavour: p = e_int * (gamma - 1))
};

template <class T> struct C2T {
  T rho;
  T m[2];
  T E;
  T p;
  T c;
};

template <class T> __device__ __forceinline__ T PMinT(T a, T b) { return a < b ? a : b; }
template <class T> __device__ __forceinline__ T PMaxT(T a, T b) { return a > b ? a : b; }

template <class T, class M = CcIeee> __device__ __forceinline__ GasT<T, M> MakeGasT(double gamma) {
  GasT<T, M> g;
  g.gamma = T(gamma);
  g.gamma_minus_1_inv = T(1.0 / (gamma - 1.0));
  g.gm1 = T(gamma - 1.0);
  return g;
}

// PerfectGas<2>::CompleteFromCons (PerfectGas.cpp:96-110): e_kin = 0.5 |m|^2
// / rho, p = (E - e_kin) / gamma_minus_1_inv, c = sqrt(gamma p / rho).
template <class T, class M>
__device__ __forceinline__ void CompleteT(const GasT<T, M>& eq, C2T<T>& q, const T* u) {
  q.rho = u[0];
  q.m[0] = u[1];
  q.m[1] = u[2];
  q.E = u[3];
  if constexpr (M::kFast) {
    const T ir = M::Rcp(q.rho);
    const T e_kin = T(0.5) * (q.m[0] * q.m[0] + q.m[1] * q.m[1]) * ir;
    q.p = (q.E - e_kin) * eq.gm1;
    q.c = M::Sqrt(eq.gamma * q.p * ir);
  } else {
    const T e_kin = T(0.5) * (q.m[0] * q.m[0] + q.m[1] * q.m[1]) / q.rho;
    const T e_int = q.E - e_kin;
    q.p = e_int / eq.gamma_minus_1_inv;
    q.c = sqrt(eq.gamma * q.p / q.rho);
  }
}

// PerfectGas<2>::Flux (PerfectGas.cpp:52-64).
template <class M, class T> __device__ __forceinline__ void FluxT(T* f, const C2T<T>& q, int dir) {
  const T velocity = M::Div(q.m[dir], q.rho);
  f[0] = q.m[dir];
  f[1] = velocity * q.m[0];
  f[2] = velocity * q.m[1];
  f[1 + dir] += q.p;
  f[3] = velocity * (q.E + q.p);
}

// EinfeldtSignalVelocities (scalar, EinfeldtSignalVelocities.hpp:25-62).
template <class T, class M>
__device__ __forceinline__ void EinfeldtT(const GasT<T, M>& eq, const C2T<T>& L,
                                          const C2T<T>& R, int dir, T& sL, T& sR) {
  const T rhoL = L.rho;
  const T rhoR = R.rho;
  const T sqRhoL = M::Sqrt(rhoL);
  const T sqRhoR = M::Sqrt(rhoR);
  const T oosqRhoSum = M::Div(T(1), sqRhoL + sqRhoR);
  const T uL = M::Div(L.m[dir], rhoL);
  const T uR = M::Div(R.m[dir], rhoR);
  const T roeU = (uL * sqRhoL + uR * sqRhoR) * oosqRhoSum;
  const T hL = M::Div(L.E + L.p, rhoL);
  const T hR = M::Div(R.E + R.p, rhoR);
  const T roeH = (hL * sqRhoL + hR * sqRhoR) * oosqRhoSum;
  const T roeA2 = (eq.gamma - T(1)) * (roeH - T(0.5) * roeU * roeU);
  const T roeA = M::Sqrt(roeA2);
  sL = PMinT(uL - L.c, roeU - roeA);
  sR = PMaxT(roeU + roeA, uR + R.c);
}

// CompleteFromCons masked by `mask && rho > 0` (PerfectGas.cpp:126-144).
template <class T, class M>
__device__ __forceinline__ void CompleteMasked(const GasT<T, M>& eq, C2T<T>& q, const T* u,
                                               bool mask) {
  if (!(mask && u[0] > T(0))) {
    q.rho = T(0);
    q.m[0] = T(0);
    q.m[1] = T(0);
    q.E = T(0);
    q.p = T(0);
    q.c = T(0);
    return;
  }
  CompleteT(eq, q, u);
}

// Flux masked by `rho > 0` (PerfectGas.cpp:79-93, mask true).
template <class M, class T>
__device__ __forceinline__ void FluxMasked(T* f, const C2T<T>& q, int dir) {
  const T rho = (q.rho > T(0)) ? q.rho : T(1);
  const T velocity = M::Div(q.m[dir], rho);
  f[0] = q.m[dir];
  f[1] = velocity * q.m[0];
  f[2] = velocity * q.m[1];
  f[1 + dir] += q.p;
  f[3] = velocity * (q.E + q.p);
}

// Masked Einfeldt speeds with mask true (EinfeldtSignalVelocities.hpp:99-142).
template <class T, class M>
__device__ __forceinline__ void EinfeldtMasked(const GasT<T, M>& eq, const C2T<T>& L,
                                               const C2T<T>& R, int dir, T& sL, T& sR) {
  const T rhoL = L.rho, rhoR = R.rho;
  const T sqRhoL = M::Sqrt(rhoL);
  const T sqRhoR = M::Sqrt(rhoR);
  const T sqRho = sqRhoL + sqRhoR;
  T uL, uR, wL, wR, hL, hR;
  if constexpr (M::kFast) {
    const T irL = M::Rcp(rhoL), irR = M::Rcp(rhoR), iw = M::Rcp(sqRho);
    uL = L.m[dir] * irL;
    uR = R.m[dir] * irR;
    wL = sqRhoL * iw;
    wR = sqRhoR * iw;
    hL = (L.E + L.p) * irL;
    hR = (R.E + R.p) * irR;
  } else {
    uL = L.m[dir] / rhoL;
    uR = R.m[dir] / rhoR;
    wL = sqRhoL / sqRho;
    wR = sqRhoR / sqRho;
    hL = (L.E + L.p) / rhoL;
    hR = (R.E + R.p) / rhoR;
  }
  const T roeU = uL * wL + uR * wR;
  const T roeH = hL * wL + hR * wR;
  const T roeA2 = (eq.gamma - T(1)) * (roeH - T(0.5) * roeU * roeU);
  const T roeA = M::Sqrt(roeA2);
  sL = PMinT(uL - L.c, roeU - roeA);
  sR = PMaxT(roeU + roeA, uR + R.c);
}

// Masked MUSCL-Hancock predictor of one cell (both face states); the slope
// is zeroed unless the three cells of its window have volume.
template <class T, class M>
__device__ __forceinline__ void PredictMasked(const GasT<T, M>& eq, C2T<T>& recL, C2T<T>& recR,
                                              const T* q0, const T* q1, const T* q2, bool smask,
                                              int limiter, T lambda_half, int dir) {
  T uL[4], uR[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const T sL = smask ? q1[k] - q0[k] : T(0);
    const T sR = smask ? q2[k] - q1[k] : T(0);
    T slope;
    if (limiter == exact::kVanLeer) {
      const T c = T(2) * sL * sR;
      slope = (c > T(0)) ? M::Div(c, sL + sR) : T(0);
    } else if (limiter == exact::kMinMod) {
      slope = (sR > 0) ? PMaxT(T(0), PMinT(sL, sR)) : PMinT(T(0), PMaxT(sL, sR));
    } else {
      slope = T(0);
    }
    uL[k] = q1[k] - T(0.5) * slope;
    uR[k] = q1[k] + T(0.5) * slope;
  }
  C2T<T> qL, qR;
  CompleteMasked(eq, qL, uL, true);
  CompleteMasked(eq, qR, uR, true);
  T fL[4], fR[4];
  FluxMasked<M>(fL, qL, dir);
  FluxMasked<M>(fR, qR, dir);
  T a[4], b[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const T df = fL[k] - fR[k];
    b[k] = uR[k] + lambda_half * df;
    a[k] = uL[k] + lambda_half * df;
  }
  CompleteMasked(eq, recR, b, true);
  CompleteMasked(eq, recL, a, true);
}

// Masked HLL flux of a face with beta > 0 (HllMethod.hpp:295-335).
template <class T, class M>
__device__ __forceinline__ void HllMasked(const GasT<T, M>& eq, T* nf, const C2T<T>& L,
                                          const C2T<T>& R, int dir) {
  T s0, s1;
  EinfeldtMasked(eq, L, R, dir, s0, s1);
  T fL[4], fR[4];
  FluxMasked<M>(fL, L, dir);
  FluxMasked<M>(fR, R, dir);
  const T qL[4] = {L.rho, L.m[0], L.m[1], L.E};
  const T qR[4] = {R.rho, R.m[0], R.m[1], R.E};
  const T sL = PMinT(s0, T(0));
  const T sR = PMaxT(s1, T(0));
  const T sLsR = sL * sR;
  const T ds = sR - sL;
  if constexpr (M::kFast) {
    const T ids = M::Rcp(ds);
#pragma unroll
    for (int k = 0; k < 4; ++k) nf[k] = (sR * fL[k] - sL * fR[k] + sLsR * (qR[k] - qL[k])) * ids;
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) nf[k] = (sR * fL[k] - sL * fR[k] + sLsR * (qR[k] - qL[k])) / ds;
  }
}

// HllBase::SolveRiemannProblem (scalar, HllMethod.hpp:161-184), direction x.
template <class T, class M>
__device__ __forceinline__ void HllRiemannState(const GasT<T, M>& eq, C2T<T>& sol,
                                                const C2T<T>& L, const C2T<T>& R) {
  T sL, sR;
  EinfeldtT(eq, L, R, 0, sL, sR);
  T fL[4], fR[4];
  FluxT<M>(fL, L, 0);
  FluxT<M>(fR, R, 0);
  const T qL[4] = {L.rho, L.m[0], L.m[1], L.E};
  const T qR[4] = {R.rho, R.m[0], R.m[1], R.E};
  const T ds = sL != sR ? sR - sL : T(1);
  if (T(0) < sL) {
    sol = L;
  } else if (sR < T(0)) {
    sol = R;
  } else {
    T u[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) u[k] = M::Div(sR * qR[k] - sL * qL[k] + fL[k] - fR[k], ds);
    CompleteT(eq, sol, u);
  }
}

// Rotation taking unit vector a to b applied to the momentum (MakeRotation).
template <class T>
__device__ __forceinline__ void RotateMomentum(C2T<T>& q, T a0, T a1, T b0, T b1) {
  if (a0 == -b0 && a1 == -b1) {
    q.m[0] = -q.m[0];
    q.m[1] = -q.m[1];
    return;
  }
  const T s = a0 * b1 - a1 * b0;
  const T c = a0 * b0 + a1 * b1;
  const T m0 = q.m[0], m1 = q.m[1];
  q.m[0] = c * m0 + (-s) * m1;
  q.m[1] = s * m0 + c * m1;
}

// Wall state: HLL solution of (reflected | state) in the frame of the
// boundary normal, rotated back (KbnStabilisation.hpp:188-210, 229-238).
template <class T, class M>
__device__ __forceinline__ C2T<T> WallSolution(const GasT<T, M>& eq, const C2T<T>& state, T n0,
                                               T n1) {
  C2T<T> rot = state;
  RotateMomentum(rot, n0, n1, T(1), T(0));
  C2T<T> refl = rot;
  const T dot = rot.m[0] * T(1) + rot.m[1] * T(0);
  const T p0 = dot * T(1), p1 = dot * T(0);
  refl.m[0] = rot.m[0] - 2 * p0;
  refl.m[1] = rot.m[1] - 2 * p1;
  C2T<T> sol;
  HllRiemannState(eq, sol, refl, rot);
  RotateMomentum(sol, T(1), T(0), n0, n1);
  return sol;
}

__device__ __forceinline__ double Clamp01(double x) {
  x = x < 0.0 ? 0.0 : x;
  return 1.0 < x ? 1.0 : x;
}

__device__ __forceinline__ void LoadCons(const CcStateArgs& a, int i, int j, double* u) {
  const int si = BcIndex(i, a.g.nx, a.bc[0]);
  const int sj = BcIndex(j, a.g.ny, a.bc[1]);
  const int64_t cs = int64_t(a.g.nx) * a.g.ny;
  const int64_t off = int64_t(sj) * a.g.nx + si;
#pragma unroll
  for (int k = 0; k < 4; ++k) u[k] = __ldg(a.in + k * cs + off);
}

template <class T> __device__ __forceinline__ void Narrow(T* t, const double* u) {
#pragma unroll
  for (int k = 0; k < 4; ++k) t[k] = NarrowTo<T>(u[k]);
}

// KbnCutCellMethod::PreAdvanceHierarchy for the cut cells of [-1, n+1)^2.
template <class T, class M> __global__ void ReferenceStatesKernel(CcStateArgs a) {
  const int w = a.g.nx + 2, h = a.g.ny + 2;
  const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (id >= int64_t(w) * h) return;
  const int i = static_cast<int>(id % w) - 1, j = static_cast<int>(id / w) - 1;
  const int64_t c = a.g.CellIndex(i, j);
  if (!a.g.cut[c]) return;
  const GasT<T, M> eq = MakeGasT<T, M>(a.gamma);
  double ud[4];
  LoadCons(a, i, j, ud);
  T u[4];
  Narrow(u, ud);
  C2T<T> q;
  CompleteMasked(eq, q, u, a.g.alpha[c] > 0.0);
  const int64_t plane = int64_t(a.g.NX()) * a.g.NY();
  C2T<T> r;
  if (q.rho > T(0)) {
    r = WallSolution(eq, q, NarrowTo<T>(a.g.normal[c]), NarrowTo<T>(a.g.normal[plane + c]));
  } else {
    r = C2T<T>{T(0), {T(0), T(0)}, T(0), T(0), T(0)};
  }
  a.refs[c] = Widen(r.rho);
  a.refs[plane + c] = Widen(r.m[0]);
  a.refs[2 * plane + c] = Widen(r.m[1]);
  a.refs[3 * plane + c] = Widen(r.E);
  a.refs[4 * plane + c] = Widen(r.p);
  a.refs[5 * plane + c] = Widen(r.c);
}

// The fused KBN sweep over the cut tiles (CcGeom::band): one warp per tile,
// each thread marching the tile's cells of one grid line along `dir`,
// evaluating per cell the masked predictor and the boundary flux, per face
// the masked HLLE flux, the h-box stabilised fluxes and the CFL speed, and per
// cell the cut-cell update.  Blocks are one warp.
struct FaceData {
  double f[4], fs[4], fsL[4], fsR[4];
  double beta, us, sL, sR;
};

// False when the sweep must not run: the run was aborted or finished, or the
// previous sweep's CFL check failed.
__device__ __forceinline__ bool SweepGateCc(const CcSweepArgs& a, double split_dt) {
  if (a.ctrl) {
    if (a.ctrl->abort || a.ctrl->done) return false;
    if (a.prev_check >= 0) {
      const double smax = BitsToDouble(a.ctrl->smax_check[a.prev_check]);
      if (a.prev_dx / smax < split_dt) return false;
    }
  }
  return true;
}

template <class T, class M, int kMinBlocks>
__global__ void __launch_bounds__(128, kMinBlocks) KbnSweepKernel(CcSweepArgs a) {
  const CcGeom& g = a.s.g;
  const int dir = a.dir;
  const int nd = dir == 0 ? g.nx : g.ny;
  const int nt = dir == 0 ? g.ny : g.nx;
  // the warp's tile; warps beyond the list only join the block reduction
  const int slot = static_cast<int>(blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5));
  const bool has_tile = slot < g.nband[dir];
  const int tile_id = has_tile ? g.band[dir][slot] : 0;
  const int group = tile_id / g.NTiles(dir), tile = tile_id % g.NTiles(dir);
  const int64_t t64 = has_tile ? int64_t(group) * 32 + (threadIdx.x & 31) : int64_t(nt);
  const int j0 = tile * kCcTile;
  const int j1 = min(nd, j0 + kCcTile);
  const double split_dt = a.dt_ptr ? a.dt_scale * (*a.dt_ptr) : a.dt_value;
  if (!BlockAll(SweepGateCc(a, split_dt))) return;
  T smax = T(0);
  int status = 0;
  // CFL speeds: none in a step's first sweep (skip_cfl: the stable-dt pass
  // measured the same faces of the same state); in FP64 flavours screened in
  // FP32 as the uniform sweeps do (fvs_sweep.cuh, FilteredCfl), with the
  // masked states and faces of beta > 0
  constexpr bool kScreen = sizeof(T) == 8;
  const bool skip_cfl = kScreen && a.skip_cfl != 0;
  const bool screen = kScreen && a.s.gamma > 1.0 && a.s.gamma <= 2.0;
  const unsigned amask = __ballot_sync(0xffffffffu, t64 < nt);
  if (t64 < nt) {
    const int t = static_cast<int>(t64);
    const GasT<T, M> eq = MakeGasT<T, M>(a.s.gamma);
    const double dx = a.dx;
    const T lambda_half = NarrowTo<T>(0.5 * split_dt / dx);
    const double dt_dx = split_dt / dx;
    const int64_t plane = int64_t(g.NX()) * g.NY();
    const int64_t cs = int64_t(g.nx) * g.ny;
    auto cell_ij = [&](int c, int& i, int& j) {
      if (dir == 0) {
        i = c;
        j = t;
      } else {
        i = t;
        j = c;
      }
    };
    // masked complete state (alpha > 0 and rho > 0) of cell c
    auto load_cell = [&](int c, T* u, double& alpha) {
      int i, j;
      cell_ij(c, i, j);
      double vd[4];
      LoadCons(a.s, i, j, vd);
      T v[4];
      Narrow(v, vd);
      alpha = g.alpha[g.CellIndex(i, j)];
      C2T<T> q;
      CompleteMasked(eq, q, v, alpha > 0.0);
      u[0] = q.rho;
      u[1] = q.m[0];
      u[2] = q.m[1];
      u[3] = q.E;
    };
    // boundary flux of cell c (0 unless it is a cut cell)
    auto boundary_flux = [&](int c, const T* u, double* fb) {
      int i, j;
      cell_ij(c, i, j);
      const int64_t ci = g.CellIndex(i, j);
#pragma unroll
      for (int k = 0; k < 4; ++k) fb[k] = 0.0;
      if (!g.cut[ci]) return;
      C2T<T> ref;
      ref.rho = NarrowTo<T>(a.s.refs[ci]);
      ref.m[0] = NarrowTo<T>(a.s.refs[plane + ci]);
      ref.m[1] = NarrowTo<T>(a.s.refs[2 * plane + ci]);
      ref.E = NarrowTo<T>(a.s.refs[3 * plane + ci]);
      ref.p = NarrowTo<T>(a.s.refs[4 * plane + ci]);
      ref.c = NarrowTo<T>(a.s.refs[5 * plane + ci]);
      C2T<T> q;
      CompleteMasked(eq, q, u, g.alpha[ci] > 0.0);
      T f[4];
      FluxT<M>(f, ref, dir);
      const C2T<T> sol =
          WallSolution(eq, q, NarrowTo<T>(g.normal[ci]), NarrowTo<T>(g.normal[plane + ci]));
      f[1 + dir] += sol.p - ref.p;
#pragma unroll
      for (int k = 0; k < 4; ++k) fb[k] = Widen(f[k]);
    };
    auto center_of = [&](int c) {
      int i, j;
      cell_ij(c, i, j);
      return g.center[int64_t(dir) * plane + g.CellIndex(i, j)];
    };
    T um[4], uc[4], up[4];
    double am, ac, ap;
    load_cell(j0 - 2, um, am);
    load_cell(j0 - 1, uc, ac);
    C2T<T> recR_prev;
    double fb_prev[4];
    double xb_prev = 0.0;
    C2T<T> q_prev;
    FaceData F_prev;
    fast::Gas<float> g32;
    g32.gamma = static_cast<float>(a.s.gamma);
    g32.gm1 = static_cast<float>(a.s.gamma - 1.0);
    fast::Wave<float> v_prev{};
    bool ok_prev = false;
    bool have_prev = false;  // q_prev holds the complete state of cell j-1
    float thr = 0.0f;
    if (kScreen && !skip_cfl && a.smax_out)
      thr = CflFloatBelow(CflSync(a.smax_out, 0.0, amask));
    for (int j = j0 - 1; j <= j1; ++j) {
      load_cell(j + 1, up, ap);
      const bool smask = am > 0.0 && ac > 0.0 && ap > 0.0;
      C2T<T> recL, recR;
      PredictMasked(eq, recL, recR, um, uc, up, smask, a.limiter, lambda_half, dir);
      double fb[4];
      boundary_flux(j, uc, fb);
      const double xb = center_of(j);
      C2T<T> q;
      fast::Wave<float> v{};
      bool ok = false;
      if constexpr (kScreen) {
        if (!skip_cfl) {
          float c32[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) c32[k] = CflToF32(uc[k]);
          v = fast::MakeWave<2, float>(g32, c32, dir);
          ok = screen && CflInRange<2>(c32) && v.a > 0.0f;
        }
      } else {
        CompleteMasked(eq, q, uc, true);  // uc is already masked by alpha
      }
      if (j >= j0) {
        FaceData F;
        const int64_t fi = g.FaceIndex(dir, j, t);
        F.beta = g.beta[dir][fi];
        F.us = g.us[dir][fi];
        F.sL = g.sL[dir][fi];
        F.sR = g.sR[dir][fi];
        const double us_rel = g.us_rel[dir][fi];
        const double sL_rel = g.sL_rel[dir][fi];
        const double sR_rel = g.sR_rel[dir][fi];
        if constexpr (kScreen) {
          if (!skip_cfl) {
            bool need = false;
            if (F.beta > 0.0) {
              const float s32 = fast::FaceMaxSpeed<float>(g32, v_prev, v);
              const float sh = fast::Math<float>::Sqrt(fmaxf(v_prev.h, v.h));
              need = !(ok && ok_prev && fmaf(s32, kCflRel, fmaf(kCflScale, sh, kCflAbs)) < thr);
            }
            if (__any_sync(amask, need)) {
              // the whole warp evaluates (the same instructions as some lanes)
              if (!have_prev) CompleteMasked(eq, q_prev, um, true);
              CompleteMasked(eq, q, uc, true);
              if (F.beta > 0.0) {
                T s0, s1;
                EinfeldtMasked(eq, q_prev, q, dir, s0, s1);
                const T mx = PMaxT(PMaxT(T(0), fabs(s0)), fabs(s1));
                smax = mx > smax ? mx : smax;
              }
              thr = fmaxf(thr, CflFloatBelow(static_cast<double>(smax)));
              q_prev = q;
              have_prev = true;
            } else {
              have_prev = false;
            }
            if (a.smax_out && ((j - j0) % kCflSyncRows) == kCflSyncRows - 1)
              thr = fmaxf(thr, CflFloatBelow(CflSync(a.smax_out, static_cast<double>(smax),
                                                     amask)));
          }
        }
        if (F.beta > 0.0) {
          T f[4];
          HllMasked(eq, f, recR_prev, recL, dir);
#pragma unroll
          for (int k = 0; k < 4; ++k) F.f[k] = Widen(f[k]);
          if constexpr (!kScreen) {
            T s0, s1;
            EinfeldtMasked(eq, q_prev, q, dir, s0, s1);
            const T mx = PMaxT(PMaxT(T(0), fabs(s0)), fabs(s1));
            smax = mx > smax ? mx : smax;
          }
        } else {
#pragma unroll
          for (int k = 0; k < 4; ++k) F.f[k] = 0.0;
        }
        const double dL = Clamp01(0.5 - xb_prev);
        const double dR = Clamp01(0.5 + xb);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const double fk = F.f[k];
          const double sLk = dL * fk + (1.0 - dL) * fb_prev[k];
          const double sRk = dR * fk + (1.0 - dR) * fb[k];
          F.fsL[k] = sLk;
          F.fsR[k] = sRk;
          F.fs[k] = us_rel * fk + sL_rel * sLk + sR_rel * sRk;
        }
        if (j > j0) {
          // cut-cell update of cell j-1 (faces j-1 and j)
          const int c = j - 1;
          int i, jj;
          cell_ij(c, i, jj);
          const int64_t out = int64_t(jj) * g.nx + i;
          const double alpha = am;  // alpha of cell j-1
          const double betaL = F_prev.beta, betaR = F.beta;
          const double center = xb_prev;
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            double next;
            if (alpha == 0.0) {
              next = 0.0;
            } else {
              const double prev = __ldg(a.s.in + k * cs + out);
              const double fLs = F_prev.fs[k], fRs = F.fs[k];
              const double fLu = F_prev.f[k], fRu = F.f[k];
              if (betaL == betaR) {
                next = prev + dt_dx * (fLs - fRs);
              } else if (betaL > betaR) {
                const double bus = F_prev.us / alpha;
                const double bsL = F_prev.sL / alpha;
                const double dist = 0.5 + center;
                const double dBeta = Clamp01((F_prev.sR * dist) / alpha);
                const double dF_us = fLu - fRs;
                const double dF_sL = F_prev.fsL[k] - fRs;
                const double dB = fLu - fb_prev[k];
                next = prev + dt_dx * bus * dF_us + dt_dx * bsL * dF_sL + dt_dx * dBeta * dB;
              } else {
                const double bus = F.us / alpha;
                const double bsR = F.sR / alpha;
                const double dist = 0.5 - center;
                const double dBeta = Clamp01((F.sL * dist) / alpha);
                const double dF_us = fLs - fRu;
                const double dF_sR = fLs - F.fsR[k];
                const double dB = fb_prev[k] - fRu;
                next = prev + dt_dx * bus * dF_us + dt_dx * bsR * dF_sR + dt_dx * dBeta * dB;
              }
            }
            a.out[k * cs + out] = next;
          }
          if (alpha > 0.0 && __double_as_longlong(a.out[out]) <= 0)
            status |= kStatusNonPositiveDensity;
        }
        F_prev = F;
      }
      recR_prev = recR;
#pragma unroll
      for (int k = 0; k < 4; ++k) fb_prev[k] = fb[k];
      xb_prev = xb;
      if constexpr (!kScreen) q_prev = q;
      ok_prev = ok;
      v_prev = v;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        um[k] = uc[k];
        uc[k] = up[k];
      }
      am = ac;
      ac = ap;
    }
  }
  const double smax_d = static_cast<double>(smax);
  BlockMaxAtomic<1>(a.smax_out, &smax_d);
  if (status && a.ctrl) atomicOr(&a.ctrl->step_status, status);
}

// The regular and covered tiles of a KBN sweep (CcTileClass).  On a regular
// tile the KBN arithmetic reduces, bit for bit, to the masked MUSCL-Hancock
// predictor and masked HLL flux with every mask true, the stabilised flux
// us_rel f + sL_rel fsL + sR_rel fsR = 1 f + 0 fsL + 0 fsR = f + 0 (for every
// finite f; the + 0 turns a -0 into +0 as the zero terms do), and the update
// U + dt/dx (fs_L - fs_R) of cells with equal face fractions
// (src/AMReX/cutcell/TimeIntegrator.cpp:65-221): the kernel evaluates exactly
// that, from the same inline functions, and reads no geometry.  A covered
// tile's cells are 0 and its faces (beta 0) add no CFL speed.  Each thread
// marches the runs of consecutive regular tiles of its segment of one grid
// line; the tile class is the warp's, so the control flow is warp-uniform.
template <class T, class M, int kMinBlocks>
__global__ void __launch_bounds__(128, kMinBlocks) KbnRegularSweepKernel(CcSweepArgs a) {
  const CcGeom& g = a.s.g;
  const int dir = a.dir;
  const int nd = dir == 0 ? g.nx : g.ny;
  const int nt = dir == 0 ? g.ny : g.nx;
  const int64_t t64 = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int group = static_cast<int>(t64 >> 5);
  const int s0 = blockIdx.y * a.seg_len;  // a multiple of kCcTile
  const int s1 = min(nd, s0 + a.seg_len);
  const double split_dt = a.dt_ptr ? a.dt_scale * (*a.dt_ptr) : a.dt_value;
  if (!BlockAll(SweepGateCc(a, split_dt))) return;
  T smax = T(0);
  int status = 0;
  constexpr bool kScreen = sizeof(T) == 8;
  const bool skip_cfl = kScreen && a.skip_cfl != 0;
  const bool screen = kScreen && a.s.gamma > 1.0 && a.s.gamma <= 2.0;
  const unsigned amask = __ballot_sync(0xffffffffu, t64 < nt);
  if (t64 < nt) {
    const int t = static_cast<int>(t64);
    const GasT<T, M> eq = MakeGasT<T, M>(a.s.gamma);
    const T lambda_half = NarrowTo<T>(0.5 * split_dt / a.dx);
    const double dt_dx = split_dt / a.dx;
    const int64_t cs = int64_t(g.nx) * g.ny;
    const int ntl = g.NTiles(dir);
    const signed char* cls = g.tile_class[dir] + int64_t(group) * ntl;
    auto offset = [&](int c) {
      return dir == 0 ? int64_t(t) * g.nx + c : int64_t(c) * g.nx + t;
    };
    // masked state of cell c (alpha 1: zeroed only where rho <= 0)
    auto load_cell = [&](int c, T* u) {
      double vd[4];
      if (dir == 0)
        LoadCons(a.s, c, t, vd);
      else
        LoadCons(a.s, t, c, vd);
      T v[4];
      Narrow(v, vd);
      C2T<T> q;
      CompleteMasked(eq, q, v, true);
      u[0] = q.rho;
      u[1] = q.m[0];
      u[2] = q.m[1];
      u[3] = q.E;
    };
    fast::Gas<float> g32;
    g32.gamma = static_cast<float>(a.s.gamma);
    g32.gm1 = static_cast<float>(a.s.gamma - 1.0);
    float thr = 0.0f;
    if (kScreen && !skip_cfl && a.smax_out)
      thr = CflFloatBelow(CflSync(a.smax_out, 0.0, amask));
    int rows = 0;  // faces since the last publication of the warp's maximum
    const int tile_end = (s1 + kCcTile - 1) / kCcTile;
    int tile = s0 / kCcTile;
    while (tile < tile_end) {
      const int k = cls[tile];
      if (k == kCcCut) {
        ++tile;
        continue;
      }
      if (k == kCcCovered) {
        const int c1 = min(nd, (tile + 1) * kCcTile);
        for (int c = tile * kCcTile; c < c1; ++c) {
          const int64_t o = offset(c);
#pragma unroll
          for (int q = 0; q < 4; ++q) a.out[q * cs + o] = 0.0;
        }
        ++tile;
        continue;
      }
      int r1 = tile + 1;
      while (r1 < tile_end && cls[r1] == kCcRegular) ++r1;
      const int j0 = tile * kCcTile, j1 = min(nd, r1 * kCcTile);
      tile = r1;
      // march the run [j0, j1): faces j0 .. j1, cells j0 .. j1-1
      T um[4], uc[4], up[4];
      load_cell(j0 - 2, um);
      load_cell(j0 - 1, uc);
      C2T<T> recR_prev, q_prev;
      double fs_prev[4];
      fast::Wave<float> v_prev{};
      bool ok_prev = false;
      bool have_prev = false;
      for (int j = j0 - 1; j <= j1; ++j) {
        load_cell(j + 1, up);
        C2T<T> recL, recR;
        PredictMasked(eq, recL, recR, um, uc, up, true, a.limiter, lambda_half, dir);
        C2T<T> q;
        fast::Wave<float> v{};
        bool ok = false;
        if constexpr (kScreen) {
          if (!skip_cfl) {
            float c32[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) c32[c] = CflToF32(uc[c]);
            v = fast::MakeWave<2, float>(g32, c32, dir);
            ok = screen && CflInRange<2>(c32) && v.a > 0.0f;
          }
        } else {
          CompleteMasked(eq, q, uc, true);
        }
        if (j >= j0) {
          if constexpr (kScreen) {
            if (!skip_cfl) {
              const float s32 = fast::FaceMaxSpeed<float>(g32, v_prev, v);
              const float sh = fast::Math<float>::Sqrt(fmaxf(v_prev.h, v.h));
              const bool need =
                  !(ok && ok_prev && fmaf(s32, kCflRel, fmaf(kCflScale, sh, kCflAbs)) < thr);
              if (__any_sync(amask, need)) {
                if (!have_prev) CompleteMasked(eq, q_prev, um, true);
                CompleteMasked(eq, q, uc, true);
                T s0w, s1w;
                EinfeldtMasked(eq, q_prev, q, dir, s0w, s1w);
                const T mx = PMaxT(PMaxT(T(0), fabs(s0w)), fabs(s1w));
                smax = mx > smax ? mx : smax;
                thr = fmaxf(thr, CflFloatBelow(static_cast<double>(smax)));
                q_prev = q;
                have_prev = true;
              } else {
                have_prev = false;
              }
              if (a.smax_out && ++rows == kCflSyncRows) {
                rows = 0;
                thr = fmaxf(thr, CflFloatBelow(CflSync(a.smax_out, static_cast<double>(smax),
                                                       amask)));
              }
            }
          }
          T f[4];
          HllMasked(eq, f, recR_prev, recL, dir);
          double fs[4];
#pragma unroll
          for (int c = 0; c < 4; ++c) fs[c] = Widen(f[c]) + 0.0;
          if constexpr (!kScreen) {
            T s0w, s1w;
            EinfeldtMasked(eq, q_prev, q, dir, s0w, s1w);
            const T mx = PMaxT(PMaxT(T(0), fabs(s0w)), fabs(s1w));
            smax = mx > smax ? mx : smax;
          }
          if (j > j0) {
            const int64_t o = offset(j - 1);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              const double prev = __ldg(a.s.in + c * cs + o);
              a.out[c * cs + o] = prev + dt_dx * (fs_prev[c] - fs[c]);
            }
            if (__double_as_longlong(a.out[o]) <= 0) status |= kStatusNonPositiveDensity;
          }
#pragma unroll
          for (int c = 0; c < 4; ++c) fs_prev[c] = fs[c];
        }
        recR_prev = recR;
        if constexpr (!kScreen) q_prev = q;
        ok_prev = ok;
        v_prev = v;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          um[c] = uc[c];
          uc[c] = up[c];
        }
      }
    }
  }
  const double smax_d = static_cast<double>(smax);
  BlockMaxAtomic<1>(a.smax_out, &smax_d);
  if (status && a.ctrl) atomicOr(&a.ctrl->step_status, status);
}

// Masked stable dt over both directions: faces 0..n with beta > 0
// (KbnStabilisation.hpp:275-345).
template <class T, class M>
__global__ void KbnStableDtKernel(CcStateArgs a, unsigned long long* smax_out, Control* ctrl) {
  if (!BlockAll(!(ctrl && (ctrl->abort || ctrl->done)))) return;
  const CcGeom& g = a.g;
  const int w = g.nx + 1, h = g.ny + 1;
  T sm[2] = {T(0), T(0)};
  // grid-stride over faces; one atomic per block and direction at the end
  for (int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; id < int64_t(w) * h;
       id += int64_t(gridDim.x) * blockDim.x) {
    const int i = static_cast<int>(id % w), j = static_cast<int>(id / w);
    const GasT<T, M> eq = MakeGasT<T, M>(a.gamma);
    for (int d = 0; d < 2; ++d) {
      const int f = d == 0 ? i : j;
      const int t = d == 0 ? j : i;
      const int nt = d == 0 ? g.ny : g.nx;
      if (t >= nt) continue;
      if (!(g.beta[d][g.FaceIndex(d, f, t)] > 0.0)) continue;
      const int il = d == 0 ? f - 1 : t, jl = d == 0 ? t : f - 1;
      const int ir = d == 0 ? f : t, jr = d == 0 ? t : f;
      double uld[4], urd[4];
      LoadCons(a, il, jl, uld);
      LoadCons(a, ir, jr, urd);
      T ul[4], ur[4];
      Narrow(ul, uld);
      Narrow(ur, urd);
      C2T<T> L, R;
      CompleteMasked(eq, L, ul, g.alpha[g.CellIndex(il, jl)] > 0.0);
      CompleteMasked(eq, R, ur, g.alpha[g.CellIndex(ir, jr)] > 0.0);
      T s0, s1;
      EinfeldtMasked(eq, L, R, d, s0, s1);
      const T mx = PMaxT(PMaxT(T(0), fabs(s0)), fabs(s1));
      sm[d] = mx > sm[d] ? mx : sm[d];
    }
  }
  const double smd[2] = {static_cast<double>(sm[0]), static_cast<double>(sm[1])};
  BlockMaxAtomic<2>(smax_out, smd);
}

template <class T, class M> cudaError_t LaunchKbnStates(const CcStateArgs& a, cudaStream_t s) {
  const int64_t n = int64_t(a.g.nx + 2) * (a.g.ny + 2);
  const int block = 128;
  ReferenceStatesKernel<T, M><<<unsigned((n + block - 1) / block), block, 0, s>>>(a);
  return cudaGetLastError();
}

template <class T, class M>
cudaError_t LaunchKbnSweep(const CcSweepArgs& a, bool band, cudaStream_t s) {
  const int nd = a.dir == 0 ? a.s.g.nx : a.s.g.ny;
  const int nt = a.dir == 0 ? a.s.g.ny : a.s.g.nx;
  if (band) {
    // cut tiles: one warp each; register/occupancy variant: the default, or
    // compiled for 3 (FP64) / 4 (FP32) resident 128-thread blocks per SM
    // (spilling a little)
    const int n = a.s.g.nband[a.dir];
    if (n == 0) return cudaSuccess;
    constexpr int kMore = sizeof(T) == 4 ? 4 : 3;
    if (a.occupancy == kMore)
      KbnSweepKernel<T, M, kMore><<<unsigned(n), 32, 0, s>>>(a);
    else
      KbnSweepKernel<T, M, 1><<<unsigned(n), 32, 0, s>>>(a);
    return cudaGetLastError();
  }
  const int block = 128;
  int seg = a.seg_len > 0 ? a.seg_len : nd;
  seg = (seg + kCcTile - 1) / kCcTile * kCcTile;
  CcSweepArgs b = a;
  b.seg_len = seg;
  dim3 grid(unsigned((nt + block - 1) / block), unsigned((nd + seg - 1) / seg));
  KbnRegularSweepKernel<T, M, sizeof(T) == 4 ? 4 : 3><<<grid, block, 0, s>>>(b);
  return cudaGetLastError();
}

template <class T, class M>
cudaError_t LaunchKbnStableDt(const CcStateArgs& a, unsigned long long* smax_out, Control* ctrl,
                              cudaStream_t s) {
  const int64_t n = int64_t(a.g.nx + 1) * (a.g.ny + 1);
  const int block = 128;
  KbnStableDtKernel<T, M><<<GridStrideBlocks(n, block, 16), block, 0, s>>>(a, smax_out, ctrl);
  return cudaGetLastError();
}

}  // namespace cc
}  // namespace fvs
