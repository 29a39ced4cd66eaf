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

#include <algorithm>

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

// The mixed flavour's FP32 arithmetic: quotients as __fdividef, square roots
// as a times rsqrtf(a) (0 for a <= 0), as the uniform grid's mixed sweeps
// compute them (fvs_physics_fast.cuh, Math<float>); the FP32 rounding of the
// reconstruction dominates either way.
struct CcFast32 {
  static constexpr bool kFast = true;
  static __device__ __forceinline__ float Div(float a, float b) { return __fdividef(a, b); }
  static __device__ __forceinline__ float Rcp(float a) { return __fdividef(1.0f, a); }
  static __device__ __forceinline__ float Sqrt(float a) { return a > 0.0f ? a * rsqrtf(a) : 0.0f; }
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

// Component d of a 2-vector and f[1 + d] += x, for a run-time direction d:
// selects instead of indexing, so the arrays stay in registers (an indexed
// local array would live in local memory).
template <class T> __device__ __forceinline__ T Sel(const T (&m)[2], int d) {
  return d == 0 ? m[0] : m[1];
}
template <class T> __device__ __forceinline__ void AddMomentum(T* f, int d, T x) {
  if (d == 0)
    f[1] += x;
  else
    f[2] += x;
}

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
  const T velocity = M::Div(Sel(q.m, dir), q.rho);
  f[0] = Sel(q.m, dir);
  f[1] = velocity * q.m[0];
  f[2] = velocity * q.m[1];
  AddMomentum(f, dir, q.p);
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
  const T uL = M::Div(Sel(L.m, dir), rhoL);
  const T uR = M::Div(Sel(R.m, dir), rhoR);
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
  const T velocity = M::Div(Sel(q.m, dir), rho);
  f[0] = Sel(q.m, dir);
  f[1] = velocity * q.m[0];
  f[2] = velocity * q.m[1];
  AddMomentum(f, dir, q.p);
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
    uL = Sel(L.m, dir) * irL;
    uR = Sel(R.m, dir) * irR;
    wL = sqRhoL * iw;
    wR = sqRhoR * iw;
    hL = (L.E + L.p) * irL;
    hR = (R.E + R.p) * irR;
  } else {
    uL = Sel(L.m, dir) / rhoL;
    uR = Sel(R.m, dir) / rhoR;
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
    } else if (limiter == exact::kNoLimiter) {
      slope = T(0.5) * (sL + sR);
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

// Conservative state of cell (i, j), ghost cells the boundary condition's
// images.  A reflective ghost is the mirror cell's state with the momentum of
// its direction reflected, or zero where the mirror cell has no volume
// (cutcell::ReflectiveBoundary, include/fub/AMReX/cutcell/boundary_condition/
// ReflectiveBoundary.hpp:72-122; where the ghost cell itself has no volume
// the masked loads zero it).
// LoadCons without touching the loaded values: returns what the caller applies
// once they are needed (bit 0: negate m_x, bit 1: negate m_y, bit 2: zero
// the state -- a reflective image of a cell without volume), so that a
// prefetched load is not waited for at the load.
__device__ __forceinline__ int LoadConsDeferred(const CcStateArgs& a, int i, int j, double* u) {
  const int si = BcIndex(i, a.g.nx, a.bc[0]);
  const int sj = BcIndex(j, a.g.ny, a.bc[1]);
  const int64_t cs = int64_t(a.g.nx) * a.g.ny;
  const int64_t off = int64_t(sj) * a.g.nx + si;
#pragma unroll
  for (int k = 0; k < 4; ++k) u[k] = __ldg(a.in + k * cs + off);
  const bool fx = BcFlip(i, a.g.nx, a.bc[0]), fy = BcFlip(j, a.g.ny, a.bc[1]);
  int flags = (fx ? 1 : 0) | (fy ? 2 : 0);
  if ((fx || fy) && !(a.g.alpha[a.g.CellIndex(si, sj)] > 0.0)) flags |= 4;
  return flags;
}

template <class T> __device__ __forceinline__ void ApplyLoadFlags(T* u, int flags) {
  if (flags & 1) u[1] = -u[1];
  if (flags & 2) u[2] = -u[2];
  if (flags & 4) {
#pragma unroll
    for (int k = 0; k < 4; ++k) u[k] = T(0);
  }
}

__device__ __forceinline__ void LoadCons(const CcStateArgs& a, int i, int j, double* u) {
  const int si = BcIndex(i, a.g.nx, a.bc[0]);
  const int sj = BcIndex(j, a.g.ny, a.bc[1]);
  const int64_t cs = int64_t(a.g.nx) * a.g.ny;
  const int64_t off = int64_t(sj) * a.g.nx + si;
#pragma unroll
  for (int k = 0; k < 4; ++k) u[k] = __ldg(a.in + k * cs + off);
  const bool fx = BcFlip(i, a.g.nx, a.bc[0]), fy = BcFlip(j, a.g.ny, a.bc[1]);
  if (fx) u[1] = -u[1];
  if (fy) u[2] = -u[2];
  if ((fx || fy) && !(a.g.alpha[a.g.CellIndex(si, sj)] > 0.0)) {
#pragma unroll
    for (int k = 0; k < 4; ++k) u[k] = 0.0;
  }
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

// The per-sweep constants (dt / dx, the half-step factor, the gas) involve
// FP64 divisions, which cost tens of cycles of the narrow FP64 pipe; one
// thread of the block evaluates them and the sweep's gate, the others read
// them from shared memory after a barrier (`run` is block-uniform).
template <class T, class M> struct KbnConst {
  GasT<T, M> eq;
  T lambda_half;
  double dt_dx;
  int run;
};

template <class T, class M>
__device__ __forceinline__ const KbnConst<T, M>& KbnBlockConst(const CcSweepArgs& a) {
  __shared__ KbnConst<T, M> kc;
  if (threadIdx.x == 0) {
    const double split_dt = a.dt_ptr ? a.dt_scale * (*a.dt_ptr) : a.dt_value;
    kc.run = SweepGateCc(a, split_dt) ? 1 : 0;
    kc.eq = MakeGasT<T, M>(a.s.gamma);
    kc.lambda_half = NarrowTo<T>(0.5 * split_dt / a.dx);
    kc.dt_dx = split_dt / a.dx;
  }
  __syncthreads();
  return kc;
}

// One cell of a KBN sweep, evaluated on its own: cell j of grid line t gets
// the masked states of cells j-2 .. j+2, the masked MUSCL-Hancock predictors
// of cells j-1, j, j+1, the boundary fluxes and centroids of those three
// cells, the masked HLLE fluxes and h-box stabilised fluxes of its faces j and
// j+1, and the cut-cell update (KbnStabilisation.hpp:347-429,
// KbnStabilisation.cpp:55-105, TimeIntegrator.cpp:65-221).  Every quantity
// comes from the same inline functions on the same operands as in a sweep
// that marches the line, so the result is the same to the bit; a face is
// evaluated by both of its cells.  The CFL speed of face j (and of face j+1
// when `right_face`) is folded into smax unless `cfl` is false.
template <class T, class M>
__device__ __forceinline__ void KbnCell(const CcSweepArgs& a, int t, int j, bool right_face,
                                        bool cfl, const KbnConst<T, M>& kc, T& smax,
                                        int& status) {
  const CcGeom& g = a.s.g;
  const int dir = a.dir;
  const GasT<T, M> eq = kc.eq;
  const T lambda_half = kc.lambda_half;
  const double dt_dx = kc.dt_dx;
  const int64_t plane = int64_t(g.NX()) * g.NY();
  auto gcell = [&](int c) { return dir == 0 ? g.CellIndex(c, t) : g.CellIndex(t, c); };
  // masked states (alpha > 0 and rho > 0) of cells j-2 .. j+2
  T u[5][4];
  double al[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const int c = j - 2 + k;
    double vd[4];
    if (dir == 0)
      LoadCons(a.s, c, t, vd);
    else
      LoadCons(a.s, t, c, vd);
    T v[4];
    Narrow(v, vd);
    al[k] = g.alpha[gcell(c)];
    C2T<T> q;
    CompleteMasked(eq, q, v, al[k] > 0.0);
    u[k][0] = q.rho;
    u[k][1] = q.m[0];
    u[k][2] = q.m[1];
    u[k][3] = q.E;
  }
  // predictors of cells j-1 (its right state), j (both), j+1 (its left state)
  C2T<T> recLm, recRm, recL0, recR0, recLp, recRp;
  PredictMasked(eq, recLm, recRm, u[0], u[1], u[2], al[0] > 0.0 && al[1] > 0.0 && al[2] > 0.0,
                a.limiter, lambda_half, dir);
  PredictMasked(eq, recL0, recR0, u[1], u[2], u[3], al[1] > 0.0 && al[2] > 0.0 && al[3] > 0.0,
                a.limiter, lambda_half, dir);
  PredictMasked(eq, recLp, recRp, u[2], u[3], u[4], al[2] > 0.0 && al[3] > 0.0 && al[4] > 0.0,
                a.limiter, lambda_half, dir);
  // CFL speeds of faces j and j+1 from the masked states
  if (cfl) {
    C2T<T> qm, q0;
    CompleteMasked(eq, qm, u[1], true);
    CompleteMasked(eq, q0, u[2], true);
    if (g.beta[dir][g.FaceIndex(dir, j, t)] > 0.0) {
      T s0, s1;
      EinfeldtMasked(eq, qm, q0, dir, s0, s1);
      const T mx = PMaxT(PMaxT(T(0), fabs(s0)), fabs(s1));
      smax = mx > smax ? mx : smax;
    }
    if (right_face && g.beta[dir][g.FaceIndex(dir, j + 1, t)] > 0.0) {
      C2T<T> qp;
      CompleteMasked(eq, qp, u[3], true);
      T s0, s1;
      EinfeldtMasked(eq, q0, qp, dir, s0, s1);
      const T mx = PMaxT(PMaxT(T(0), fabs(s0)), fabs(s1));
      smax = mx > smax ? mx : smax;
    }
  }
  const int64_t cs = int64_t(g.nx) * g.ny;
  const int64_t out = dir == 0 ? int64_t(t) * g.nx + j : int64_t(j) * g.nx + t;
  // boundary flux of cell c (0 unless it is a cut cell), from its masked state
  auto boundary_flux = [&](int c, const T* uc, double* fb) {
    const int64_t ci = gcell(c);
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
    CompleteMasked(eq, q, uc, g.alpha[ci] > 0.0);
    T f[4];
    FluxT<M>(f, ref, dir);
    const C2T<T> sol =
        WallSolution(eq, q, NarrowTo<T>(g.normal[ci]), NarrowTo<T>(g.normal[plane + ci]));
    AddMomentum(f, dir, sol.p - ref.p);
#pragma unroll
    for (int k = 0; k < 4; ++k) fb[k] = Widen(f[k]);
  };
  double fbm[4], fb0[4], fbp[4];
  boundary_flux(j - 1, u[1], fbm);
  boundary_flux(j, u[2], fb0);
  boundary_flux(j + 1, u[3], fbp);
  const double xbm = g.center[int64_t(dir) * plane + gcell(j - 1)];
  const double xb0 = g.center[int64_t(dir) * plane + gcell(j)];
  const double xbp = g.center[int64_t(dir) * plane + gcell(j + 1)];
  // face data of face f between cells with boundary fluxes fbL, fbR and
  // centroids xbL, xbR (ComputeStableFluxComponents)
  auto face = [&](FaceData& F, int f, const C2T<T>& L, const C2T<T>& R, const double* fbL,
                  const double* fbR, double xbL, double xbR) {
    const int64_t fi = g.FaceIndex(dir, f, t);
    F.beta = g.beta[dir][fi];
    F.us = g.us[dir][fi];
    F.sL = g.sL[dir][fi];
    F.sR = g.sR[dir][fi];
    const double us_rel = g.us_rel[dir][fi];
    const double sL_rel = g.sL_rel[dir][fi];
    const double sR_rel = g.sR_rel[dir][fi];
    if (F.beta > 0.0) {
      T fl[4];
      HllMasked(eq, fl, L, R, dir);
#pragma unroll
      for (int k = 0; k < 4; ++k) F.f[k] = Widen(fl[k]);
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k) F.f[k] = 0.0;
    }
    const double dL = Clamp01(0.5 - xbL);
    const double dR = Clamp01(0.5 + xbR);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const double fk = F.f[k];
      const double sLk = dL * fk + (1.0 - dL) * fbL[k];
      const double sRk = dR * fk + (1.0 - dR) * fbR[k];
      F.fsL[k] = sLk;
      F.fsR[k] = sRk;
      F.fs[k] = us_rel * fk + sL_rel * sLk + sR_rel * sRk;
    }
  };
  FaceData Fl, Fr;
  face(Fl, j, recRm, recL0, fbm, fb0, xbm, xb0);
  face(Fr, j + 1, recR0, recLp, fb0, fbp, xb0, xbp);
  // UpdateConservatively_Row for cell j (faces j and j+1)
  const double alpha = al[2];
  const double betaL = Fl.beta, betaR = Fr.beta;
  const double center = xb0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    double next;
    if (alpha == 0.0) {
      next = 0.0;
    } else {
      const double prev = __ldg(a.s.in + k * cs + out);
      const double fLs = Fl.fs[k], fRs = Fr.fs[k];
      const double fLu = Fl.f[k], fRu = Fr.f[k];
      if (betaL == betaR) {
        next = prev + dt_dx * (fLs - fRs);
      } else if (betaL > betaR) {
        const double bus = Fl.us / alpha;
        const double bsL = Fl.sL / alpha;
        const double dist = 0.5 + center;
        const double dBeta = Clamp01((Fl.sR * dist) / alpha);
        const double dF_us = fLu - fRs;
        const double dF_sL = Fl.fsL[k] - fRs;
        const double dB = fLu - fb0[k];
        next = prev + dt_dx * bus * dF_us + dt_dx * bsL * dF_sL + dt_dx * dBeta * dB;
      } else {
        const double bus = Fr.us / alpha;
        const double bsR = Fr.sR / alpha;
        const double dist = 0.5 - center;
        const double dBeta = Clamp01((Fr.sL * dist) / alpha);
        const double dF_us = fLs - fRu;
        const double dF_sR = fLs - Fr.fsR[k];
        const double dB = fb0[k] - fRu;
        next = prev + dt_dx * bus * dF_us + dt_dx * bsR * dF_sR + dt_dx * dBeta * dB;
      }
    }
    a.out[k * cs + out] = next;
  }
  if (alpha > 0.0 && __double_as_longlong(a.out[out]) <= 0) status |= kStatusNonPositiveDensity;
}

// The band cells of a KBN sweep (CcGeom::band), one thread per cell
// (KbnCell, the full KBN arithmetic) with both of its faces' CFL speeds.  The
// FP64 flavours evaluate every CFL speed of the band (their screened sweeps
// give the same maximum), none in a step's first sweep.
template <class T, class M>
__global__ void __launch_bounds__(64, 1) KbnBandKernel(CcSweepArgs a) {
  const CcGeom& g = a.s.g;
  const int dir = a.dir;
  const KbnConst<T, M>& kc = KbnBlockConst<T, M>(a);
  if (!kc.run) return;  // block-uniform
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const bool cfl = !(sizeof(T) == 8 && a.skip_cfl != 0) && a.smax_out;
  T smax = T(0);
  int status = 0;
  if (k < g.nband[dir]) {
    const int id = g.band[dir][k];
    const int i = id % g.nx, jj = id / g.nx;
    KbnCell<T, M>(a, dir == 0 ? jj : i, dir == 0 ? i : jj, true, cfl, kc, smax, status);
  }
  const double smax_d = static_cast<double>(smax);
  BlockMaxAtomic<1>(a.smax_out, &smax_d);
  if (status && a.ctrl) atomicOr(&a.ctrl->step_status, status);
}

// Class of cell c of grid line t for sweeps in direction dir (CcCellClass);
// cells outside the interior count as band (neither written nor regular).
__device__ __forceinline__ int CellClassAt(const CcGeom& g, int dir, int t, int c) {
  const int nd = dir == 0 ? g.nx : g.ny;
  if (c < 0 || c >= nd) return kCcBand;
  const int64_t id = dir == 0 ? int64_t(t) * g.nx + c : int64_t(c) * g.nx + t;
  return g.cell_class[dir][id];
}

// The regular and covered cells of a mixed-precision KBN sweep, staged in
// shared memory.  A block takes 32 grid lines (one tile group) x 64 cells (8
// tiles) along the sweep direction: it loads the masked FP32 states of the
// cells and their 2-cell halos, and their classes, once (coalesced, one
// conversion per value; the x sweep's lanes run along x) into shared memory,
// then each warp marches one tile that holds a regular cell -- its lanes the
// 32 lines, each thread 8 cells -- from shared memory: masked MUSCL-Hancock
// + HLL with every mask true, f + 0 and U + dt/dx (fs_L - fs_R).  On a
// regular cell the KBN arithmetic is exactly this (the stabilised flux
// us_rel f + sL_rel fsL + sR_rel fsR = 1 f + 0 fsL + 0 fsR is f + 0 for
// every finite f; the + 0 turns a -0 into +0 as the zero terms do), and its
// stencil (cells j-2 .. j+2) holds only regular-valued data, so computing
// every cell of the tile this way and writing the regular ones is exact.
// Covered cells are written as 0; band cells are the band kernel's.  A
// face's CFL speed is counted here when one of its cells is regular.
//
// y sweeps update in the march (a warp's lanes hold 32 x-neighbouring
// cells: coalesced).  In x sweeps the lanes hold 32 rows, so the march
// stores its face fluxes in shared memory and, after a barrier, the block
// updates the tile with its threads along x: the re-read of the FP64 state,
// the stores and the class reads are coalesced.
constexpr int kTileLines = 32;
constexpr int kTileSegs = 8;                          // tiles per block
constexpr int kTileCells = kCcTile * kTileSegs;      // cells per block along dir
constexpr int kTileHalo = kTileCells + 4;            // with the 2-cell halos
constexpr int kTilePitch = kTileLines + 1;           // padded line stride
template <class T> constexpr size_t KbnTileSmemBytes(int dir) {
  return sizeof(T) * 4 * kTileHalo * kTilePitch + size_t(kTileHalo) * kTilePitch +
         (dir == 0 ? sizeof(T) * 4 * (kTileCells + 1) * kTilePitch : 0);
}

template <class T, class M>
__global__ void __launch_bounds__(256, 3) KbnRegularTileKernel(CcSweepArgs a) {
  constexpr int kL = kTileLines, kNSeg = kTileSegs, kC = kTileCells, kH = kTileHalo,
                kP = kTilePitch;
  extern __shared__ __align__(16) unsigned char tile_smem[];
  T (*su)[kH][kP] = reinterpret_cast<T (*)[kH][kP]>(tile_smem);  // [4][kH][kP]
  signed char (*scls)[kP] =
      reinterpret_cast<signed char (*)[kP]>(tile_smem + sizeof(T) * 4 * kH * kP);
  // x sweeps: the face fluxes of the block's cells, faces C0 .. C0 + kC
  T (*sf)[kC + 1][kP] = reinterpret_cast<T (*)[kC + 1][kP]>(
      tile_smem + ((sizeof(T) * 4 * kH * kP + size_t(kH) * kP + 15) / 16) * 16);
  const CcGeom& g = a.s.g;
  const int dir = a.dir;
  const int nd = dir == 0 ? g.nx : g.ny;
  const int nt = dir == 0 ? g.ny : g.nx;
  const int ntl = g.NTiles(dir);
  const int nsup = (ntl + kNSeg - 1) / kNSeg;
  const int group = blockIdx.x / nsup, sup = blockIdx.x % nsup;
  const int C0 = sup * kC;
  const signed char* treg = g.tile_regular[dir] + int64_t(group) * ntl;
  bool any_regular = false;  // block-uniform
#pragma unroll
  for (int k = 0; k < kNSeg; ++k) {
    const int tl = sup * kNSeg + k;
    any_regular = any_regular || (tl < ntl && treg[tl] != 0);
  }
  const KbnConst<T, M>& kc = KbnBlockConst<T, M>(a);
  if (!kc.run) return;  // block-uniform
  const GasT<T, M> eq = kc.eq;
  for (int idx = threadIdx.x; idx < kH * kL; idx += blockDim.x) {
    int line, cell;
    if (dir == 0) {
      cell = idx % kH;
      line = idx / kH;
    } else {
      line = idx % kL;
      cell = idx / kL;
    }
    const int t = group * kL + line, c = C0 - 2 + cell;
    scls[cell][line] = static_cast<signed char>(t < nt ? CellClassAt(g, dir, t, c) : kCcBand);
    if (!any_regular) continue;
    T v[4] = {T(0), T(0), T(0), T(0)};
    if (t < nt && c <= nd + 1) {
      double vd[4];
      if (dir == 0)
        LoadCons(a.s, c, t, vd);
      else
        LoadCons(a.s, t, c, vd);
      T w[4];
      Narrow(w, vd);
      // the masked state (CompleteMasked with mask true): zero unless rho > 0
      const bool pos = w[0] > T(0);
#pragma unroll
      for (int k = 0; k < 4; ++k) v[k] = pos ? w[k] : T(0);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) su[k][cell][line] = v[k];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tile = sup * kNSeg + warp;
  const int t = group * kL + lane;
  const int c0 = tile * kCcTile, c1 = min(nd, c0 + kCcTile);
  const int64_t cs = int64_t(g.nx) * g.ny;
  const double dt_dx = kc.dt_dx;
  auto offset = [&](int tt, int c) {
    return dir == 0 ? int64_t(tt) * g.nx + c : int64_t(c) * g.nx + tt;
  };
  auto cls_at = [&](int c) { return static_cast<int>(scls[c - C0 + 2][lane]); };
  T smax = T(0);
  int status = 0;
  if (tile < ntl && t < nt) {
    if (treg[tile] == 0) {
      if (dir != 0)
        for (int c = c0; c < c1; ++c)
          if (cls_at(c) == kCcCovered) {
            const int64_t o = offset(t, c);
#pragma unroll
            for (int k = 0; k < 4; ++k) a.out[k * cs + o] = 0.0;
          }
    } else {
      const T lambda_half = kc.lambda_half;
      auto fetch = [&](int c, T* u) {
#pragma unroll
        for (int k = 0; k < 4; ++k) u[k] = su[k][c - C0 + 2][lane];
      };
      T um[4], uc[4], up[4];
      fetch(c0 - 2, um);
      fetch(c0 - 1, uc);
      C2T<T> recR_prev, q_prev;
      // the previous face's flux (FP32 in the mixed flavour: the FP64
      // difference is formed by DiffToDouble, one FP64 operation per
      // component in the update)
      T f_prev[4];
      int cls_prev = cls_at(c0 - 1);
      const bool next_marches =
          warp + 1 < kNSeg && tile + 1 < ntl && treg[tile + 1] != 0 && c1 < nd;
      for (int j = c0 - 1; j <= c1; ++j) {
        fetch(j + 1, up);
        C2T<T> recL, recR;
        PredictMasked(eq, recL, recR, um, uc, up, true, a.limiter, lambda_half, dir);
        C2T<T> q;
        CompleteMasked(eq, q, uc, true);
        if (j >= c0) {
          const int cls = cls_at(j);
          T f[4];
          HllMasked(eq, f, recR_prev, recL, dir);
          if (cls == kCcRegular || cls_prev == kCcRegular) {
            T s0w, s1w;
            EinfeldtMasked(eq, q_prev, q, dir, s0w, s1w);
            const T mx = PMaxT(PMaxT(T(0), fabs(s0w)), fabs(s1w));
            smax = mx > smax ? mx : smax;
          }
          if (dir == 0) {
            // face j for the block's update: faces c0 .. c1 - 1 of this
            // tile, and face c1 unless the block's next warp marches (it
            // computes that face as its first, from the same data)
            if (j < c1 || !next_marches)
#pragma unroll
              for (int k = 0; k < 4; ++k) sf[k][j - C0][lane] = f[k];
          } else if (j > c0 && cls_prev != kCcBand) {
            // cell j-1: regular, or covered (0)
            const int64_t o = offset(t, j - 1);
            if (cls_prev == kCcRegular) {
#pragma unroll
              for (int k = 0; k < 4; ++k) {
                const double prev = __ldg(a.s.in + k * cs + o);
                double d;
                if constexpr (sizeof(T) == 4)
                  d = DiffToDouble(f_prev[k], f[k]);
                else
                  d = Widen(f_prev[k] + T(0)) - Widen(f[k] + T(0));
                a.out[k * cs + o] = prev + dt_dx * d;
              }
              if (__double_as_longlong(a.out[o]) <= 0) status |= kStatusNonPositiveDensity;
            } else {
#pragma unroll
              for (int k = 0; k < 4; ++k) a.out[k * cs + o] = 0.0;
            }
          }
#pragma unroll
          for (int k = 0; k < 4; ++k) f_prev[k] = f[k];
          cls_prev = cls;
        }
        recR_prev = recR;
        q_prev = q;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          um[k] = uc[k];
          uc[k] = up[k];
        }
      }
    }
  }
  if (dir == 0) {
    // the block's update, threads along x: regular cells from the two face
    // fluxes, covered cells 0 (band cells are the band kernel's)
    __syncthreads();
    for (int idx = threadIdx.x; idx < kC * kL; idx += blockDim.x) {
      const int cell = idx % kC, line = idx / kC;
      const int c = C0 + cell, tt = group * kL + line;
      if (c >= nd || tt >= nt) continue;
      const int cls = scls[cell + 2][line];
      if (cls == kCcBand) continue;
      const int64_t o = offset(tt, c);
      if (cls == kCcCovered) {
#pragma unroll
        for (int k = 0; k < 4; ++k) a.out[k * cs + o] = 0.0;
        continue;
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const double prev = __ldg(a.s.in + k * cs + o);
        double d;
        if constexpr (sizeof(T) == 4)
          d = DiffToDouble(sf[k][cell][line], sf[k][cell + 1][line]);
        else
          d = Widen(sf[k][cell][line] + T(0)) - Widen(sf[k][cell + 1][line] + T(0));
        a.out[k * cs + o] = prev + dt_dx * d;
      }
      if (__double_as_longlong(a.out[o]) <= 0) status |= kStatusNonPositiveDensity;
    }
  }
  const double smax_d = static_cast<double>(smax);
  BlockMaxAtomic<1>(a.smax_out, &smax_d);
  if (status && a.ctrl) atomicOr(&a.ctrl->step_status, status);
}

// The regular and covered cells of a KBN sweep in the FP64 flavours (bound by
// the FP64 pipe): each thread marches the runs of consecutive tiles with a
// regular cell in its segment of one grid line, one predictor per cell, with
// the arithmetic and the regular-cell argument of KbnRegularTileKernel; the
// CFL speeds are screened in FP32 as in the uniform sweeps (FilteredCfl,
// fvs_sweep.cuh), none in a step's first sweep.  Tiles without a regular
// cell only write their covered cells (0).  The tile flag is the warp's, so
// the control flow is warp-uniform.
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
  const KbnConst<T, M>& kc = KbnBlockConst<T, M>(a);
  if (!kc.run) return;  // block-uniform
  T smax = T(0);
  int status = 0;
  constexpr bool kScreen = sizeof(T) == 8;
  const bool skip_cfl = kScreen && a.skip_cfl != 0;
  const bool screen = kScreen && a.s.gamma > 1.0 && a.s.gamma <= 2.0;
  const unsigned amask = __ballot_sync(0xffffffffu, t64 < nt);
  if (t64 < nt) {
    const int t = static_cast<int>(t64);
    const GasT<T, M> eq = kc.eq;
    const T lambda_half = kc.lambda_half;
    const double dt_dx = kc.dt_dx;
    const int64_t cs = int64_t(g.nx) * g.ny;
    const int ntl = g.NTiles(dir);
    const signed char* treg = g.tile_regular[dir] + int64_t(group) * ntl;
    auto offset = [&](int c) {
      return dir == 0 ? int64_t(t) * g.nx + c : int64_t(c) * g.nx + t;
    };
    // state of cell c masked as on a regular cell (alpha 1: zeroed only where
    // rho <= 0): the FP64 load (fetch, one cell ahead of its use) and its
    // conversion (finish)
    auto fetch = [&](int c, double* vd) {
      return dir == 0 ? LoadConsDeferred(a.s, c, t, vd) : LoadConsDeferred(a.s, t, c, vd);
    };
    auto finish = [&](const double* vd, int flags, T* u) {
      T v[4];
      Narrow(v, vd);
      ApplyLoadFlags(v, flags);
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
      if (treg[tile] == 0) {
        const int c1 = min(nd, (tile + 1) * kCcTile);
        for (int c = tile * kCcTile; c < c1; ++c)
          if (CellClassAt(g, dir, t, c) == kCcCovered) {
            const int64_t o = offset(c);
#pragma unroll
            for (int q = 0; q < 4; ++q) a.out[q * cs + o] = 0.0;
          }
        ++tile;
        continue;
      }
      int r1 = tile + 1;
      while (r1 < tile_end && treg[r1] != 0) ++r1;
      const int j0 = tile * kCcTile, j1 = min(nd, r1 * kCcTile);
      tile = r1;
      // march the run [j0, j1): faces j0 .. j1, cells j0 .. j1-1
      T um[4], uc[4], up[4];
      double dn[4];
      int fl = fetch(j0 - 2, dn);
      finish(dn, fl, um);
      fl = fetch(j0 - 1, dn);
      finish(dn, fl, uc);
      int fl_dn = fetch(j0, dn);
      C2T<T> recR_prev, q_prev;
      T f_prev[4];
      fast::Wave<float> v_prev{};
      bool ok_prev = false;
      bool have_prev = false;
      int cls_prev = CellClassAt(g, dir, t, j0 - 1);
      for (int j = j0 - 1; j <= j1; ++j) {
        finish(dn, fl_dn, up);
        if (j + 2 <= j1 + 1) fl_dn = fetch(j + 2, dn);
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
          const int cls = CellClassAt(g, dir, t, j);
          const bool count = cls == kCcRegular || cls_prev == kCcRegular;
          if constexpr (kScreen) {
            if (!skip_cfl) {
              bool need = false;
              if (count) {
                const float s32 = fast::FaceMaxSpeed<float>(g32, v_prev, v);
                const float sh = fast::Math<float>::Sqrt(fmaxf(v_prev.h, v.h));
                need = !(ok && ok_prev &&
                         fmaf(s32, kCflRel, fmaf(kCflScale, sh, kCflAbs)) < thr);
              }
              if (__any_sync(amask, need)) {
                if (!have_prev) CompleteMasked(eq, q_prev, um, true);
                CompleteMasked(eq, q, uc, true);
                if (count) {
                  T s0w, s1w;
                  EinfeldtMasked(eq, q_prev, q, dir, s0w, s1w);
                  const T mx = PMaxT(PMaxT(T(0), fabs(s0w)), fabs(s1w));
                  smax = mx > smax ? mx : smax;
                }
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
          if constexpr (!kScreen) {
            if (count) {
              T s0w, s1w;
              EinfeldtMasked(eq, q_prev, q, dir, s0w, s1w);
              const T mx = PMaxT(PMaxT(T(0), fabs(s0w)), fabs(s1w));
              smax = mx > smax ? mx : smax;
            }
          }
          if (j > j0 && cls_prev != kCcBand) {
            const int64_t o = offset(j - 1);
            if (cls_prev == kCcRegular) {
#pragma unroll
              for (int c = 0; c < 4; ++c) {
                const double prev = __ldg(a.s.in + c * cs + o);
                // the FP64 flux difference (mixed: formed exactly by
                // DiffToDouble, as the tile kernel does)
                double d;
                if constexpr (sizeof(T) == 4)
                  d = DiffToDouble(f_prev[c], f[c]);
                else
                  d = Widen(f_prev[c] + T(0)) - Widen(f[c] + T(0));
                a.out[c * cs + o] = prev + dt_dx * d;
              }
              if (__double_as_longlong(a.out[o]) <= 0) status |= kStatusNonPositiveDensity;
            } else {
#pragma unroll
              for (int c = 0; c < 4; ++c) a.out[c * cs + o] = 0.0;
            }
          }
#pragma unroll
          for (int c = 0; c < 4; ++c) f_prev[c] = f[c];
          cls_prev = cls;
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
// (KbnStabilisation.hpp:275-345).  A warp owns 32 neighbouring columns,
// ic = 31 w - 1 + lane (the next warp's lane 0 repeats this warp's lane 31),
// and a segment of `rows` rows; each lane loads and completes its cells once,
// marching up the column, and pairs each cell with the one below it (kept
// from the previous row: the y face) and with the one to its left (lane - 1,
// a shuffle: the x face).  Every face is evaluated once, by the lane of its
// right / upper cell, with the arithmetic of the per-face form (masked
// completion of both cells, masked Einfeldt speeds, max(0, |sL|, |sR|)), so
// the maximum is the same bit for bit; the per-face form loaded and completed
// every cell four times.
template <class T, class M>
__global__ void __launch_bounds__(128)
    KbnStableDtKernel(CcStateArgs a, int rows, unsigned long long* smax_out, Control* ctrl) {
  if (!BlockAll(!(ctrl && (ctrl->abort || ctrl->done)))) return;
  const CcGeom& g = a.g;
  const int lane = threadIdx.x & 31;
  const int64_t gw = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int ncw = (g.nx + 1 + 30) / 31;     // x faces 0..nx on lanes 1..31
  const int nseg = (g.ny + 1 + rows - 1) / rows;  // face rows 0..ny
  T sm[2] = {T(0), T(0)};
  if (gw < int64_t(ncw) * nseg) {  // warp-uniform
    const int ic = 31 * static_cast<int>(gw % ncw) - 1 + lane;
    const bool in_grid = ic <= g.nx;  // lanes past column nx load column nx, unused
    const int icl = in_grid ? ic : g.nx;
    const int j0 = static_cast<int>(gw / ncw) * rows;
    const int j1 = min(j0 + rows, g.ny + 1);
    const GasT<T, M> eq = MakeGasT<T, M>(a.gamma);
    // a row's cell with its volume fraction and the fractions of its x face
    // (left) and y face (below), loaded one row before its use
    struct Row {
      double u[4];
      int flags;
      double alpha, bx, by;
    };
    const bool x_face = lane >= 1 && in_grid, y_face = lane >= 1 && ic < g.nx;
    auto fetch = [&](int j, Row& r) {
      r.flags = LoadConsDeferred(a, icl, j, r.u);
      r.alpha = g.alpha[g.CellIndex(icl, j)];
      r.bx = (x_face && j >= 0 && j < g.ny) ? g.beta[0][g.FaceIndex(0, ic, j)] : 0.0;
      r.by = (y_face && j >= 0) ? g.beta[1][g.FaceIndex(1, j, ic)] : 0.0;
    };
    auto complete = [&](const Row& r, C2T<T>& q) {
      T u[4];
      Narrow(u, r.u);
      ApplyLoadFlags(u, r.flags);
      CompleteMasked(eq, q, u, r.alpha > 0.0);
    };
    Row next;
    fetch(j0 - 1, next);
    C2T<T> below;
    complete(next, below);
    fetch(j0, next);
    for (int j = j0; j < j1; ++j) {
      const Row row = next;
      if (j + 1 < j1) fetch(j + 1, next);  // the next row, early
      C2T<T> cur;
      complete(row, cur);
      const C2T<T> left = ShflUp(cur, 1);
      // x face ic of row j (cells ic - 1 and ic)
      if (row.bx > 0.0) {
        T s0, s1;
        EinfeldtMasked(eq, left, cur, 0, s0, s1);
        const T mx = PMaxT(PMaxT(T(0), fabs(s0)), fabs(s1));
        sm[0] = mx > sm[0] ? mx : sm[0];
      }
      // y face j of column ic (cells j - 1 and j)
      if (row.by > 0.0) {
        T s0, s1;
        EinfeldtMasked(eq, below, cur, 1, s0, s1);
        const T mx = PMaxT(PMaxT(T(0), fabs(s0)), fabs(s1));
        sm[1] = mx > sm[1] ? mx : sm[1];
      }
      below = cur;
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
    const int n = a.s.g.nband[a.dir];
    if (n > 0) KbnBandKernel<T, M><<<unsigned((n + 63) / 64), 64, 0, s>>>(a);
    return cudaGetLastError();
  }
  if (sizeof(T) == 4 && !(a.dir == 1 && a.occupancy == 10)) {
    // mixed: tiles staged in shared memory, 32 lines x 64 cells per block
    const int64_t blocks = int64_t(a.s.g.NGroups(a.dir)) * ((a.s.g.NTiles(a.dir) + 7) / 8);
    static bool attr_set = false;
    if (!attr_set) {
      const cudaError_t e =
          cudaFuncSetAttribute(KbnRegularTileKernel<T, M>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               int(KbnTileSmemBytes<T>(0) + 16));
      if (e != cudaSuccess) return e;
      attr_set = true;
    }
    if (blocks > 0)
      KbnRegularTileKernel<T, M>
          <<<unsigned(blocks), 256, KbnTileSmemBytes<T>(a.dir) + 16, s>>>(a);
  } else {
    // FP64 flavours (bound by the FP64 pipe), and the mixed flavour's y
    // sweeps as launch variant 10: threads march runs of tiles, one
    // predictor per cell
    const int block = 128;
    int seg = a.seg_len > 0 ? a.seg_len : nd;
    seg = (seg + kCcTile - 1) / kCcTile * kCcTile;
    CcSweepArgs b = a;
    b.seg_len = seg;
    dim3 grid(unsigned((nt + block - 1) / block), unsigned((nd + seg - 1) / seg));
    if constexpr (sizeof(T) == 4)
      KbnRegularSweepKernel<T, M, 5><<<grid, block, 0, s>>>(b);
    else
      KbnRegularSweepKernel<T, M, 3><<<grid, block, 0, s>>>(b);
  }
  return cudaGetLastError();
}

template <class T, class M>
cudaError_t LaunchKbnStableDt(const CcStateArgs& a, unsigned long long* smax_out, Control* ctrl,
                              cudaStream_t s) {
  // segments of 4..32 rows, short enough for about 32 warps per SM of 152
  const int64_t ncw = (a.g.nx + 1 + 30) / 31;
  const int64_t target = int64_t(152) * 32;
  const int rows = static_cast<int>(
      std::min<int64_t>(32, std::max<int64_t>(4, (int64_t(a.g.ny + 1) * ncw + target - 1) / target)));
  const int64_t warps = ncw * ((a.g.ny + 1 + rows - 1) / rows);
  const int block = 128;
  KbnStableDtKernel<T, M><<<unsigned((warps * 32 + block - 1) / block), block, 0, s>>>(
      a, rows, smax_out, ctrl);
  return cudaGetLastError();
}

}  // namespace cc
}  // namespace fvs
