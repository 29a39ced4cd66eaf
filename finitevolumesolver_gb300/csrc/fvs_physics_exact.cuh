// fvs_physics_exact.cuh -- perfect-gas Euler physics in FP64 with the
// reference's exact operation order.
//
// Translation units that include this header are compiled with -fmad=false:
// every a*b+c stays a rounded multiply followed by a rounded add, division and
// sqrt are the IEEE correctly rounded ones, so the results are bit-identical
// to the reference's x86-64 SSE2 build (no FMA contraction).
//
// Reference functions restated here (maikel/FiniteVolumeSolver):
//   PerfectGas<D>::CompleteFromCons, Flux   src/equations/PerfectGas.cpp:25-124
//   EinfeldtSignalVelocities<PerfectGas<D>> src/equations/perfect_gas/EinfeldtSignalVelocities.hpp:64-97
//   Hll<...>::ComputeNumericFlux (array)    include/fub/flux_method/HllMethod.hpp:260-293
//   VanLeer / MinMod slopes                 include/fub/flux_method/MusclHancockMethod.hpp:92-187
//   MusclHancock::ComputeNumericFlux        include/fub/flux_method/MusclHancockMethod.hpp:419-485
#pragma once

#include <cstdint>

namespace fvs {
namespace exact {

struct Gas {
  double gamma;
  double gamma_minus_1_inv;
};

template <int D> struct Complete {
  double rho;
  double m[D];
  double E;
  double p;
  double c;
};

// |m|^2 in the order of the reference's array path (Eigen default traversal
// splits the 3-term sum as m0^2 + (m1^2 + m2^2)).
template <int D> __device__ __forceinline__ double SquaredNorm(const double* m) {
  if constexpr (D == 1) {
    return m[0] * m[0];
  } else if constexpr (D == 2) {
    return m[0] * m[0] + m[1] * m[1];
  } else {
    return m[0] * m[0] + (m[1] * m[1] + m[2] * m[2]);
  }
}

__device__ __forceinline__ double PMin(double a, double b) { return a < b ? a : b; }
__device__ __forceinline__ double PMax(double a, double b) { return a > b ? a : b; }

// CompleteFromCons: e_kin = 0.5*|m|^2/rho, p = (E - e_kin) / gamma_minus_1_inv,
// c = sqrt(gamma*p/rho).
template <int D>
__device__ __forceinline__ void CompleteFromCons(const Gas& eq, Complete<D>& q,
                                                 const double* u) {
  q.rho = u[0];
#pragma unroll
  for (int d = 0; d < D; ++d) q.m[d] = u[1 + d];
  q.E = u[1 + D];
  const double e_kin = 0.5 * SquaredNorm<D>(q.m) / q.rho;
  const double e_int = q.E - e_kin;
  q.p = e_int / eq.gamma_minus_1_inv;
  q.c = sqrt(eq.gamma * q.p / q.rho);
}

template <int D>
__device__ __forceinline__ void Flux(double* f, const Complete<D>& q, int dir) {
  const double velocity = q.m[dir] / q.rho;
  f[0] = q.m[dir];
#pragma unroll
  for (int d = 0; d < D; ++d) f[1 + d] = velocity * q.m[d];
  f[1 + dir] += q.p;
  f[1 + D] = velocity * (q.E + q.p);
}

template <int D>
__device__ __forceinline__ void AsCons(double* u, const Complete<D>& q) {
  u[0] = q.rho;
#pragma unroll
  for (int d = 0; d < D; ++d) u[1 + d] = q.m[d];
  u[1 + D] = q.E;
}

template <int D>
__device__ __forceinline__ void Einfeldt(const Gas& eq, const Complete<D>& L,
                                         const Complete<D>& R, int dir,
                                         double& sL, double& sR) {
  const double rhoL = L.rho;
  const double rhoR = R.rho;
  const double sqRhoL = sqrt(rhoL);
  const double sqRhoR = sqrt(rhoR);
  const double oosqRhoSum = 1.0 / (sqRhoL + sqRhoR);
  const double uL = L.m[dir] / rhoL;
  const double uR = R.m[dir] / rhoR;
  const double roeU = (uL * sqRhoL + uR * sqRhoR) * oosqRhoSum;
  const double hL = (L.E + L.p) / rhoL;
  const double hR = (R.E + R.p) / rhoR;
  const double roeH = (hL * sqRhoL + hR * sqRhoR) * oosqRhoSum;
  const double roeA2 = (eq.gamma - 1.0) * (roeH - 0.5 * roeU * roeU);
  const double roeA = sqrt(roeA2);
  sL = PMin(uL - L.c, roeU - roeA);
  sR = PMax(roeU + roeA, uR + R.c);
}

template <int D>
__device__ __forceinline__ void HllFlux(const Gas& eq, double* nf,
                                        const Complete<D>& L,
                                        const Complete<D>& R, int dir) {
  constexpr int K = D + 2;
  double s0, s1;
  Einfeldt<D>(eq, L, R, dir, s0, s1);
  double fL[K], fR[K], qL[K], qR[K];
  Flux<D>(fL, L, dir);
  Flux<D>(fR, R, dir);
  AsCons<D>(qL, L);
  AsCons<D>(qR, R);
  const double sL = PMin(s0, 0.0);
  const double sR = PMax(s1, 0.0);
  const double sLsR = sL * sR;
  double ds = sR - sL;
  ds = (ds > 0.0) ? ds : 1.0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    nf[k] = (sR * fL[k] - sL * fR[k] + sLsR * (qR[k] - qL[k])) / ds;
  }
}

// Per-cell quantities of the HLLE stable-dt estimate (Einfeldt speeds of the
// two cells of a face): sqrt(rho), normal velocity, enthalpy, sound speed.
struct CellWave {
  double sq;
  double u;
  double h;
  double a;
};

template <int D>
__device__ __forceinline__ CellWave MakeCellWave(const Gas& eq, const double* u,
                                                 int dir) {
  Complete<D> q;
  CompleteFromCons<D>(eq, q, u);
  CellWave w;
  w.sq = sqrt(q.rho);
  w.u = q.m[dir] / q.rho;
  w.h = (q.E + q.p) / q.rho;
  w.a = q.c;
  return w;
}

// max(0, |sL|, |sR|) of the face between two cells; the stable dt of the face
// is dx divided by it (Hll::ComputeStableDt, HllMethod.hpp:337-347).
__device__ __forceinline__ double FaceMaxSpeed(const Gas& eq, const CellWave& L,
                                               const CellWave& R) {
  const double oosqRhoSum = 1.0 / (L.sq + R.sq);
  const double roeU = (L.u * L.sq + R.u * R.sq) * oosqRhoSum;
  const double roeH = (L.h * L.sq + R.h * R.sq) * oosqRhoSum;
  const double roeA2 = (eq.gamma - 1.0) * (roeH - 0.5 * roeU * roeU);
  const double roeA = sqrt(roeA2);
  const double sL = PMin(L.u - L.a, roeU - roeA);
  const double sR = PMax(roeU + roeA, R.u + R.a);
  return PMax(PMax(0.0, fabs(sL)), fabs(sR));
}

// VanLeer, MinMod, NoLimiter (the central slope, unlimited) and NoGradient
// (slope 0) -- include/fub/flux_method/MusclHancockMethod.hpp:31-187.
enum Limiter : int { kVanLeer = 0, kMinMod = 1, kNoLimiter = 2, kNoGradient = 3 };

__device__ __forceinline__ double LimitedSlope(int limiter, double qL, double qM,
                                               double qR) {
  const double sL = qM - qL;
  const double sR = qR - qM;
  if (limiter == kVanLeer) {
    const double c = 2.0 * sL * sR;
    return (c > 0.0) ? c / (sL + sR) : 0.0;
  }
  if (limiter == kMinMod) {
    return (sR > 0) ? PMax(0.0, PMin(sL, sR)) : PMin(0.0, PMax(sL, sR));
  }
  if (limiter == kNoLimiter) return 0.5 * (sL + sR);
  return 0.0;
}

// MUSCL-Hancock predictor of one cell: the Hancock-evolved states at its left
// face (recL, the reference's rec_[1] when the cell is stencil[2]) and at its
// right face (recR, rec_[0] when the cell is stencil[1]).  Computing both once
// per cell gives bit-identical face states to the reference, which computes
// each cell's predictor twice (once for each of its faces).
template <int D>
__device__ __forceinline__ void MusclPredictBoth(const Gas& eq, Complete<D>& recL,
                                                 Complete<D>& recR,
                                                 const double* q0,
                                                 const double* q1,
                                                 const double* q2, int limiter,
                                                 double lambda_half, int dir) {
  constexpr int K = D + 2;
  double uL[K], uR[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const double slope = LimitedSlope(limiter, q0[k], q1[k], q2[k]);
    uL[k] = q1[k] - 0.5 * slope;
    uR[k] = q1[k] + 0.5 * slope;
  }
  Complete<D> qL, qR;
  CompleteFromCons<D>(eq, qL, uL);
  CompleteFromCons<D>(eq, qR, uR);
  double fL[K], fR[K];
  Flux<D>(fL, qL, dir);
  Flux<D>(fR, qR, dir);
  double a[K], b[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const double df = fL[k] - fR[k];
    b[k] = uR[k] + lambda_half * df;
    a[k] = uL[k] + lambda_half * df;
  }
  CompleteFromCons<D>(eq, recR, b);
  CompleteFromCons<D>(eq, recL, a);
}

}  // namespace exact
}  // namespace fvs
