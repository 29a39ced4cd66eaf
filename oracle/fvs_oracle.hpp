// fvs_oracle.hpp -- CPU oracle for the split finite-volume patch update.
//
// TEST INFRASTRUCTURE ONLY.  This is a scalar C++17 restatement of the
// reference's (maikel/FiniteVolumeSolver) perfect-gas Euler patch update,
// written to reproduce its arithmetic operation by operation so that the GPU
// kernels can be checked against it.  Only tests/, __graft_entry__.smoke()
// and the CPU-baseline leg of bench.py may load it; the product path never
// does.
//
// Build flags: -O2 -ffp-contract=off -fno-fast-math (no FMA contraction), the
// same IEEE behaviour as the reference's x86-64 SSE2 build (CMakeLists.txt
// sets no -march and no fast-math).
//
// Every function names the reference file:line it follows.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>

namespace fvs_oracle {

// PerfectGas<D> parameters: include/fub/equations/PerfectGas.hpp:207-211.
struct Gas {
  double gamma = 1.4;
  double gamma_minus_1_inv = 1.0 / (1.4 - 1.0);
};

template <int D> struct Cons {
  double rho;
  double m[D];
  double E;
};

// Complete state component order (rho, m[D], E, p, c):
// include/fub/equations/PerfectGas.hpp:132-161.
template <int D> struct Complete {
  double rho;
  double m[D];
  double E;
  double p;
  double c;
};

// sum_d m_d^2 in the evaluation order of the reference's array (production)
// path: Eigen's colwise().squaredNorm() over the row-major Dim x 8 momentum
// block uses the default (non-vectorised, fully unrolled) traversal, which
// splits the sum recursively into halves: m0^2 + (m1^2 + m2^2) for D = 3.
// src/equations/PerfectGas.cpp:32-37.
template <int D> inline double SquaredNorm(const double* m) {
  if constexpr (D == 1) {
    return m[0] * m[0];
  } else if constexpr (D == 2) {
    return m[0] * m[0] + m[1] * m[1];
  } else {
    return m[0] * m[0] + (m[1] * m[1] + m[2] * m[2]);
  }
}

// KineticEnergy: 0.5 * |m|^2 / rho.  src/equations/PerfectGas.cpp:25-37.
template <int D> inline double KineticEnergy(double rho, const double* m) {
  return 0.5 * SquaredNorm<D>(m) / rho;
}

// PerfectGas<D>::CompleteFromCons  src/equations/PerfectGas.cpp:96-124.
// Note the pressure is e_int DIVIDED by gamma_minus_1_inv (not multiplied by
// gamma - 1).
template <int D>
inline void CompleteFromCons(const Gas& eq, Complete<D>& q, const double* u) {
  q.rho = u[0];
  for (int d = 0; d < D; ++d) q.m[d] = u[1 + d];
  q.E = u[1 + D];
  const double e_kin = KineticEnergy<D>(q.rho, q.m);
  const double e_int = q.E - e_kin;
  q.p = e_int / eq.gamma_minus_1_inv;
  q.c = std::sqrt(eq.gamma * q.p / q.rho);
}

// Masked CompleteFromCons: zero where the mask is false or rho <= 0.
// src/equations/PerfectGas.cpp:126-144.
template <int D>
inline void CompleteFromConsMasked(const Gas& eq, Complete<D>& q,
                                   const double* u, bool mask) {
  mask = mask && (u[0] > 0.0);
  if (!mask) {
    q.rho = 0.0;
    for (int d = 0; d < D; ++d) q.m[d] = 0.0;
    q.E = 0.0;
    q.p = 0.0;
    q.c = 0.0;
    return;
  }
  CompleteFromCons<D>(eq, q, u);
}

template <int D> inline void AsCons(double* u, const Complete<D>& q) {
  u[0] = q.rho;
  for (int d = 0; d < D; ++d) u[1 + d] = q.m[d];
  u[1 + D] = q.E;
}

// PerfectGas<D>::Flux  src/equations/PerfectGas.cpp:52-77.
template <int D>
inline void Flux(double* f, const Complete<D>& q, int dir) {
  const double velocity = q.m[dir] / q.rho;
  f[0] = q.m[dir];
  for (int d = 0; d < D; ++d) f[1 + d] = velocity * q.m[d];
  f[1 + dir] += q.p;
  f[1 + D] = velocity * (q.E + q.p);
}

// Masked flux: rho replaced by 1 where the mask is false or rho <= 0.
// src/equations/PerfectGas.cpp:79-93.
template <int D>
inline void FluxMasked(double* f, const Complete<D>& q, bool mask, int dir) {
  mask = mask && (q.rho > 0.0);
  const double rho = mask ? q.rho : 1.0;
  const double velocity = q.m[dir] / rho;
  f[0] = q.m[dir];
  for (int d = 0; d < D; ++d) f[1 + d] = velocity * q.m[d];
  f[1 + dir] += q.p;
  f[1 + D] = velocity * (q.E + q.p);
}

// Eigen's SSE2 packet min / max (_mm_min_pd / _mm_max_pd semantics), used by
// the reference's array path.
inline double PMin(double a, double b) { return a < b ? a : b; }
inline double PMax(double a, double b) { return a > b ? a : b; }

// EinfeldtSignalVelocities<PerfectGas<D>>
// src/equations/perfect_gas/EinfeldtSignalVelocities.hpp:25-97.
template <int D>
inline void Einfeldt(const Gas& eq, const Complete<D>& L, const Complete<D>& R,
                     int dir, double& sL, double& sR) {
  const double rhoL = L.rho;
  const double rhoR = R.rho;
  const double rhoUL = L.m[dir];
  const double rhoUR = R.m[dir];
  const double aL = L.c;
  const double aR = R.c;
  const double sqRhoL = std::sqrt(rhoL);
  const double sqRhoR = std::sqrt(rhoR);
  const double oosqRhoSum = 1.0 / (sqRhoL + sqRhoR);
  const double uL = rhoUL / rhoL;
  const double uR = rhoUR / rhoR;
  const double roeU = (uL * sqRhoL + uR * sqRhoR) * oosqRhoSum;
  const double hL = (L.E + L.p) / rhoL;
  const double hR = (R.E + R.p) / rhoR;
  const double roeH = (hL * sqRhoL + hR * sqRhoR) * oosqRhoSum;
  const double roeA2 = (eq.gamma - 1.0) * (roeH - 0.5 * roeU * roeU);
  const double roeA = std::sqrt(roeA2);
  const double sL1 = uL - aL;
  const double sL2 = roeU - roeA;
  const double sR1 = roeU + roeA;
  const double sR2 = uR + aR;
  sL = PMin(sL1, sL2);
  sR = PMax(sR1, sR2);
}

// Masked Einfeldt: uses sqrt(rho)/sum weights (a different operation order).
// src/equations/perfect_gas/EinfeldtSignalVelocities.hpp:99-142.
template <int D>
inline void EinfeldtMasked(const Gas& eq, const Complete<D>& L,
                           const Complete<D>& R, bool mask, int dir,
                           double& sL, double& sR) {
  const double rhoL = L.rho;
  const double rhoR = R.rho;
  const double rhoUL = mask ? L.m[dir] : 0.0;
  const double rhoUR = mask ? R.m[dir] : 0.0;
  const double aL = mask ? L.c : 0.0;
  const double aR = mask ? R.c : 0.0;
  const double rhoLs = mask ? rhoL : 1.0;
  const double rhoRs = mask ? rhoR : 1.0;
  const double sqRhoL = std::sqrt(rhoLs);
  const double sqRhoR = std::sqrt(rhoRs);
  const double sqRho = sqRhoL + sqRhoR;
  const double uL = rhoUL / rhoLs;
  const double uR = rhoUR / rhoRs;
  const double wL = sqRhoL / sqRho;
  const double wR = sqRhoR / sqRho;
  const double roeU = uL * wL + uR * wR;
  const double rhoEL = mask ? L.E : 0.0;
  const double rhoER = mask ? R.E : 0.0;
  const double pL = mask ? L.p : 0.0;
  const double pR = mask ? R.p : 0.0;
  // the reference divides by the unmasked densities here
  const double hL = (rhoEL + pL) / rhoL;
  const double hR = (rhoER + pR) / rhoR;
  const double roeH = hL * wL + hR * wR;
  const double roeA2 = (eq.gamma - 1.0) * (roeH - 0.5 * roeU * roeU);
  const double roeA = std::sqrt(roeA2);
  sL = PMin(uL - aL, roeU - roeA);
  sR = PMax(roeU + roeA, uR + aR);
}

// Hll<Eq, Einfeldt>::ComputeNumericFlux (array path)
// include/fub/flux_method/HllMethod.hpp:260-293.
template <int D>
inline void HllFlux(const Gas& eq, double* nf, const Complete<D>& L,
                    const Complete<D>& R, int dir) {
  double s0, s1;
  Einfeldt<D>(eq, L, R, dir, s0, s1);
  double fL[D + 2], fR[D + 2], qL[D + 2], qR[D + 2];
  Flux<D>(fL, L, dir);
  Flux<D>(fR, R, dir);
  AsCons<D>(qL, L);
  AsCons<D>(qR, R);
  const double sL = PMin(s0, 0.0);
  const double sR = PMax(s1, 0.0);
  const double sLsR = sL * sR;
  double ds = sR - sL;
  ds = (ds > 0.0) ? ds : 1.0;
  for (int k = 0; k < D + 2; ++k) {
    nf[k] = (sR * fL[k] - sL * fR[k] + sLsR * (qR[k] - qL[k])) / ds;
  }
}

// Hll<Eq, Einfeldt>::ComputeStableDt  include/fub/flux_method/HllMethod.hpp:337-347.
template <int D>
inline double HllStableDt(const Gas& eq, const Complete<D>& L,
                          const Complete<D>& R, double dx, int dir) {
  double s0, s1;
  Einfeldt<D>(eq, L, R, dir, s0, s1);
  const double mx = PMax(PMax(0.0, std::abs(s0)), std::abs(s1));
  return dx / mx;
}

// Hll<Eq, Einfeldt>::SolveRiemannProblem (scalar path, completes the
// middle state)  include/fub/flux_method/HllMethod.hpp:161-184.
template <int D>
inline void HllRiemannState(const Gas& eq, Complete<D>& sol,
                            const Complete<D>& L, const Complete<D>& R,
                            int dir) {
  double sL, sR;
  Einfeldt<D>(eq, L, R, dir, sL, sR);
  double fL[D + 2], fR[D + 2], qL[D + 2], qR[D + 2];
  Flux<D>(fL, L, dir);
  Flux<D>(fR, R, dir);
  AsCons<D>(qL, L);
  AsCons<D>(qR, R);
  const double ds = sL != sR ? sR - sL : 1.0;
  if (0.0 < sL) {
    sol = L;
  } else if (sR < 0.0) {
    sol = R;
  } else {
    double u[D + 2];
    for (int k = 0; k < D + 2; ++k) {
      u[k] = (sR * qR[k] - sL * qL[k] + fL[k] - fR[k]) / ds;
    }
    CompleteFromCons<D>(eq, sol, u);
  }
}

// Reflect (src/equations/PerfectGas.cpp:266-300) of the momentum m[D] about
// the unit normal of direction dir: m - 2 (m . e) e, the dot product summed in
// component order (the other state components are unchanged).
template <int D> inline void ReflectMomentum(double* m, int dir) {
  double e[D];
  for (int d = 0; d < D; ++d) e[d] = d == dir ? 1.0 : 0.0;
  double dot = m[0] * e[0];
  for (int d = 1; d < D; ++d) dot += m[d] * e[d];
  for (int d = 0; d < D; ++d) m[d] = m[d] - 2 * (dot * e[d]);
}

// Slope limiters  include/fub/flux_method/MusclHancockMethod.hpp:31-187:
// VanLeer, MinMod, NoLimiter (:31-69, the central slope 0.5 (sL + sR)) and
// NoGradient (:71-90, slope 0).
enum Limiter : int { kVanLeer = 0, kMinMod = 1, kNoLimiter = 2, kNoGradient = 3 };

inline double VanLeer(double sL, double sR) {
  const double c = 2.0 * sL * sR;
  return (c > 0.0) ? c / (sL + sR) : 0.0;
}

inline double MinMod(double sL, double sR) {
  // array path: (sR > 0).select(zero.max(sL.min(sR)), zero.min(sL.max(sR)))
  return (sR > 0) ? PMax(0.0, PMin(sL, sR)) : PMin(0.0, PMax(sL, sR));
}

inline double LimitedSlope(int limiter, double qL, double qM, double qR) {
  const double sL = qM - qL;
  const double sR = qR - qM;
  switch (limiter) {
  case kMinMod:
    return MinMod(sL, sR);
  case kNoLimiter:
    return 0.5 * (sL + sR);
  case kNoGradient:
    return 0.0;
  default:
    return VanLeer(sL, sR);
  }
}

// One half of MusclHancock::ComputeNumericFlux: the predicted (Hancock) state
// of a cell at its right face (side = +1, "rec_[0]") or its left face
// (side = -1, "rec_[1]").  q0, q1, q2 are the cell's left neighbour, the cell
// and its right neighbour.  include/fub/flux_method/MusclHancockMethod.hpp:419-485.
template <int D>
inline void MusclPredict(const Gas& eq, Complete<D>& rec, const double* q0,
                         const double* q1, const double* q2, int limiter,
                         double lambda_half, int dir, int side) {
  constexpr int K = D + 2;
  double slope[K], uL[K], uR[K];
  for (int k = 0; k < K; ++k) slope[k] = LimitedSlope(limiter, q0[k], q1[k], q2[k]);
  for (int k = 0; k < K; ++k) {
    uL[k] = q1[k] - 0.5 * slope[k];
    uR[k] = q1[k] + 0.5 * slope[k];
  }
  Complete<D> qL, qR;
  CompleteFromCons<D>(eq, qL, uL);
  CompleteFromCons<D>(eq, qR, uR);
  double fL[K], fR[K];
  Flux<D>(fL, qL, dir);
  Flux<D>(fR, qR, dir);
  double u[K];
  const double* base = side > 0 ? uR : uL;
  for (int k = 0; k < K; ++k) u[k] = base[k] + lambda_half * (fL[k] - fR[k]);
  CompleteFromCons<D>(eq, rec, u);
}

// Hllem<PerfectGas<D>, Larrouturou = true>::ComputeNumericFlux, array path
// (src/equations/perfect_gas/HllemMethod.hpp:711-1072), for one face; MaSq
// of the perfect gas is 1 (include/fub/equations/EulerEquation.hpp:53-62).
// Larrouturou: the tangential momenta of both states are removed (their
// kinetic energy taken out of E, the stored p and c kept), the HLLE flux of
// the reduced states is corrected along the second eigenvector, and the
// tangential momentum and kinetic-energy fluxes are upwinded by the sign of
// the mass flux.  The operation order is the reference's, including its 3-D
// normal-momentum correction with roeU[iy] (HllemMethod.hpp:991-992).
template <int D>
inline void HllemFlux(const Gas& eq, double* nf, const Complete<D>& left,
                      const Complete<D>& right, int ix) {
  constexpr int K = D + 2;
  const double Msq = 1.0;
  const double Minv = 1.0 / std::sqrt(Msq);
  Complete<D> L = left, R = right;
  const double rhoL = L.rho, rhoR = R.rho;
  double vL_[D], vR_[D];
  double eKinRL = 0.0, eKinRR = 0.0;
  for (int i = 0; i < D; ++i) {
    const int mask = i == ix;
    vL_[i] = L.m[i] / rhoL;
    vR_[i] = R.m[i] / rhoR;
    eKinRL += (1 - mask) * vL_[i] * vL_[i];
    eKinRR += (1 - mask) * vR_[i] * vR_[i];
    L.m[i] *= mask;
    R.m[i] *= mask;
  }
  eKinRL *= 0.5 * Msq;
  eKinRR *= 0.5 * Msq;
  L.E -= rhoL * eKinRL;
  R.E -= rhoR * eKinRR;
  double fL[K], fR[K];
  Flux<D>(fL, L, ix);
  Flux<D>(fR, R, ix);
  const double aL = L.c, aR = R.c;
  const double rhoEL = L.E, rhoER = R.E;
  const double pL = L.p, pR = R.p;
  const double hL = (rhoEL + pL) / rhoL;
  const double hR = (rhoER + pR) / rhoR;
  const double sqRhoL = std::sqrt(rhoL);
  const double sqRhoR = std::sqrt(rhoR);
  const double sqRhoSum = sqRhoL + sqRhoR;
  const double wL = sqRhoL / sqRhoSum;
  const double wR = sqRhoR / sqRhoSum;
  double uL[D], uR[D], roeU[D];
  for (int i = 0; i < D; ++i) {
    uL[i] = L.m[i] / rhoL;
    uR[i] = R.m[i] / rhoR;
    roeU[i] = wL * uL[i] + wR * uR[i];
  }
  const double roeH = wL * hL + wR * hR;
  double sqN = 0.0;
  for (int i = 0; i < D; ++i) sqN += roeU[i] * roeU[i];
  sqN *= Msq;
  const double sqN_half = 0.5 * sqN;
  const double roeGamma = (sqRhoL * eq.gamma + sqRhoR * eq.gamma) / sqRhoSum;
  const double gm1 = roeGamma - 1.0;
  const double roeA2 = gm1 * (roeH - sqN_half);
  const double roeA = std::sqrt(roeA2);
  const double maxA = PMax(aL, aR);
  const double sL1 = uL[ix] - maxA * Minv;
  const double sL2 = roeU[ix] - roeA * Minv;
  const double sR1 = roeU[ix] + roeA * Minv;
  const double sR2 = uR[ix] + maxA * Minv;
  const double sL = PMin(sL1, sL2);
  const double sR = PMax(sR1, sR2);
  const double bL = PMin(sL, 0.0);
  const double bR = PMax(sR, 0.0);
  const double bLbR = bL * bR;
  const double db = bR - bL;
  const double dbp = (db > 0.0) ? db : 1.0;
  double qL[K], qR[K], hlle[K];
  AsCons<D>(qL, L);
  AsCons<D>(qR, R);
  for (int k = 0; k < K; ++k) hlle[k] = (bR * fL[k] - bL * fR[k] + bLbR * (qR[k] - qL[k])) / dbp;
  const double u_bar = 0.5 * (sR + sL);
  const double delta = roeA / (roeA + std::abs(u_bar));
  const double b = bLbR / dbp;
  const double dRho = rhoR - rhoL;
  double dRhoU[D];
  for (int i = 0; i < D; ++i) dRhoU[i] = R.m[i] - L.m[i];
  const double dRhoE = rhoER - rhoEL;
  const double g = gm1 / roeA2;
  if constexpr (D == 1) {
    const double l21 = g * (roeH - sqN);
    const double l22 = g * Msq * roeU[0];
    const double l23 = g * (-1.0);
    const double alpha_2 = l21 * dRho + l22 * dRhoU[0] + l23 * dRhoE;
    const double bda2 = b * delta * alpha_2;
    nf[0] = hlle[0] - bda2;
    nf[1] = hlle[1] - bda2 * roeU[0];
    nf[2] = hlle[2] - bda2 * sqN_half;
  } else if constexpr (D == 2) {
    const int iy = (ix == 0);
    const double l21 = g * (roeH - sqN);
    const double l22 = g * Msq * roeU[0];
    const double l23 = g * roeU[1];
    const double l24 = -g;
    const double alpha_2 = l21 * dRho + l22 * dRhoU[0] + l23 * dRhoU[1] + l24 * dRhoE;
    const double bd = b * delta;
    const double bda2 = bd * alpha_2;
    nf[0] = hlle[0] - bda2;
    nf[1 + ix] = hlle[1 + ix] - bda2 * roeU[ix];
    const bool upwind = nf[0] > 0.0;
    nf[1 + iy] = nf[0] * (upwind ? vL_[iy] : vR_[iy]);
    nf[3] = hlle[3] - bda2 * sqN_half + nf[0] * (upwind ? eKinRL : eKinRR);
  } else {
    const int iy = (ix + 1) % 3;
    const int iz = (iy + 1) % 3;
    const double l21 = g * (roeH - sqN);
    const double l22 = g * Msq * roeU[0];
    const double l23 = g * roeU[1];
    const double l24 = g * roeU[2];
    const double l25 = -g;
    const double alpha_2 =
        l21 * dRho + l22 * dRhoU[0] + l23 * dRhoU[1] + l24 * dRhoU[2] + l25 * dRhoE;
    const double bd = b * delta;
    const double bda2 = bd * alpha_2;
    nf[0] = hlle[0] - bda2;
    nf[1 + ix] = hlle[1 + ix] - bda2 * roeU[iy];
    const bool upwind = nf[0] > 0.0;
    nf[1 + iy] = nf[0] * (upwind ? vL_[iy] : vR_[iy]);
    nf[1 + iz] = nf[0] * (upwind ? vL_[iz] : vR_[iz]);
    nf[4] = hlle[4] - bda2 * sqN_half + nf[0] * (upwind ? eKinRL : eKinRR);
  }
}

// Hllem::ComputeStableDt, array path (HllemMethod.hpp:1152-1216): Einfeldt
// speeds with max(aL, aR) on both sides, unreduced states.
template <int D>
inline double HllemStableDt(const Gas& eq, const Complete<D>& L, const Complete<D>& R,
                            double dx, int ix) {
  const double gm1 = eq.gamma - 1.0;
  const double Msq = 1.0;
  const double Minv = 1.0 / std::sqrt(Msq);
  const double rhoL = L.rho, rhoR = R.rho;
  const double hL = (L.E + L.p) / rhoL;
  const double hR = (R.E + R.p) / rhoR;
  const double sqRhoL = std::sqrt(rhoL);
  const double sqRhoR = std::sqrt(rhoR);
  const double sqRhoSum = sqRhoL + sqRhoR;
  const double wL = sqRhoL / sqRhoSum;
  const double wR = sqRhoR / sqRhoSum;
  double uL[D], uR[D], roeU[D];
  for (int i = 0; i < D; ++i) {
    uL[i] = L.m[i] / rhoL;
    uR[i] = R.m[i] / rhoR;
    roeU[i] = wL * uL[i] + wR * uR[i];
  }
  const double roeH = wL * hL + wR * hR;
  double sqN = 0.0;
  for (int i = 0; i < D; ++i) sqN += roeU[i] * roeU[i];
  sqN *= Msq;
  const double roeA2 = gm1 * (roeH - 0.5 * sqN);
  const double roeA = std::sqrt(roeA2);
  const double maxA = PMax(L.c, R.c);
  const double sL = PMin(uL[ix] - maxA * Minv, roeU[ix] - roeA * Minv);
  const double sR = PMax(roeU[ix] + roeA * Minv, uR[ix] + maxA * Minv);
  const double maxS = PMax(std::abs(sL), std::abs(sR));
  return dx / maxS;
}

// MusclHancockCharacteristic<Rank>: one side of the characteristic
// reconstruction, array path (src/equations/perfect_gas/
// MusclHancockCharacteristicMethod.hpp:51-64 ComputeAmplitudes, :77-85
// Recombine, :108-128 ComputeSlopes, :170-180 DoTimeStep, :235-256
// Reconstruct; src/equations/PerfectGas.cpp:160-174 CompleteFromPrim).  s[0..2] are the
// cell's left neighbour, the cell and its right neighbour; sign = +1 gives
// the state at the cell's right face ("is_right_side" 0), -1 at its left
// face.  Primitive velocities are three-vectors (zero beyond D) indexed by
// ix, iy = (ix+1)%3, iz = (iy+1)%3, as the reference's Primitives are.
// The slopes of the five amplitudes are limited with VanLeer's functor
// (MusclHancockMethod.hpp:137-149), the only limiter the method accepts.
template <int D>
inline void CharPredict(const Gas& eq, Complete<D>& rec, const Complete<D>* s,
                        double lambda, int ix, double sign) {
  const int iy = (ix + 1) % 3;
  const int iz = (iy + 1) % 3;
  const Complete<D>& q = s[1];
  const double rho = q.rho;
  const double u = q.m[ix] / rho;
  const double c = q.c;
  const double rhoc = rho * c;
  const double ooc2 = 1.0 / (c * c);
  double v[3][3];
  for (int k = 0; k < 3; ++k)
    for (int d = 0; d < 3; ++d) v[k][d] = d < D ? s[k].m[d] / s[k].rho : 0.0;
  double amp[2][5];
  for (int h = 0; h < 2; ++h) {
    const Complete<D>& l = s[h];
    const Complete<D>& r = s[h + 1];
    const double dp = r.p - l.p;
    const double du = v[h + 1][ix] - v[h][ix];
    const double drho = r.rho - l.rho;
    amp[h][0] = dp - rhoc * du;    // minus
    amp[h][1] = drho - ooc2 * dp;  // zero
    amp[h][2] = dp + rhoc * du;    // plus
    amp[h][3] = v[h + 1][iy] - v[h][iy];
    amp[h][4] = v[h + 1][iz] - v[h][iz];
  }
  double slope[5];
  for (int k = 0; k < 5; ++k) slope[k] = VanLeer(amp[0][k], amp[1][k]);
  const double minus = sign * 0.5 * slope[0] * (1.0 - sign * lambda * (u - c));
  const double zero = sign * 0.5 * slope[1] * (1.0 - sign * lambda * u);
  const double plus = sign * 0.5 * slope[2] * (1.0 - sign * lambda * (u + c));
  const double dv = sign * 0.5 * slope[3] * (1.0 - sign * lambda * u);
  const double dw = sign * 0.5 * slope[4] * (1.0 - sign * lambda * u);
  double dvel[3];
  const double dpres = 0.5 * (minus + plus);
  const double drho = ooc2 * dpres + zero;
  dvel[ix] = 0.5 * (plus - minus) / rhoc;
  dvel[iy] = dv;
  dvel[iz] = dw;
  const double w_rho = drho + rho;
  const double w_p = dpres + q.p;
  rec.rho = w_rho;
  for (int d = 0; d < D; ++d) rec.m[d] = w_rho * (dvel[d] + q.m[d] / q.rho);
  rec.p = w_p;
  const double e_kin = KineticEnergy<D>(rec.rho, rec.m);
  rec.E = e_kin + w_p * eq.gamma_minus_1_inv;
  rec.c = std::sqrt(eq.gamma * rec.p / rec.rho);
}

// The slope limiter of MusclHancockPrim<Dim>::ComputeNumericFlux
// (src/equations/perfect_gas/MusclHancockPrimMethod.hpp:63-77): the van
// Leer function of the smaller of the two one-sided ratios to the central
// difference, times the central difference; flat below |dq| = 1e-12.
inline double PrimLimiter(double qL, double qM, double qR) {
  const double delta_q = 0.5 * (qR - qL);
  const bool is_relevant = std::abs(delta_q) > 1e-12;
  const double dq = is_relevant ? delta_q : 1.0;
  const double rL = is_relevant ? (qM - qL) / dq : 0.0;
  const double rR = is_relevant ? (qR - qM) / dq : 0.0;
  const bool is_positive = rL > 0.0 && rR > 0.0;
  const double r = is_positive ? PMin(rL, rR) : 0.0;
  const double r_1 = 2.0 * r / (1.0 + r);
  const double r_2 = 0.5 * (r + 1.0);
  const double sigma = r < 1.0 ? r_1 : r_2;
  return sigma * delta_q;
}

// MusclHancockPrim<Dim>: the Hancock-predicted primitive state of the cell
// s[1] at its right face (side = +1, the "_l" formulas) or its left face
// (side = -1, the "_r" formulas), array path
// (src/equations/perfect_gas/MusclHancockPrimMethod.hpp:78-175).
template <int D>
inline void PrimPredict(const Gas& eq, Complete<D>& rec, const Complete<D>* s,
                        double lambda, int d, int side) {
  double u[3][D];
  for (int k = 0; k < 3; ++k)
    for (int i = 0; i < D; ++i) u[k][i] = s[k].m[i] / s[k].rho;
  const double rho = s[1].rho, p = s[1].p, a = s[1].c;
  const double drho = PrimLimiter(s[0].rho, rho, s[2].rho);
  const double dp = PrimLimiter(s[0].p, p, s[2].p);
  double du[D];
  for (int i = 0; i < D; ++i) du[i] = PrimLimiter(u[0][i], u[1][i], u[2][i]);
  const double* ul = u[1];
  double rec_rho, rec_p, rec_u[D];
  if (side > 0) {
    rec_rho = rho + 0.5 * (drho - lambda * (ul[d] * drho + rho * du[d]));
    rec_p = p + 0.5 * (dp - lambda * (rho * a * a * du[d] + ul[d] * dp));
    for (int i = 0; i < D; ++i)
      rec_u[i] = ul[i] + 0.5 * (du[i] - lambda * (ul[d] * du[i]));
  } else {
    rec_rho = rho - 0.5 * (drho + lambda * (ul[d] * drho + rho * du[d]));
    rec_p = p - 0.5 * (dp + lambda * (rho * a * a * du[d] + ul[d] * dp));
    for (int i = 0; i < D; ++i)
      rec_u[i] = ul[i] - 0.5 * (du[i] + lambda * (ul[d] * du[i]));
  }
  rec_u[d] -= 0.5 * lambda * dp / rho;
  rec.rho = rec_rho;
  for (int i = 0; i < D; ++i) rec.m[i] = rec_rho * rec_u[i];
  rec.p = rec_p;
  rec.c = std::sqrt(eq.gamma * rec_p / rec_rho);
  rec.E = 0.5 * rec_rho * SquaredNorm<D>(rec_u) + rec_p * eq.gamma_minus_1_inv;
}

enum Method : int {
  kMusclHlle = 0,
  kHlle = 1,
  kGodunov = 2,
  kMusclGodunov = 3,
  kHllem = 4,       // Hllem<PerfectGas, Larrouturou>
  kMusclHllem = 5,  // MusclHancock<PerfectGas, Hllem, Limiter>
  kMusclChar = 6,   // perfect_gas::MusclHancockCharacteristic (HLLEM base)
  kMusclPrim = 7    // perfect_gas::MusclHancockPrim (HLLEM base)
};

}  // namespace fvs_oracle
