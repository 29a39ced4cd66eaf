// fvs_hllem.cuh -- the HLLEM flux of the perfect gas on the device (FP64,
// the reference's operation order; included by -fmad=false translation
// units so that results are bit-identical to the oracle).
//
// Restates Hllem<PerfectGas<D>, Larrouturou = true>, array path
// (src/equations/perfect_gas/HllemMethod.hpp:711-1072) and its stable dt
// (HllemMethod.hpp:1152-1216); MaSq of the perfect gas is 1
// (include/fub/equations/EulerEquation.hpp:53-62).  Larrouturou: the
// tangential momenta of both states are removed (their kinetic energy taken
// out of E; the stored p and c are kept), the HLLE flux of the reduced states
// is corrected along the second eigenvector with the anti-diffusion factor
// delta = a_roe / (a_roe + |u_bar|), and the tangential momentum and
// kinetic-energy fluxes are upwinded by the sign of the mass flux.  The 3-D
// normal-momentum correction uses roeU[iy], as the reference does
// (HllemMethod.hpp:991-992).
#pragma once

#include "fvs_physics_exact.cuh"

namespace fvs {
namespace exact {

template <int D>
__device__ __forceinline__ void HllemFlux(const Gas& eq, double* nf, const Complete<D>& left,
                                          const Complete<D>& right, int ix) {
  constexpr int K = D + 2;
  const double Msq = 1.0;
  const double Minv = 1.0 / sqrt(Msq);
  Complete<D> L = left, R = right;
  const double rhoL = L.rho, rhoR = R.rho;
  double vL_[D], vR_[D];
  double eKinRL = 0.0, eKinRR = 0.0;
#pragma unroll
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
  const double sqRhoL = sqrt(rhoL);
  const double sqRhoR = sqrt(rhoR);
  const double sqRhoSum = sqRhoL + sqRhoR;
  const double wL = sqRhoL / sqRhoSum;
  const double wR = sqRhoR / sqRhoSum;
  double uL[D], uR[D], roeU[D];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    uL[i] = L.m[i] / rhoL;
    uR[i] = R.m[i] / rhoR;
    roeU[i] = wL * uL[i] + wR * uR[i];
  }
  const double roeH = wL * hL + wR * hR;
  double sqN = 0.0;
#pragma unroll
  for (int i = 0; i < D; ++i) sqN += roeU[i] * roeU[i];
  sqN *= Msq;
  const double sqN_half = 0.5 * sqN;
  const double roeGamma = (sqRhoL * eq.gamma + sqRhoR * eq.gamma) / sqRhoSum;
  const double gm1 = roeGamma - 1.0;
  const double roeA2 = gm1 * (roeH - sqN_half);
  const double roeA = sqrt(roeA2);
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
#pragma unroll
  for (int k = 0; k < K; ++k)
    hlle[k] = (bR * fL[k] - bL * fR[k] + bLbR * (qR[k] - qL[k])) / dbp;
  const double u_bar = 0.5 * (sR + sL);
  const double delta = roeA / (roeA + fabs(u_bar));
  const double b = bLbR / dbp;
  const double dRho = rhoR - rhoL;
  double dRhoU[D];
#pragma unroll
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

// max(|sL|, |sR|) of Hllem::ComputeStableDt: Einfeldt speeds with
// max(aL, aR) on both sides, unreduced states; dt = dx / it.
template <int D>
__device__ __forceinline__ double HllemMaxSpeed(const Gas& eq, const Complete<D>& L,
                                                const Complete<D>& R, int ix) {
  const double gm1 = eq.gamma - 1.0;
  const double Msq = 1.0;
  const double Minv = 1.0 / sqrt(Msq);
  const double rhoL = L.rho, rhoR = R.rho;
  const double hL = (L.E + L.p) / rhoL;
  const double hR = (R.E + R.p) / rhoR;
  const double sqRhoL = sqrt(rhoL);
  const double sqRhoR = sqrt(rhoR);
  const double sqRhoSum = sqRhoL + sqRhoR;
  const double wL = sqRhoL / sqRhoSum;
  const double wR = sqRhoR / sqRhoSum;
  double uL[D], uR[D], roeU[D];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    uL[i] = L.m[i] / rhoL;
    uR[i] = R.m[i] / rhoR;
    roeU[i] = wL * uL[i] + wR * uR[i];
  }
  const double roeH = wL * hL + wR * hR;
  double sqN = 0.0;
#pragma unroll
  for (int i = 0; i < D; ++i) sqN += roeU[i] * roeU[i];
  sqN *= Msq;
  const double roeA2 = gm1 * (roeH - 0.5 * sqN);
  const double roeA = sqrt(roeA2);
  const double maxA = PMax(L.c, R.c);
  const double sL = PMin(uL[ix] - maxA * Minv, roeU[ix] - roeA * Minv);
  const double sR = PMax(roeU[ix] + roeA * Minv, uR[ix] + maxA * Minv);
  return PMax(fabs(sL), fabs(sR));
}

}  // namespace exact
}  // namespace fvs
