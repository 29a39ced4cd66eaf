// fvs_recon_hllem.cuh -- the two perfect-gas MUSCL-Hancock variants whose
// face flux is Hllem<PerfectGas, Larrouturou>: the characteristic
// reconstruction (perfect_gas::MusclHancockCharacteristic) and the primitive
// reconstruction (perfect_gas::MusclHancockPrim).  FP64 in the reference's
// operation order; included only by -fmad=false translation units, so the
// face states are bit-identical to the oracle's.
//
// Both reconstruct each of the two inner cells of a face's four-cell
// stencil from the cell and its two neighbours; computing a cell's left-face
// and right-face states once per cell (from the same slopes) gives the same
// bits as the reference, which reconstructs every cell once per face.
#pragma once

#include "fvs_physics_exact.cuh"

namespace fvs {
namespace exact {

// VanLeer::operator()(sL, sR) (include/fub/flux_method/MusclHancockMethod.hpp:
// 137-149): the harmonic mean 2 sL sR / (sL + sR) of two one-sided slopes
// of the same sign, else 0.
__device__ __forceinline__ double VanLeerOf(double sL, double sR) {
  const double r = 2.0 * sL * sR;
  return (r > 0.0) ? r / (sL + sR) : 0.0;
}

// MusclHancockCharacteristic<Rank>, array path
// (src/equations/perfect_gas/MusclHancockCharacteristicMethod.hpp:51-64
// ComputeAmplitudes, :77-85 Recombine, :108-128 ComputeSlopes, :170-180
// DoTimeStep, :235-256 Reconstruct; src/equations/PerfectGas.cpp:160-174
// CompleteFromPrim).  The amplitudes of the jumps (minus = dp - rho c du,
// zero = drho - dp / c^2, plus = dp + rho c du and the two transverse
// velocity jumps) are limited with the van Leer function, advanced half a
// step with their characteristic speeds u - c, u, u + c, and recombined
// into primitive increments.  Velocities are three-vectors indexed by
// ix, iy = (ix+1)%3, iz = (iy+1)%3 (zero beyond D), as the reference's
// Primitives are.  recR is the cell's state at its right face (sign +1),
// recL at its left face (sign -1).
template <int D>
__device__ __forceinline__ void CharPredictBoth(const Gas& eq, Complete<D>& recL,
                                                Complete<D>& recR, const Complete<D>& s0,
                                                const Complete<D>& s1, const Complete<D>& s2,
                                                double lambda, int ix) {
  const int iy = (ix + 1) % 3;
  const int iz = (iy + 1) % 3;
  const double rho = s1.rho;
  const double u = s1.m[ix] / rho;
  const double c = s1.c;
  const double rhoc = rho * c;
  const double ooc2 = 1.0 / (c * c);
  double v0[3], v1[3], v2[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    v0[d] = d < D ? s0.m[d] / s0.rho : 0.0;
    v1[d] = d < D ? s1.m[d] / s1.rho : 0.0;
    v2[d] = d < D ? s2.m[d] / s2.rho : 0.0;
  }
  double slope[5];
  {
    const double dpL = s1.p - s0.p, dpR = s2.p - s1.p;
    const double duL = v1[ix] - v0[ix], duR = v2[ix] - v1[ix];
    const double drL = s1.rho - s0.rho, drR = s2.rho - s1.rho;
    slope[0] = VanLeerOf(dpL - rhoc * duL, dpR - rhoc * duR);
    slope[1] = VanLeerOf(drL - ooc2 * dpL, drR - ooc2 * dpR);
    slope[2] = VanLeerOf(dpL + rhoc * duL, dpR + rhoc * duR);
    slope[3] = VanLeerOf(v1[iy] - v0[iy], v2[iy] - v1[iy]);
    slope[4] = VanLeerOf(v1[iz] - v0[iz], v2[iz] - v1[iz]);
  }
  double um[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) um[d] = d < D ? s1.m[d] / s1.rho : 0.0;
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const double sign = side == 0 ? 1.0 : -1.0;
    const double minus = sign * 0.5 * slope[0] * (1.0 - sign * lambda * (u - c));
    const double zero = sign * 0.5 * slope[1] * (1.0 - sign * lambda * u);
    const double plus = sign * 0.5 * slope[2] * (1.0 - sign * lambda * (u + c));
    const double dv = sign * 0.5 * slope[3] * (1.0 - sign * lambda * u);
    const double dw = sign * 0.5 * slope[4] * (1.0 - sign * lambda * u);
    const double dpres = 0.5 * (minus + plus);
    const double drho = ooc2 * dpres + zero;
    double dvel[3];
    dvel[ix] = 0.5 * (plus - minus) / rhoc;
    dvel[iy] = dv;
    dvel[iz] = dw;
    const double w_rho = drho + rho;
    const double w_p = dpres + s1.p;
    Complete<D>& rec = side == 0 ? recR : recL;
    rec.rho = w_rho;
#pragma unroll
    for (int d = 0; d < D; ++d) rec.m[d] = w_rho * (dvel[d] + um[d]);
    rec.p = w_p;
    const double e_kin = 0.5 * SquaredNorm<D>(rec.m) / w_rho;
    rec.E = e_kin + w_p * eq.gamma_minus_1_inv;
    rec.c = sqrt(eq.gamma * w_p / w_rho);
  }
}

// The slope limiter of MusclHancockPrim<Dim>::ComputeNumericFlux
// (src/equations/perfect_gas/MusclHancockPrimMethod.hpp:63-77): the van
// Leer function of the smaller of the two one-sided ratios to the central
// difference, times the central difference; flat below |dq| = 1e-12.
__device__ __forceinline__ double PrimLimiter(double qL, double qM, double qR) {
  const double delta_q = 0.5 * (qR - qL);
  const bool is_relevant = fabs(delta_q) > 1e-12;
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

// MusclHancockPrim<Dim>, array path
// (src/equations/perfect_gas/MusclHancockPrimMethod.hpp:78-175): limited
// slopes of rho, p and the velocity components, advanced half a step with
// the primitive-variable Euler equations.  recR is the cell's state at its
// right face (the reference's "_l" formulas), recL at its left face ("_r").
template <int D>
__device__ __forceinline__ void PrimPredictBoth(const Gas& eq, Complete<D>& recL,
                                                Complete<D>& recR, const Complete<D>& s0,
                                                const Complete<D>& s1, const Complete<D>& s2,
                                                double lambda, int d) {
  double u0[D], u1[D], u2[D];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    u0[i] = s0.m[i] / s0.rho;
    u1[i] = s1.m[i] / s1.rho;
    u2[i] = s2.m[i] / s2.rho;
  }
  const double rho = s1.rho, p = s1.p, a = s1.c;
  const double drho = PrimLimiter(s0.rho, rho, s2.rho);
  const double dp = PrimLimiter(s0.p, p, s2.p);
  double du[D];
#pragma unroll
  for (int i = 0; i < D; ++i) du[i] = PrimLimiter(u0[i], u1[i], u2[i]);
  const double ud = u1[d], dud = du[d];
  const double tr = lambda * (ud * drho + rho * dud);
  const double tp = lambda * (rho * a * a * dud + ud * dp);
  const double ucorr = 0.5 * lambda * dp / rho;
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    double rec_rho, rec_p, rec_u[D];
    if (side == 0) {
      rec_rho = rho + 0.5 * (drho - tr);
      rec_p = p + 0.5 * (dp - tp);
#pragma unroll
      for (int i = 0; i < D; ++i) rec_u[i] = u1[i] + 0.5 * (du[i] - lambda * (ud * du[i]));
    } else {
      rec_rho = rho - 0.5 * (drho + tr);
      rec_p = p - 0.5 * (dp + tp);
#pragma unroll
      for (int i = 0; i < D; ++i) rec_u[i] = u1[i] - 0.5 * (du[i] + lambda * (ud * du[i]));
    }
    rec_u[d] -= ucorr;
    Complete<D>& rec = side == 0 ? recR : recL;
    rec.rho = rec_rho;
#pragma unroll
    for (int i = 0; i < D; ++i) rec.m[i] = rec_rho * rec_u[i];
    rec.p = rec_p;
    rec.c = sqrt(eq.gamma * rec_p / rec_rho);
    rec.E = 0.5 * rec_rho * SquaredNorm<D>(rec_u) + rec_p * eq.gamma_minus_1_inv;
  }
}

}  // namespace exact
}  // namespace fvs
