// fvs_policy_exact.cuh -- sweep policy with the reference's exact FP64
// arithmetic (shared by the uniform-grid and the AMR patch sweeps).  Every
// translation unit that includes it is compiled with -fmad=false.
#pragma once

#include "fvs_internal.h"
#include "fvs_physics_exact.cuh"
#include "fvs_sweep.cuh"

namespace fvs {

// Exact policy for the marching sweep.
template <int D> struct ExactPolicy {
  using Real = double;
  static constexpr bool kWarpX = false;
  static constexpr int kMinBlocks = 3;  // at most 168 registers
  static constexpr bool kEinfeldtCfl = true;  // CFL speeds screened in FP32
  using Gas = exact::Gas;
  using Wave = exact::CellWave;
  using Rec = exact::Complete<D>;
  static __device__ __forceinline__ Gas MakeGas(double gamma) {
    Gas g;
    g.gamma = gamma;
    g.gamma_minus_1_inv = 1.0 / (gamma - 1.0);
    return g;
  }
  static __device__ __forceinline__ Gas MakeGasFor(const SweepArgs& a) {
    return MakeGas(a.gamma);
  }
  static __device__ __forceinline__ void ToCell(double* c, const double* u) {
#pragma unroll
    for (int k = 0; k < D + 2; ++k) c[k] = u[k];
  }
  static __device__ __forceinline__ void Predict(const Gas& eq, Rec& recL,
                                                 Rec& recR, const double* q0,
                                                 const double* q1,
                                                 const double* q2, int limiter,
                                                 double lambda_half, int dir) {
    exact::MusclPredictBoth<D>(eq, recL, recR, q0, q1, q2, limiter,
                               lambda_half, dir);
  }
  using Stats = NoStats;
  static __device__ __forceinline__ void FluxOnly(const Gas& eq, double* F, const Rec& L,
                                                  const Rec& R, int dir) {
    exact::HllFlux<D>(eq, F, L, R, dir);
  }
  static __device__ __forceinline__ double Face(const Gas& eq, double* F, const Rec& L,
                                                const Rec& R, const Wave& wL,
                                                const Wave& wR, int dir, Stats&) {
    exact::HllFlux<D>(eq, F, L, R, dir);
    return exact::FaceMaxSpeed(eq, wL, wR);
  }
  static __device__ __forceinline__ Wave MakeWave(const Gas& eq, const double* u,
                                                  int dir) {
    return exact::MakeCellWave<D>(eq, u, dir);
  }
  // the waves of all D directions from one CompleteFromCons (each equal to
  // MakeWave's: the same operations)
  static __device__ __forceinline__ void MakeWaves(const Gas& eq, const double* u, Wave* w) {
    exact::Complete<D> q;
    exact::CompleteFromCons<D>(eq, q, u);
    const double sq = sqrt(q.rho);
    const double h = (q.E + q.p) / q.rho;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      w[d].sq = sq;
      w[d].u = q.m[d] / q.rho;
      w[d].h = h;
      w[d].a = q.c;
    }
  }
  static __device__ __forceinline__ double FaceMaxSpeed(const Gas& eq, const Wave& wL,
                                                        const Wave& wR) {
    return exact::FaceMaxSpeed(eq, wL, wR);
  }
};

}  // namespace fvs
