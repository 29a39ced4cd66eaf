// fvs_policy_fast.cuh -- sweep policies of the fast FP64 and the
// mixed-precision flavours (shared by the uniform-grid and the AMR patch
// sweeps).
//
// Fast FP64: the reference's formulas with shared reciprocals, FMA
// contraction and Newton-refined reciprocal / reciprocal-square-root seeds;
// per call within ~1e-13 relative of the exact flavour.
// Mixed: MUSCL-Hancock reconstruction, limiter, HLLE flux and the CFL
// speeds in FP32; state storage and the conservative update
// U' = U + dt/dx (F_L - F_R) in FP64 (the fluxes are widened to FP64 before
// the update, so mass, momentum and energy are conserved to FP64 round-off).
#pragma once

#include "fvs_convert.cuh"
#include "fvs_internal.h"
#include "fvs_physics_fast.cuh"
#include "fvs_sweep.cuh"

namespace fvs {

template <int D, typename T> struct FastBase {
  using Real = T;
  // the mixed flavour is memory-bound: its x sweep uses lanes along x
  static constexpr bool kWarpX = sizeof(T) == 4;
  static constexpr int kMinBlocks = 1;
  // FP64 and double-float: the sweep screens the Einfeldt CFL speeds in FP32
  static constexpr bool kEinfeldtCfl = sizeof(T) != 4;
  using Gas = fast::Gas<T>;
  using Rec = fast::State<D, T>;
  using Wave = fast::Wave<T>;
  static constexpr int K = D + 2;
  static __device__ __forceinline__ Gas MakeGas(double gamma) {
    Gas g;
    g.gamma = T(gamma);
    g.gm1 = T(gamma - 1.0);
    return g;
  }
  static __device__ __forceinline__ Gas MakeGasFor(const SweepArgs& a) {
    return MakeGas(a.gamma);
  }
  static __device__ __forceinline__ void ToCell(T* c, const double* u) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if constexpr (sizeof(T) == 4) {
        c[k] = DoubleToFloatBits(u[k]);
      } else {
        c[k] = u[k];
      }
    }
  }
  static __device__ __forceinline__ void Predict(const Gas& eq, Rec& recL, Rec& recR,
                                                 const T* q0, const T* q1, const T* q2,
                                                 int limiter, double lambda_half, int dir) {
    fast::PredictBoth<D, T>(eq, recL, recR, q0, q1, q2, limiter, T(lambda_half), dir);
  }
  using Stats = NoStats;
  // the mixed flavour hands its FP32 fluxes to the sweep unwidened
  static constexpr bool kFloatFlux = sizeof(T) == 4;
  static __device__ __forceinline__ T FaceR(const Gas& eq, T* f, const Rec& L, const Rec& R,
                                            const Wave& wL, const Wave& wR, int dir, Stats&) {
    fast::HllFlux<D, T>(eq, f, L, R, dir);
    return fast::FaceMaxSpeed<T>(eq, wL, wR);
  }
  // the face flux alone (no CFL speed): FP64 (widened) and compute precision
  static __device__ __forceinline__ void FluxOnly(const Gas& eq, double* F, const Rec& L,
                                                  const Rec& R, int dir) {
    HllFlux(eq, F, L, R, dir);
  }
  static __device__ __forceinline__ void FluxOnlyR(const Gas& eq, T* f, const Rec& L,
                                                   const Rec& R, int dir) {
    fast::HllFlux<D, T>(eq, f, L, R, dir);
  }
  static __device__ __forceinline__ T Face(const Gas& eq, double* F, const Rec& L,
                                           const Rec& R, const Wave& wL, const Wave& wR,
                                           int dir, Stats&) {
    HllFlux(eq, F, L, R, dir);
    return fast::FaceMaxSpeed<T>(eq, wL, wR);
  }
  static __device__ __forceinline__ void HllFlux(const Gas& eq, double* F, const Rec& L,
                                                 const Rec& R, int dir) {
    T nf[K];
    fast::HllFlux<D, T>(eq, nf, L, R, dir);
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if constexpr (sizeof(T) == 4) {
        F[k] = FloatToDoubleBits(nf[k]);
      } else {
        F[k] = nf[k];
      }
    }
  }
  static __device__ __forceinline__ Wave MakeWave(const Gas& eq, const T* u, int dir) {
    return fast::MakeWave<D, T>(eq, u, dir);
  }
  static __device__ __forceinline__ void MakeWaves(const Gas& eq, const T* u, Wave* w) {
    fast::MakeWaves<D, T>(eq, u, w);
  }
  static __device__ __forceinline__ T FaceMaxSpeed(const Gas& eq, const Wave& L,
                                                   const Wave& R) {
    return fast::FaceMaxSpeed<T>(eq, L, R);
  }
};

// three resident blocks of 128 threads (at most 168 registers)
template <int D> struct Fast64Policy : FastBase<D, double> {
  static constexpr int kMinBlocks = 3;
};
template <int D> struct Mixed32Policy : FastBase<D, float> {};
// The same arithmetic compiled for more resident blocks per SM (fewer
// registers per thread, more warps to hide latency); the autotuner picks.
template <int D> struct Mixed32PolicyOcc4 : FastBase<D, float> {
  static constexpr int kMinBlocks = 4;
};
template <int D> struct Mixed32PolicyOcc5 : FastBase<D, float> {
  static constexpr int kMinBlocks = 5;
};
// The mixed flavour with the marching kernel in x as well (a thread walks a
// row; each row's loads are reused from L1 instead of exchanged by shuffles).
template <int D> struct Mixed32PolicyMarchX : FastBase<D, float> {
  static constexpr bool kWarpX = false;
};
template <int D> struct Mixed32PolicyMarchXOcc4 : FastBase<D, float> {
  static constexpr bool kWarpX = false;
  static constexpr int kMinBlocks = 4;
};
template <int D> struct Mixed32PolicyMarchXOcc5 : FastBase<D, float> {
  static constexpr bool kWarpX = false;
  static constexpr int kMinBlocks = 5;
};

}  // namespace fvs
