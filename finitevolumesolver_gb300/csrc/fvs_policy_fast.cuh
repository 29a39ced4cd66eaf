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

#include "fvs_internal.h"
#include "fvs_physics_fast.cuh"
#include "fvs_sweep.cuh"

namespace fvs {

// FP64 <-> FP32 conversions on the integer pipes.  The FP64 pipe of the
// GB300 issues 2 operations per SM and cycle; F2F conversions run on it and
// would dominate the mixed sweep, so the mixed flavour moves them to integer
// bit manipulation (64 lanes per SM and cycle).
//
// double -> float: round to nearest (ties away from zero); magnitudes below
// the FP32 normal range flush to a signed zero, above it saturate to inf.
__device__ __forceinline__ float DoubleToFloatBits(double x) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  const unsigned hi = static_cast<unsigned>(b >> 32);
  const unsigned lo = static_cast<unsigned>(b);
  const unsigned e = (hi >> 20) & 0x7FFu;
  const unsigned sign = hi & 0x80000000u;
  unsigned f = sign | ((e - 896u) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
  f += (lo >> 28) & 1u;
  f = (e <= 896u) ? sign : f;
  f = (e >= 1151u) ? (sign | 0x7F800000u) : f;
  return __uint_as_float(f);
}

// float -> double, exact for zero and every normal float (FP32 subnormals
// flush to zero).
__device__ __forceinline__ double FloatToDoubleBits(float x) {
  const unsigned f = __float_as_uint(x);
  const unsigned e = (f >> 23) & 0xFFu;
  const unsigned sign = f & 0x80000000u;
  unsigned hi = sign | ((e + 896u) << 20) | ((f & 0x7FFFFFu) >> 3);
  unsigned lo = f << 29;
  hi = (e == 0u) ? sign : hi;
  lo = (e == 0u) ? 0u : lo;
  hi = (e == 255u) ? (sign | 0x7FF00000u | ((f & 0x7FFFFFu) >> 3)) : hi;
  return __hiloint2double(static_cast<int>(hi), static_cast<int>(lo));
}

template <int D, typename T> struct FastBase {
  using Real = T;
  // the mixed flavour is memory-bound: its x sweep uses lanes along x
  static constexpr bool kWarpX = sizeof(T) == 4;
  static constexpr int kMinBlocks = 1;
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
  static __device__ __forceinline__ T FaceMaxSpeed(const Gas& eq, const Wave& L,
                                                   const Wave& R) {
    return fast::FaceMaxSpeed<T>(eq, L, R);
  }
};

template <int D> struct Fast64Policy : FastBase<D, double> {};
template <int D> struct Mixed32Policy : FastBase<D, float> {};
// The same arithmetic compiled for more resident blocks per SM (fewer
// registers per thread, more warps to hide latency); the autotuner picks.
template <int D> struct Mixed32PolicyOcc4 : FastBase<D, float> {
  static constexpr int kMinBlocks = 4;
};
template <int D> struct Mixed32PolicyOcc5 : FastBase<D, float> {
  static constexpr int kMinBlocks = 5;
};

}  // namespace fvs
