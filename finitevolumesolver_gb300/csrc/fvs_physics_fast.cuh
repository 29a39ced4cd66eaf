// fvs_physics_fast.cuh -- perfect-gas Euler physics for the fast flavours.
//
// The same functions as fvs_physics_exact.cuh (PerfectGas CompleteFromCons
// and Flux, Einfeldt speeds, HLL flux, van Leer / MinMod MUSCL-Hancock
// predictor -- src/equations/PerfectGas.cpp:52-124,
// src/equations/perfect_gas/EinfeldtSignalVelocities.hpp:25-97,
// include/fub/flux_method/HllMethod.hpp:260-293,
// include/fub/flux_method/MusclHancockMethod.hpp:92-187, 419-485), rewritten
// for throughput instead of bit parity:
//  - every state computes one reciprocal square root of rho and derives
//    sqrt(rho) = rho * rs and 1/rho = rs^2 from it, so the divisions by rho
//    become multiplications;
//  - p = (E - e_kin) * (gamma - 1) (the reference divides by 1/(gamma-1));
//  - the HLL flux multiplies by 1/(sR - sL) instead of dividing 5 times;
//  - FMA contraction is allowed.
// T = double gives the FP64 "fast" flavour (results within ~1e-13 relative of
// the exact flavour per call); T = float gives the mixed flavour's FP32
// reconstruction and flux.
//
// Reciprocal and reciprocal square root in FP64 start from the PTX
// rcp.approx.ftz.f64 / rsqrt.approx.ftz.f64 estimates (measured on GB300: at
// most 2^-20 relative error) and refine them with one third-order step from
// the series of the exact value in the residual r of the estimate y0:
//   1/a       = y0 / (1 - r),        r = 1 - a y0:   y0 (1 + r + r^2 + ...)
//   1/sqrt(a) = y0 (1 - r)^(-1/2),   r = 1 - a y0^2: y0 (1 + r/2 + 3 r^2/8 + ...)
// truncated after the r^2 term, so the refined value is off by ~r^3 < 2^-60
// (a few ulp after rounding).  a/b = a * (1/b) and sqrt(a) = a * (1/sqrt(a))
// then carry about one more ulp.
#pragma once

#include <cstdint>

namespace fvs {
namespace fast {

template <typename T> struct Math;

template <> struct Math<double> {
  static __device__ __forceinline__ double RcpSeed(double a) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(a));
    return y;
  }
  static __device__ __forceinline__ double RsqrtSeed(double a) {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(a));
    return y;
  }
  // 1/a: y0 (1 + r + r^2), r = 1 - a y0.
  static __device__ __forceinline__ double Rcp(double a) {
    const double y = RcpSeed(a);
    const double r = fma(-a, y, 1.0);
    return fma(y, fma(r, r, r), y);
  }
  // a/b as a times the refined reciprocal.
  static __device__ __forceinline__ double Div(double a, double b) { return a * Rcp(b); }
  // 1/sqrt(a), a > 0: y0 (1 + r (1/2 + 3 r/8)), r = 1 - a y0^2.
  static __device__ __forceinline__ double Rsqrt(double a) {
    const double y = RsqrtSeed(a);
    const double r = fma(-a, y * y, 1.0);
    return fma(y * r, fma(0.375, r, 0.5), y);
  }
  // sqrt(a) for a >= 0 (0 for a <= 0).
  static __device__ __forceinline__ double Sqrt(double a) {
    if (!(a > 0.0)) return 0.0;
    return a * Rsqrt(a);
  }
};

template <> struct Math<float> {
  static __device__ __forceinline__ float Rcp(float a) { return __fdividef(1.0f, a); }
  static __device__ __forceinline__ float Div(float a, float b) { return __fdividef(a, b); }
  static __device__ __forceinline__ float Rsqrt(float a) { return rsqrtf(a); }
  static __device__ __forceinline__ float Sqrt(float a) { return a > 0.0f ? a * rsqrtf(a) : 0.0f; }
};

template <typename T> struct Gas {
  T gamma;
  T gm1;  // gamma - 1
};

// A state with the derived quantities the HLL flux and the Einfeldt speeds
// need.
template <int D, typename T> struct State {
  T rho;
  T m[D];
  T E;
  T p;   // pressure
  T a;   // sound speed
  T u;   // normal velocity
  T sq;  // sqrt(rho)
  T h;   // (E + p) / rho
};

template <int D, typename T> __device__ __forceinline__ T SquaredNorm(const T* m) {
  if constexpr (D == 1) {
    return m[0] * m[0];
  } else if constexpr (D == 2) {
    return fma(m[1], m[1], m[0] * m[0]);
  } else {
    return fma(m[2], m[2], fma(m[1], m[1], m[0] * m[0]));
  }
}

// Complete a conservative state with all derived quantities.
template <int D, typename T>
__device__ __forceinline__ void Prepare(const Gas<T>& eq, State<D, T>& s, const T* u,
                                        int dir) {
  using M = Math<T>;
  s.rho = u[0];
#pragma unroll
  for (int d = 0; d < D; ++d) s.m[d] = u[1 + d];
  s.E = u[1 + D];
  const T rs = M::Rsqrt(s.rho);
  const T ir = rs * rs;
  s.sq = s.rho * rs;
  const T ke = T(0.5) * SquaredNorm<D, T>(s.m) * ir;
  s.p = (s.E - ke) * eq.gm1;
  s.u = s.m[dir] * ir;
  s.h = (s.E + s.p) * ir;
  s.a = M::Sqrt(eq.gamma * s.p * ir);
}

// Physical flux of a conservative state (PerfectGas::Flux), no sound speed.
template <int D, typename T>
__device__ __forceinline__ void FluxOfCons(const Gas<T>& eq, T* f, const T* u, int dir) {
  using M = Math<T>;
  const T ir = M::Rcp(u[0]);
  const T ke = T(0.5) * SquaredNorm<D, T>(u + 1) * ir;
  const T p = (u[1 + D] - ke) * eq.gm1;
  const T v = u[1 + dir] * ir;
  f[0] = u[1 + dir];
#pragma unroll
  for (int d = 0; d < D; ++d) f[1 + d] = v * u[1 + d];
  f[1 + dir] += p;
  f[1 + D] = v * (u[1 + D] + p);
}

template <int D, typename T>
__device__ __forceinline__ void FluxOfState(T* f, const State<D, T>& s, int dir) {
  f[0] = s.m[dir];
#pragma unroll
  for (int d = 0; d < D; ++d) f[1 + d] = s.u * s.m[d];
  f[1 + dir] += s.p;
  f[1 + D] = s.u * (s.E + s.p);
}

template <int D, typename T>
__device__ __forceinline__ void ConsOf(T* q, const State<D, T>& s) {
  q[0] = s.rho;
#pragma unroll
  for (int d = 0; d < D; ++d) q[1 + d] = s.m[d];
  q[1 + D] = s.E;
}

template <typename T> __device__ __forceinline__ T Min(T a, T b) { return a < b ? a : b; }
template <typename T> __device__ __forceinline__ T Max(T a, T b) { return a > b ? a : b; }

// Einfeldt speeds from the states' precomputed sqrt(rho), u, h, a.
template <typename T, class S>
__device__ __forceinline__ void Einfeldt(const T gm1, const S& L, const S& R, T& sL, T& sR) {
  using M = Math<T>;
  const T oo = M::Rcp(L.sq + R.sq);
  const T roeU = fma(L.u, L.sq, R.u * R.sq) * oo;
  const T roeH = fma(L.h, L.sq, R.h * R.sq) * oo;
  const T roeA = M::Sqrt(gm1 * fma(T(-0.5) * roeU, roeU, roeH));
  sL = Min(L.u - L.a, roeU - roeA);
  sR = Max(roeU + roeA, R.u + R.a);
}

// HLL flux with Einfeldt speeds (Hll::ComputeNumericFlux, array path).
template <int D, typename T>
__device__ __forceinline__ void HllFlux(const Gas<T>& eq, T* nf, const State<D, T>& L,
                                        const State<D, T>& R, int dir) {
  constexpr int K = D + 2;
  T s0, s1;
  Einfeldt<T>(eq.gm1, L, R, s0, s1);
  T fL[K], fR[K];
  FluxOfState<D, T>(fL, L, dir);
  FluxOfState<D, T>(fR, R, dir);
  const T sL = Min(s0, T(0));
  const T sR = Max(s1, T(0));
  const T sLsR = sL * sR;
  T ds = sR - sL;
  ds = (ds > T(0)) ? ds : T(1);
  const T ids = Math<T>::Rcp(ds);
  // (sR fL - sL fR + sL sR (qR - qL)) / ds with the three weights divided once
  const T wL = sR * ids, wR = sL * ids, wq = sLsR * ids;
  T qL[K], qR[K];
  ConsOf<D, T>(qL, L);
  ConsOf<D, T>(qR, R);
#pragma unroll
  for (int k = 0; k < K; ++k) nf[k] = fma(wL, fL[k], fma(-wR, fR[k], wq * (qR[k] - qL[k])));
}

// Half the limited slope (what the predictor adds and subtracts).  Van Leer:
// (2 sL sR / (sL + sR)) / 2 = sL sR / (sL + sR), the factors 2 and 1/2 being
// exact they are left out.
template <typename T>
__device__ __forceinline__ T HalfSlope(int limiter, T qL, T qM, T qR) {
  const T sL = qM - qL;
  const T sR = qR - qM;
  if (limiter == 0) {  // van Leer
    const T c = sL * sR;
    return (c > T(0)) ? Math<T>::Div(c, sL + sR) : T(0);
  }
  if (limiter == 1) {  // MinMod
    return T(0.5) * ((sR > T(0)) ? Max(T(0), Min(sL, sR)) : Min(T(0), Max(sL, sR)));
  }
  if (limiter == 2) return T(0.25) * (sL + sR);  // NoLimiter: half of 0.5 (sL + sR)
  return T(0);  // NoGradient
}

// MUSCL-Hancock predictor of one cell: its left-face and right-face states.
template <int D, typename T>
__device__ __forceinline__ void PredictBoth(const Gas<T>& eq, State<D, T>& recL,
                                            State<D, T>& recR, const T* q0, const T* q1,
                                            const T* q2, int limiter, T lambda_half,
                                            int dir) {
  constexpr int K = D + 2;
  T uL[K], uR[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const T hs = HalfSlope<T>(limiter, q0[k], q1[k], q2[k]);
    uL[k] = q1[k] - hs;
    uR[k] = q1[k] + hs;
  }
  T fL[K], fR[K];
  FluxOfCons<D, T>(eq, fL, uL, dir);
  FluxOfCons<D, T>(eq, fR, uR, dir);
  T a[K], b[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const T df = fL[k] - fR[k];
    b[k] = fma(lambda_half, df, uR[k]);
    a[k] = fma(lambda_half, df, uL[k]);
  }
  Prepare<D, T>(eq, recR, b, dir);
  Prepare<D, T>(eq, recL, a, dir);
}

// Cell data of the stable-dt estimate.
template <typename T> struct Wave {
  T sq;
  T u;
  T h;
  T a;
};

template <int D, typename T>
__device__ __forceinline__ Wave<T> MakeWave(const Gas<T>& eq, const T* u, int dir) {
  State<D, T> s;
  Prepare<D, T>(eq, s, u, dir);
  return Wave<T>{s.sq, s.u, s.h, s.a};
}

// The waves of a cell in the D directions from one preparation: the same
// operations as Prepare (so each wave equals MakeWave's), with the
// direction-free part (sqrt(rho), 1/rho, h, a) computed once.
template <int D, typename T>
__device__ __forceinline__ void MakeWaves(const Gas<T>& eq, const T* u, Wave<T>* w) {
  using M = Math<T>;
  const T rho = u[0];
  const T rs = M::Rsqrt(rho);
  const T ir = rs * rs;
  const T sq = rho * rs;
  const T ke = T(0.5) * SquaredNorm<D, T>(u + 1) * ir;
  const T p = (u[1 + D] - ke) * eq.gm1;
  const T h = (u[1 + D] + p) * ir;
  const T a = M::Sqrt(eq.gamma * p * ir);
#pragma unroll
  for (int d = 0; d < D; ++d) w[d] = Wave<T>{sq, u[1 + d] * ir, h, a};
}

template <typename T>
__device__ __forceinline__ T FaceMaxSpeed(const Gas<T>& eq, const Wave<T>& L, const Wave<T>& R) {
  T sL, sR;
  Einfeldt<T>(eq.gm1, L, R, sL, sR);
  return Max(Max(T(0), fabs(sL)), fabs(sR));
}

}  // namespace fast
}  // namespace fvs
