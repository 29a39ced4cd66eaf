// fvs_df64.cuh -- "double-float" arithmetic: a value is the unevaluated sum
// hi + lo of two FP32 numbers (|lo| <= ulp(hi)/2), carried through FP32
// error-free transformations (Dekker, "A floating-point technique for
// extending the available precision", 1971; Knuth's TwoSum; the FMA form of
// TwoProduct).  About 48 significant bits (relative error ~4e-15 per
// operation) computed on the FP32 pipes, which on GB300 issue 64 times as many
// operations per SM and clock as the FP64 pipe.
//
// Every FP32 operation of the error-free transformations uses an explicitly
// rounded intrinsic (__fadd_rn, __fmul_rn, __fmaf_rn), so FMA contraction by
// the compiler cannot change them.  Conversions from double split into hi and
// the rounded remainder (one FP64 subtraction); conversions to double add the
// two widened parts (one FP64 addition).  The exponent range is FP32's.
#pragma once

#include "fvs_convert.cuh"
#include "fvs_physics_fast.cuh"

namespace fvs {

struct df64 {
  float hi, lo;
  df64() = default;
  __device__ __forceinline__ df64(float h, float l) : hi(h), lo(l) {}
  __device__ __forceinline__ df64(int i) : hi(static_cast<float>(i)), lo(0.0f) {}
  __device__ __forceinline__ df64(double x) {
    hi = DoubleToFloatBits(x);
    lo = DoubleToFloatBits(x - FloatToDoubleBits(hi));
  }
  __device__ __forceinline__ operator double() const {
    return FloatToDoubleBits(hi) + FloatToDoubleBits(lo);
  }
};

namespace dfops {

// s + e == a + b exactly (Knuth)
__device__ __forceinline__ df64 TwoSum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float v = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v));
  return df64(s, e);
}

// s + e == a + b exactly when |a| >= |b| (Dekker)
__device__ __forceinline__ df64 QuickTwoSum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float e = __fsub_rn(b, __fsub_rn(s, a));
  return df64(s, e);
}

}  // namespace dfops

__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  df64 s = dfops::TwoSum(a.hi, b.hi);
  const df64 t = dfops::TwoSum(a.lo, b.lo);
  s.lo = __fadd_rn(s.lo, t.hi);
  s = dfops::QuickTwoSum(s.hi, s.lo);
  s.lo = __fadd_rn(s.lo, t.lo);
  return dfops::QuickTwoSum(s.hi, s.lo);
}

__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }

__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return dfops::QuickTwoSum(p, e);
}

__device__ __forceinline__ df64& operator+=(df64& a, df64 b) { return a = a + b; }
__device__ __forceinline__ df64& operator*=(df64& a, df64 b) { return a = a * b; }

__device__ __forceinline__ bool operator<(df64 a, df64 b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}
__device__ __forceinline__ bool operator>(df64 a, df64 b) { return b < a; }
__device__ __forceinline__ bool operator<=(df64 a, df64 b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(df64 a, df64 b) { return !(a < b); }
__device__ __forceinline__ bool operator==(df64 a, df64 b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(df64 a, df64 b) { return !(a == b); }

__device__ __forceinline__ df64 fabs(df64 a) { return a.hi < 0.0f ? -a : a; }
__device__ __forceinline__ df64 fma(df64 a, df64 b, df64 c) { return a * b + c; }

namespace fast {

template <> struct Math<df64> {
  // 1/a: y = 1/a.hi rounded to nearest, the residual r = 1 - a y from FMAs
  // (for a correctly rounded y, 1 - a.hi y is exact in FP32), and
  // 1/a = y / (1 - r) = y (1 + r + r^2 + ...) with the correction y (r + r^2)
  // in the low word: relative error ~ r^3 + 2^-48.
  static __device__ __forceinline__ df64 Rcp(df64 a) {
    const float y = __frcp_rn(a.hi);
    const float r = __fmaf_rn(-a.lo, y, __fmaf_rn(-a.hi, y, 1.0f));
    return dfops::QuickTwoSum(y, __fmul_rn(y, __fmaf_rn(r, r, r)));
  }
  // a/b as a times the reciprocal (relative error ~2^-46)
  static __device__ __forceinline__ df64 Div(df64 a, df64 b) { return a * Rcp(b); }
  // 1/sqrt(a), a > 0: y = rsqrt(a.hi), r = 1 - a y^2 in double-float, and
  // 1/sqrt(a) = y (1 - r)^(-1/2) = y (1 + r/2 + 3 r^2/8 + ...); the
  // correction goes to the low word.
  static __device__ __forceinline__ df64 Rsqrt(df64 a) {
    const float y = rsqrtf(a.hi);
    const df64 t = df64(y, 0.0f) * df64(y, 0.0f);
    const df64 r = df64(1) - a * t;
    const float c = __fmaf_rn(__fmul_rn(0.375f, r.hi), r.hi, __fmul_rn(0.5f, r.hi));
    return dfops::QuickTwoSum(y, __fmul_rn(y, c));
  }
  // sqrt(a) for a >= 0 (0 for a <= 0): a times the reciprocal square root
  // (relative error ~2^-46).
  static __device__ __forceinline__ df64 Sqrt(df64 a) {
    if (!(a.hi > 0.0f)) return df64(0);
    return a * Rsqrt(a);
  }
};

}  // namespace fast
}  // namespace fvs
