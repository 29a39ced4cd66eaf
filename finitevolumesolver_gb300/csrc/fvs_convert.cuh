// fvs_convert.cuh -- FP64 <-> FP32 conversions for the mixed-precision
// kernels.
#pragma once

#include <cstring>

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

__host__ __device__ __forceinline__ unsigned FloatBits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  unsigned u;
  memcpy(&u, &x, sizeof(u));
  return u;
#endif
}

__host__ __device__ __forceinline__ double DoubleFromBits(unsigned long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(static_cast<long long>(b));
#else
  double d;
  memcpy(&d, &b, sizeof(d));
  return d;
#endif
}

// a - b of two FP32 numbers as an FP64 number, without the FP64 pipe.
// Knuth's TwoSum in FP32 splits the exact difference into s + e with
// s = fl32(a - b) and |e| <= ulp32(s) / 2, so e's exponent is at least 24
// below s's.  s widens exactly, and its FP64 form leaves the 29 low mantissa
// bits zero; e is added there in units of s's FP64 ulp,
// k = m_e 2^(29 - (E_s - E_e)) < 2^29 (no carry out of those bits).  Where e
// has the other sign the magnitude shrinks: the bit pattern is decremented
// by k, counted in the ulp of the binade below when s is a power of two.
// The result is the exact difference, hence equal to the FP64 subtraction
// of the widened operands, whenever the exact difference has at most 53
// significant bits (every pair whose exponents differ by at most 28);
// otherwise e is truncated to the result's FP64 ulp (within 1 ulp).  A
// subnormal s flushes to a signed zero and a subnormal e (|s| < 2^-102) is
// dropped; inf and NaN pass through.  The mixed flavour's update forms its
// flux difference here, so each component costs one FP64 operation (the
// FMA with dt/dx) instead of two.
__host__ __device__ __forceinline__ double DiffToDouble(float a, float b) {
  const float s = a - b;
  const float t = s - a;
  const float e = (a - (s - t)) + (-b - t);
  const unsigned sb = FloatBits(s), eb = FloatBits(e);
  const int es = static_cast<int>((sb >> 23) & 0xFFu);
  const int ee = static_cast<int>((eb >> 23) & 0xFFu);
  const unsigned sign = sb & 0x80000000u;
  const unsigned hi = sign | (((sb & 0x7FFFFFFFu) >> 3) + 0x38000000u);
  const unsigned lo = sb << 29;
  unsigned long long bits = (static_cast<unsigned long long>(hi) << 32) | lo;
  const bool shrink = ((sb ^ eb) & 0x80000000u) != 0u;
  // k in units of s's FP64 ulp, or of half of it where e takes a power of
  // two s into the binade below: k = m_e 2^(5 - shift)
  const int finer = (shrink && (sb & 0x7FFFFFu) == 0u) ? 1 : 0;
  const int shift = es - ee - 24 - finer;  // >= 0 for a nonzero normal e
  unsigned k = (((eb & 0x7FFFFFu) | 0x800000u) << 5) >> (shift & 31);
  k = (ee == 0 || shift < 0 || shift > 31) ? 0u : k;
  bits = shrink ? bits - k : bits + k;
  if (es == 0) bits = static_cast<unsigned long long>(sign) << 32;
  if (es == 255)
    bits = (static_cast<unsigned long long>(sign | 0x7FF00000u | ((sb & 0x7FFFFFu) >> 3)) << 32) |
           lo;
  return DoubleFromBits(bits);
}

// Narrowing / widening for code generic over the compute type T.
template <class T> __device__ __forceinline__ T NarrowTo(double x) {
  if constexpr (sizeof(T) == 4) {
    return DoubleToFloatBits(x);
  } else {
    return x;
  }
}

template <class T> __device__ __forceinline__ double Widen(T x) {
  if constexpr (sizeof(T) == 4) {
    return FloatToDoubleBits(x);
  } else {
    return x;
  }
}

}  // namespace fvs
