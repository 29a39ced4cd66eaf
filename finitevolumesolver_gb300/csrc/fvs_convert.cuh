// fvs_convert.cuh -- FP64 <-> FP32 conversions for the mixed-precision
// kernels.
#pragma once

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
