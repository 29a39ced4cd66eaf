// fvs_roots.cuh -- powers of pressure ratios for the exact Riemann solver
// (host and device, so that a host check can compare them with pow()).
#pragma once

#include <cmath>

#include "fvs_convert.cuh"

namespace fvs {
namespace riemann {

// Powers of pressure ratios.  The solver raises ratios to z = (gamma-1)/(2 gamma)
// and to exponents derived from it.  Where n = 2 gamma / (gamma - 1) is an
// integer (7 for gamma = 1.4, 5 for 5/3, 12 for 1.2) they are all powers of
// r = x^(-1/n): x^z = x r^(n-1), x^(z-1) = x^(-(gamma+1)/(2 gamma)) = r^(n-1),
// x^(1/gamma) = x^((n-2)/n) = x r^2, and the integer powers b^(n-2) =
// b^(2/(gamma-1)) and b^n = b^(2 gamma/(gamma-1)).  r is Newton's method for
// r^-n = x, r <- r (1 + (1 - x r^n) / n) (no division), from an FP32 estimate
// (relative error ~1e-6): two steps square the error twice, below FP64
// rounding.  That is ~20 FP64 operations where pow() evaluates a logarithm
// and an exponential in extended precision; the results are within 2e-14
// relative of pow() with the solver's FP64 exponents, which are themselves
// roundings of the rationals above (tests/cpp/root_check.cu).  Other gammas,
// and ratios outside [1e-30, 1e30], take pow() with the reference's
// exponents.
__host__ __device__ inline int RootOrder(double gamma) {
  if (!(gamma > 1.0)) return 0;
  const double q = 2.0 * gamma / (gamma - 1.0);
  if (!(q > 2.5 && q < 64.5)) return 0;
  const int k = static_cast<int>(q + 0.5);
  return fabs(q - k) <= 1e-12 * k ? k : 0;
}

// b^k for 1 <= k (square and multiply).
__host__ __device__ __forceinline__ double IPow(double b, int k) {
  double result = 1.0;
  bool first = true;
  while (k) {
    if (k & 1) {
      result = first ? b : result * b;
      first = false;
    }
    k >>= 1;
    if (k) b *= b;
  }
  return result;
}

struct Powers {
  int n;
  double inv_n;
  __host__ __device__ explicit Powers(int root_n) : n(root_n), inv_n(root_n > 0 ? 1.0 / root_n : 0.0) {}
  // true where x^(-1/n) replaces pow()
  __host__ __device__ bool Fast(double x) const { return n > 0 && x > 1e-30 && x < 1e30; }
  // x^(-1/n) for Fast(x)
  __host__ __device__ double RecipRoot(double x) const {
#ifdef __CUDA_ARCH__
    // the estimate's conversions on the integer pipe (the FP64 pipe is the
    // solver's bottleneck)
    const float xf = DoubleToFloatBits(x);
    double r = FloatToDoubleBits(exp2f(-__log2f(xf) * static_cast<float>(inv_n)));
#else
    double r = static_cast<double>(exp2f(-log2f(static_cast<float>(x)) * static_cast<float>(inv_n)));
#endif
#pragma unroll
    for (int it = 0; it < 2; ++it) {
      const double e = fma(-x, IPow(r, n), 1.0);
      r = fma(r, e * inv_n, r);
    }
    return r;
  }
  // x^z (z = the caller's (gamma-1)/(2 gamma) expression, for pow())
  __host__ __device__ double Z(double x, double z) const {
    return Fast(x) ? x * IPow(RecipRoot(x), n - 1) : pow(x, z);
  }
  // x^(z-1) = x^(-(gamma+1)/(2 gamma))
  __host__ __device__ double ZMinus1(double x, double e) const {
    return Fast(x) ? IPow(RecipRoot(x), n - 1) : pow(x, e);
  }
  // x^(1/gamma)
  __host__ __device__ double InvGamma(double x, double e) const {
    if (!Fast(x)) return pow(x, e);
    const double r = RecipRoot(x);
    return x * (r * r);
  }
  // b^(2/(gamma-1)) = b^(n-2) and b^(2 gamma/(gamma-1)) = b^n
  __host__ __device__ double N2(double b, double e) const { return n > 0 ? IPow(b, n - 2) : pow(b, e); }
  __host__ __device__ double N(double b, double e) const { return n > 0 ? IPow(b, n) : pow(b, e); }
};

struct Star {
  double p;
  double u;
  int iterations;
  int converged;
  int fallback;  // the learned start value was rejected
};

}  // namespace riemann
}  // namespace fvs
