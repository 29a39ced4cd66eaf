// Host check of fvs::DiffToDouble (csrc/fvs_convert.cuh), compiled by nvcc as
// host code: the FP32 TwoSum + integer packing must give the FP64 difference
// of the widened operands bit for bit whenever the operands' exponents differ
// by at most 28 (the exact difference then has at most 53 significant bits),
// and stay within 1 ulp of it otherwise.  Prints the counts and exits 1 on a
// violation.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

#include "fvs_convert.cuh"

namespace {

uint64_t Bits(double x) {
  uint64_t b;
  std::memcpy(&b, &x, 8);
  return b;
}

int Exponent(float x) {
  uint32_t b;
  std::memcpy(&b, &x, 4);
  return static_cast<int>((b >> 23) & 0xFF);
}

// Distance in ulps between two finite doubles of the same sign (or zero).
uint64_t UlpDistance(double a, double b) {
  const int64_t ia = static_cast<int64_t>(Bits(a)), ib = static_cast<int64_t>(Bits(b));
  const int64_t oa = ia < 0 ? INT64_MIN - ia : ia;  // monotonic order of the patterns
  const int64_t ob = ib < 0 ? INT64_MIN - ib : ib;
  return oa > ob ? static_cast<uint64_t>(oa - ob) : static_cast<uint64_t>(ob - oa);
}

}  // namespace

int main() {
  std::mt19937_64 rng(20261204);
  std::uniform_real_distribution<double> unit(1.0, 2.0);
  std::uniform_int_distribution<int> expo(-60, 60), gap(0, 40), coin(0, 1), tweak(-3, 3);
  long exact_cases = 0, exact_fail = 0, near_cases = 0, near_fail = 0;
  for (long n = 0; n < 4000000; ++n) {
    const int ea = expo(rng);
    float a = static_cast<float>((coin(rng) ? -1.0 : 1.0) * std::ldexp(unit(rng), ea));
    float b;
    const int mode = static_cast<int>(n % 4);
    if (mode == 0) {  // b near a: cancellation, carries and power-of-two results
      uint32_t ab;
      std::memcpy(&ab, &a, 4);
      ab = static_cast<uint32_t>(static_cast<int64_t>(ab) + tweak(rng) * (1 + (n % 7)));
      std::memcpy(&b, &ab, 4);
      if (coin(rng)) b = -b;
    } else if (mode == 1) {  // a power of two on one side
      b = static_cast<float>((coin(rng) ? -1.0 : 1.0) * std::ldexp(1.0, ea - gap(rng)));
    } else if (mode == 2) {
      b = static_cast<float>((coin(rng) ? -1.0 : 1.0) * std::ldexp(unit(rng), ea - gap(rng)));
    } else {  // a a power of two and a small b of its sign: s = a, e of the other sign
      a = static_cast<float>((coin(rng) ? -1.0 : 1.0) * std::ldexp(1.0, ea));
      b = std::copysign(static_cast<float>(std::ldexp(unit(rng), ea - 25 - gap(rng) % 8)), a);
    }
    if (n % 97 == 0) b = a;  // an exact zero
    const double ref = static_cast<double>(a) - static_cast<double>(b);
    const double got = fvs::DiffToDouble(a, b);
    const int g = std::abs(Exponent(a) - Exponent(b));
    if (g <= 28 || a == 0.0f || b == 0.0f) {
      ++exact_cases;
      if (Bits(got) != Bits(ref) && !(got == 0.0 && ref == 0.0)) {
        if (exact_fail < 5)
          std::printf("exact mismatch a=%a b=%a ref=%a got=%a\n", a, b, ref, got);
        ++exact_fail;
      }
    } else {
      ++near_cases;
      if ((ref < 0) != (got < 0) || UlpDistance(got, ref) > 1) {
        if (near_fail < 5) std::printf("near mismatch a=%a b=%a ref=%a got=%a\n", a, b, ref, got);
        ++near_fail;
      }
    }
  }
  // zero, inf and NaN
  const float inf = INFINITY;
  int special_fail = 0;
  special_fail += !(fvs::DiffToDouble(1.5f, 1.5f) == 0.0);
  special_fail += !(fvs::DiffToDouble(0.0f, 0.0f) == 0.0);
  special_fail += !(fvs::DiffToDouble(inf, 1.0f) == static_cast<double>(inf));
  special_fail += !(fvs::DiffToDouble(1.0f, inf) == -static_cast<double>(inf));
  special_fail += !std::isnan(fvs::DiffToDouble(inf, inf));
  special_fail += !std::isnan(fvs::DiffToDouble(NAN, 1.0f));
  std::printf("exact %ld (fail %ld) near %ld (fail %ld) special fail %d\n", exact_cases,
              exact_fail, near_cases, near_fail, special_fail);
  return (exact_fail || near_fail || special_fail || exact_cases < 1000000) ? 1 : 0;
}
