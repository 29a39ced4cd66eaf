// Host check of the exact Riemann solver's powers of pressure ratios
// (csrc/fvs_roots.cuh), compiled by nvcc as host code: for gamma = 1.4, 5/3
// and 1.2 (n = 7, 5, 12) every power the solver takes -- x^z, x^(z-1),
// x^(1/gamma) and the integer powers b^(2/(gamma-1)), b^(2 gamma/(gamma-1))
// -- against pow() with the solver's own FP64 exponent expressions, over
// log-uniform ratios in [1e-12, 1e12].  Prints the largest relative
// difference per power (and in ulps) and exits 1 when one exceeds 2e-14;
// also checks RootOrder and the pow() fallbacks.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

#include "fvs_roots.cuh"

namespace {

int64_t Ordered(double x) {
  int64_t b;
  std::memcpy(&b, &x, 8);
  return b < 0 ? INT64_MIN - b : b;
}

double Ulps(double got, double ref) {
  const int64_t a = Ordered(got), b = Ordered(ref);
  return static_cast<double>(a > b ? a - b : b - a);
}

double Rel(double got, double ref) { return std::fabs(got - ref) / std::fabs(ref); }

}  // namespace

int main() {
  using fvs::riemann::Powers;
  using fvs::riemann::RootOrder;
  int fail = 0;
  const double gammas[] = {1.4, 5.0 / 3.0, 1.2};
  const int orders[] = {7, 5, 12};
  for (int gi = 0; gi < 3; ++gi) {
    const double g = gammas[gi];
    const int n = RootOrder(g);
    if (n != orders[gi]) {
      std::printf("RootOrder(%g) = %d, expected %d\n", g, n, orders[gi]);
      fail = 1;
      continue;
    }
    const Powers pw(n);
    const double gp1 = g + 1.0, gm1 = g - 1.0;
    const double z = 0.5 * gm1 / g, dz = -0.5 * gp1 / g;  // the solver's exponents
    const double zs = gm1 / (2.0 * g), ig = 1 / g, e2 = 2.0 / gm1, en = 2.0 * g / gm1;
    std::mt19937_64 rng(1234 + gi);
    std::uniform_real_distribution<double> lg(-12.0, 12.0), base(0.05, 3.0);
    double worst[6] = {0, 0, 0, 0, 0, 0}, worst_ulps[6] = {0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 2000000; ++k) {
      const double x = std::pow(10.0, lg(rng));
      const double b = base(rng);
      const double got[6] = {pw.Z(x, z), pw.Z(x, zs), pw.ZMinus1(x, dz), pw.InvGamma(x, ig),
                             pw.N2(b, e2), pw.N(b, en)};
      const double ref[6] = {std::pow(x, z), std::pow(x, zs), std::pow(x, dz), std::pow(x, ig),
                             std::pow(b, e2), std::pow(b, en)};
      for (int i = 0; i < 6; ++i) {
        const double r = Rel(got[i], ref[i]), u = Ulps(got[i], ref[i]);
        worst[i] = r > worst[i] ? r : worst[i];
        worst_ulps[i] = u > worst_ulps[i] ? u : worst_ulps[i];
      }
    }
    // Most of the difference is pow()'s: the solver's exponents are FP64
    // roundings of the rationals 1/n, -(n-1)/n, (n-2)/n, n-2 and n, off by up
    // to ~2^-52 relative, which moves x^e by |e ln x| of that.
    std::printf("gamma %.6f n %d max relative (ulps): x^z %.1e (%.0f) x^z' %.1e (%.0f) "
                "x^(z-1) %.1e (%.0f) x^(1/g) %.1e (%.0f) b^(n-2) %.1e (%.0f) b^n %.1e (%.0f)\n",
                g, n, worst[0], worst_ulps[0], worst[1], worst_ulps[1], worst[2], worst_ulps[2],
                worst[3], worst_ulps[3], worst[4], worst_ulps[4], worst[5], worst_ulps[5]);
    for (int i = 0; i < 6; ++i) fail |= !(worst[i] <= 2e-14);
  }
  // no root order: gamma whose 2 gamma / (gamma - 1) is not an integer
  const double others[] = {1.3, 1.35, 1.0, 0.5, 1.0 + 1e-12};
  for (double g : others) {
    if (RootOrder(g) != 0) {
      std::printf("RootOrder(%g) = %d, expected 0\n", g, RootOrder(g));
      fail = 1;
    }
  }
  // outside the estimate's range and with n = 0: pow() itself
  const Powers none(0), seven(7);
  const double z = 0.5 * 0.4 / 1.4;
  fail |= !(none.Z(2.5, z) == std::pow(2.5, z));
  fail |= !(seven.Z(1e-35, z) == std::pow(1e-35, z));
  fail |= !(seven.Z(1e35, z) == std::pow(1e35, z));
  std::printf("fail %d\n", fail);
  return fail;
}
