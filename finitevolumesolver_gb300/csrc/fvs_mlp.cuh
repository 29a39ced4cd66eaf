// fvs_mlp.cuh -- the learned start value of the exact Riemann solver's
// Newton iteration (no counterpart in the reference).
//
// A 5 -> 64 -> 64 -> 1 perceptron with GELU activations predicts
// y = log(p* / max(pL, pR)) from five dimensionless features of the two
// states; the start value is max(pL, pR) * exp(y).  The weights are BF16
// values (stored here widened to FP32) trained on the GPU by the project's
// own kernels on Riemann problems the exact solver has solved.
//
// Features (c = max(aL, aR)):
//   x0 = log(rhoR / rhoL), x1 = log(pR / pL), x2 = (uR - uL) / c,
//   x3 = aL / c,           x4 = aR / c
// each standardised with the training set's mean and standard deviation.
#pragma once

namespace fvs {
namespace mlp {

constexpr int kIn = 5;
constexpr int kHidden = 64;
// Parameter blob layout (floats).
constexpr int kOffMean = 0;
constexpr int kOffInvStd = kOffMean + kIn;
constexpr int kOffW1 = kOffInvStd + kIn;          // [kHidden][kIn]
constexpr int kOffB1 = kOffW1 + kHidden * kIn;    // [kHidden]
constexpr int kOffW2 = kOffB1 + kHidden;          // [kHidden][kHidden]
constexpr int kOffB2 = kOffW2 + kHidden * kHidden;
constexpr int kOffW3 = kOffB2 + kHidden;          // [kHidden]
constexpr int kOffB3 = kOffW3 + kHidden;
constexpr int kParams = kOffB3 + 1;

// GELU, tanh form: 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))).
__device__ __forceinline__ float Gelu(float x) {
  const float k0 = 0.7978845608028654f;
  const float k1 = 0.044715f;
  const float t = tanhf(k0 * fmaf(k1 * x * x, x, x));
  return 0.5f * x * (1.0f + t);
}

__device__ __forceinline__ void Features(float* x, double rhoL, double uL, double pL, double aL,
                                         double rhoR, double uR, double pR, double aR) {
  const double c = aL > aR ? aL : aR;
  x[0] = static_cast<float>(log(rhoR / rhoL));
  x[1] = static_cast<float>(log(pR / pL));
  x[2] = static_cast<float>((uR - uL) / c);
  x[3] = static_cast<float>(aL / c);
  x[4] = static_cast<float>(aR / c);
}

// Network output y for standardised-on-the-fly features (FP32, CUDA cores).
__device__ __forceinline__ float Forward(const float* __restrict__ w, const float* xin) {
  float x[kIn];
#pragma unroll
  for (int i = 0; i < kIn; ++i) x[i] = (xin[i] - __ldg(w + kOffMean + i)) * __ldg(w + kOffInvStd + i);
  float h1[kHidden];
#pragma unroll 8
  for (int o = 0; o < kHidden; ++o) {
    float acc = __ldg(w + kOffB1 + o);
#pragma unroll
    for (int i = 0; i < kIn; ++i) acc = fmaf(__ldg(w + kOffW1 + o * kIn + i), x[i], acc);
    h1[o] = Gelu(acc);
  }
  float y = __ldg(w + kOffB3);
#pragma unroll 4
  for (int o = 0; o < kHidden; ++o) {
    float acc = __ldg(w + kOffB2 + o);
#pragma unroll 16
    for (int i = 0; i < kHidden; ++i) acc = fmaf(__ldg(w + kOffW2 + o * kHidden + i), h1[i], acc);
    y = fmaf(__ldg(w + kOffW3 + o), Gelu(acc), y);
  }
  return y;
}

__device__ __forceinline__ double GuessStarPressure(const float* __restrict__ w, double rhoL,
                                                    double uL, double pL, double aL, double rhoR,
                                                    double uR, double pR, double aR) {
  float x[kIn];
  Features(x, rhoL, uL, pL, aL, rhoR, uR, pR, aR);
  const float y = Forward(w, x);
  const double pref = pL > pR ? pL : pR;
  return pref * exp(static_cast<double>(y));
}

}  // namespace mlp
}  // namespace fvs
