// fvs_kernels_fast.cu -- the fast FP64 and the mixed-precision sweeps.
//
// Fast FP64: the reference's formulas with shared reciprocals, FMA
// contraction and Newton-refined reciprocal / reciprocal-square-root seeds;
// per call within ~1e-13 relative of the exact flavour.
// Mixed: MUSCL-Hancock reconstruction, limiter, HLLE flux and the CFL
// speeds in FP32; state storage and the conservative update
// U' = U + dt/dx (F_L - F_R) in FP64 (the fluxes are widened to FP64 before
// the update, so mass, momentum and energy are conserved to FP64 round-off).
#include "fvs_internal.h"
#include "fvs_physics_fast.cuh"
#include "fvs_stable.cuh"
#include "fvs_sweep.cuh"

namespace fvs {

template <int D, typename T> struct FastBase {
  using Real = T;
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
  static __device__ __forceinline__ void ToCell(T* c, const double* u) {
#pragma unroll
    for (int k = 0; k < K; ++k) c[k] = T(u[k]);
  }
  static __device__ __forceinline__ void Predict(const Gas& eq, Rec& recL, Rec& recR,
                                                 const T* q0, const T* q1, const T* q2,
                                                 int limiter, double lambda_half, int dir) {
    fast::PredictBoth<D, T>(eq, recL, recR, q0, q1, q2, limiter, T(lambda_half), dir);
  }
  static __device__ __forceinline__ void HllFlux(const Gas& eq, double* F, const Rec& L,
                                                 const Rec& R, int dir) {
    T nf[K];
    fast::HllFlux<D, T>(eq, nf, L, R, dir);
#pragma unroll
    for (int k = 0; k < K; ++k) F[k] = double(nf[k]);
  }
  static __device__ __forceinline__ Wave MakeWave(const Gas& eq, const T* u, int dir) {
    return fast::MakeWave<D, T>(eq, u, dir);
  }
  static __device__ __forceinline__ double FaceMaxSpeed(const Gas& eq, const Wave& L,
                                                        const Wave& R) {
    return double(fast::FaceMaxSpeed<T>(eq, L, R));
  }
};

template <int D> struct Fast64Policy : FastBase<D, double> {};
template <int D> struct Mixed32Policy : FastBase<D, float> {};

cudaError_t LaunchSweepFast(const SweepArgs& a, cudaStream_t s) {
  switch (a.rank) {
  case 1:
    return LaunchSweepT<1, Fast64Policy>(a, s);
  case 2:
    return LaunchSweepT<2, Fast64Policy>(a, s);
  default:
    return LaunchSweepT<3, Fast64Policy>(a, s);
  }
}

cudaError_t LaunchSweepMixed(const SweepArgs& a, cudaStream_t s) {
  switch (a.rank) {
  case 1:
    return LaunchSweepT<1, Mixed32Policy>(a, s);
  case 2:
    return LaunchSweepT<2, Mixed32Policy>(a, s);
  default:
    return LaunchSweepT<3, Mixed32Policy>(a, s);
  }
}

cudaError_t LaunchStableDtFast(const StableDtArgs& a, cudaStream_t s) {
  return LaunchStableDtT<Fast64Policy>(a, s);
}

cudaError_t LaunchStableDtMixed(const StableDtArgs& a, cudaStream_t s) {
  return LaunchStableDtT<Mixed32Policy>(a, s);
}

}  // namespace fvs
