// fvs_kernels_df64.cu -- the double-float flavour of the uniform-grid sweep
// and stable dt: the fast flavour's formulas (fvs_physics_fast.cuh) evaluated
// in double-float arithmetic (fvs_df64.cuh) on the FP32 pipes, with the state
// and the conservative update in FP64.  About 48 significant bits per
// operation; results agree with the exact FP64 flavour to ~1e-13 relative.
#include "fvs_df64.cuh"
#include "fvs_internal.h"
#include "fvs_policy_fast.cuh"
#include "fvs_stable.cuh"
#include "fvs_sweep.cuh"

namespace fvs {

template <int D> struct Df64Policy : FastBase<D, df64> {};
// compiled for 3 resident 128-thread blocks per SM (168 registers, a few
// spilled); the autotuner picks between the two
template <int D> struct Df64PolicyOcc3 : FastBase<D, df64> {
  static constexpr int kMinBlocks = 3;
};

template <template <int> class PT> cudaError_t LaunchSweepDf64T(const SweepArgs& a, cudaStream_t s) {
  switch (a.rank) {
  case 1:
    return LaunchSweepT<1, PT>(a, s);
  case 2:
    return LaunchSweepT<2, PT>(a, s);
  default:
    return LaunchSweepT<3, PT>(a, s);
  }
}

cudaError_t LaunchSweepDf64(const SweepArgs& a, cudaStream_t s) {
  return a.occupancy == 3 ? LaunchSweepDf64T<Df64PolicyOcc3>(a, s)
                          : LaunchSweepDf64T<Df64Policy>(a, s);
}

cudaError_t LaunchStableDtDf64(const StableDtArgs& a, cudaStream_t s) {
  return LaunchStableDtT<Df64Policy>(a, s);
}

}  // namespace fvs
