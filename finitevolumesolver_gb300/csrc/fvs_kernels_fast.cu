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
#include "fvs_policy_fast.cuh"
#include "fvs_stable.cuh"
#include "fvs_sweep.cuh"

namespace fvs {

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

template <template <int> class PT> cudaError_t LaunchSweepMixedT(const SweepArgs& a, cudaStream_t s) {
  switch (a.rank) {
  case 1:
    return LaunchSweepT<1, PT>(a, s);
  case 2:
    return LaunchSweepT<2, PT>(a, s);
  default:
    return LaunchSweepT<3, PT>(a, s);
  }
}

// occupancy: 0, 4, 5 = register/occupancy variant (x sweeps with lanes along
// x); 10, 14, 15 = the same variants with the marching kernel in x.
cudaError_t LaunchSweepMixed(const SweepArgs& a, cudaStream_t s) {
  // reflective rows: the marching kernel (its loads reflect ghost states)
  if (a.dir == 0 && (a.occupancy >= 10 || a.bc == 2)) {
    switch (a.occupancy) {
    case 4:
    case 14:
      return LaunchSweepMixedT<Mixed32PolicyMarchXOcc4>(a, s);
    case 5:
    case 15:
      return LaunchSweepMixedT<Mixed32PolicyMarchXOcc5>(a, s);
    default:
      return LaunchSweepMixedT<Mixed32PolicyMarchX>(a, s);
    }
  }
  switch (a.occupancy % 10) {
  case 4:
    return LaunchSweepMixedT<Mixed32PolicyOcc4>(a, s);
  case 5:
    return LaunchSweepMixedT<Mixed32PolicyOcc5>(a, s);
  default:
    return LaunchSweepMixedT<Mixed32Policy>(a, s);
  }
}

cudaError_t LaunchStableDtFast(const StableDtArgs& a, cudaStream_t s) {
  return LaunchStableDtT<Fast64Policy>(a, s);
}

cudaError_t LaunchStableDtMixed(const StableDtArgs& a, cudaStream_t s) {
  return LaunchStableDtT<Mixed32Policy>(a, s);
}

}  // namespace fvs
