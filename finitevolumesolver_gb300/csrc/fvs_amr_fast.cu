// fvs_amr_fast.cu -- AMR patch kernels of the fast FP64 and mixed-precision
// flavours (the policies of the uniform-grid sweeps, fvs_policy_fast.cuh).
#include "fvs_amr.h"
#include "fvs_amr_kernels.cuh"
#include "fvs_policy_fast.cuh"

namespace fvs {
namespace amr {

cudaError_t LaunchPatchSweepFast(int dir, const PatchSweepArgs& a, int grid, int block,
                                 cudaStream_t s) {
  return LaunchPatchSweepT<Fast64Policy>(dir, a, grid, block, s);
}

// occupancy 0 or 5: register/occupancy variant; + 10 for the x sweep with
// the lanes of a warp along x (PatchRowWarpKernel)
cudaError_t LaunchPatchSweepMixed(int dir, const PatchSweepArgs& a, int grid, int block,
                                  int occupancy, cudaStream_t s) {
  if (dir == 0 && occupancy >= 10) {
    if (occupancy == 15) return LaunchPatchRowWarpT<Mixed32PolicyOcc5>(a, grid, block, s);
    return LaunchPatchRowWarpT<Mixed32Policy>(a, grid, block, s);
  }
  if (occupancy == 5) return LaunchPatchSweepT<Mixed32PolicyOcc5>(dir, a, grid, block, s);
  return LaunchPatchSweepT<Mixed32Policy>(dir, a, grid, block, s);
}

cudaError_t LaunchPatchMaxSpeedFast(int dir, const MaxSpeedArgs& a, int grid, int block,
                                    cudaStream_t s) {
  return LaunchPatchMaxSpeedT<Fast64Policy>(dir, a, grid, block, s);
}

cudaError_t LaunchPatchMaxSpeedMixed(int dir, const MaxSpeedArgs& a, int grid, int block,
                                     cudaStream_t s) {
  return LaunchPatchMaxSpeedT<Mixed32Policy>(dir, a, grid, block, s);
}

}  // namespace amr
}  // namespace fvs
