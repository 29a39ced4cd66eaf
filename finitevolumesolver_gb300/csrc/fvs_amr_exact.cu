// fvs_amr_exact.cu -- AMR patch kernels with the reference's exact FP64
// arithmetic, and the table-driven kernels of the AMR step (ghost fill,
// reflux, average-down, dt selection, per-sweep checks).  Compiled with
// -fmad=false: the results are bit-identical to the CPU oracle's
// restatement (oracle/fvs_oracle_amr.cpp).
#include "fvs_amr.h"
#include "fvs_amr_kernels.cuh"
#include "fvs_policy_exact.cuh"

namespace fvs {
namespace amr {

cudaError_t LaunchPatchSweepExact(int dir, const PatchSweepArgs& a, int grid, int block,
                                  cudaStream_t s) {
  return LaunchPatchSweepT<ExactPolicy>(dir, a, grid, block, s);
}

cudaError_t LaunchPatchMaxSpeedExact(int dir, const MaxSpeedArgs& a, int grid, int block,
                                     cudaStream_t s) {
  return LaunchPatchMaxSpeedT<ExactPolicy>(dir, a, grid, block, s);
}

// U += s * (0.5 * (F1 + F2) - Fc) / dx for each register slot of the cell,
// in slot order (register entry 3k: coarse sum, 3k+1 and 3k+2: the fine
// sub-faces' sums).
__global__ void RefluxKernel(double* coarse, int32_t n_coarse, const double* reg,
                             const RefluxCell* cells, int32_t ncells, const float* signs,
                             double dx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncells) return;
  const RefluxCell rc = cells[i];
  for (int k = rc.first; k < rc.first + rc.count; ++k) {
    const double sign = static_cast<double>(signs[k]);
    const double* e = reg + int64_t(3 * k) * kComp;
#pragma unroll
    for (int c = 0; c < kComp; ++c) {
      const double delta = 0.5 * (e[kComp + c] + e[2 * kComp + c]) - e[c];
      double& U = coarse[int64_t(c) * n_coarse + rc.cell];
      U = U + sign * delta / dx;
    }
  }
}

cudaError_t LaunchReflux(double* coarse, int32_t n_coarse, const double* reg,
                         const RefluxCell* cells, int32_t ncells, const float* signs, double dx,
                         cudaStream_t s) {
  if (ncells == 0) return cudaSuccess;
  RefluxKernel<<<(ncells + 127) / 128, 128, 0, s>>>(coarse, n_coarse, reg, cells, ncells, signs,
                                                    dx);
  return cudaGetLastError();
}

// U_c = (((f(2i,2j) + f(2i+1,2j)) + f(2i,2j+1)) + f(2i+1,2j+1)) * 0.25
__global__ void AverageDownKernel(double* coarse, int32_t n_coarse, const double* fine,
                                  int32_t n_fine, const AvgDown* e, int32_t count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const AvgDown a = e[i];
#pragma unroll
  for (int c = 0; c < kComp; ++c) {
    const double* f = fine + int64_t(c) * n_fine + a.fine;
    const double v = (((f[0] + f[1]) + f[a.pitch]) + f[a.pitch + 1]) * 0.25;
    coarse[int64_t(c) * n_coarse + a.coarse] = v;
  }
}

cudaError_t LaunchAverageDown(double* coarse, int32_t n_coarse, const double* fine,
                              int32_t n_fine, const AvgDown* e, int32_t count, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  AverageDownKernel<<<(count + 255) / 256, 256, 0, s>>>(coarse, n_coarse, fine, n_fine, e, count);
  return cudaGetLastError();
}

// dt = min(t_end - t, cfl * stable), stable = min over levels l and
// directions d of 2^l * dx_l / smax(l, d), or the failed step's dt
// (SubcycleFineFirstSolver.hpp:100-112, RunSimulation.hpp:126-151).
__global__ void AmrDtKernel(AmrControl* ctrl, int nlevels, LevelDx dx) {
  double stable;
  if (ctrl->failure_dt > 0.0) {
    stable = ctrl->failure_dt;
  } else {
    stable = 1.7976931348623157e308;
    for (int l = 0; l < nlevels; ++l) {
      for (int d = 0; d < 2; ++d) {
        const double s = BitsToDouble(ctrl->smax_stable[l][d]);
        const double dt_l = dx.dx[l] / s;
        const double v = double(1 << l) * dt_l;
        stable = v < stable ? v : stable;
      }
    }
  }
  const double a = ctrl->t_end - ctrl->t;
  const double b = ctrl->cfl * stable;
  ctrl->dt = a < b ? a : b;
  ctrl->step_status = 0;
}

cudaError_t LaunchAmrDt(AmrControl* ctrl, int nlevels, LevelDx dx, cudaStream_t s) {
  AmrDtKernel<<<1, 1, 0, s>>>(ctrl, nlevels, dx);
  return cudaGetLastError();
}

// Per-sweep checks in execution order (the first failing sweep decides the
// retry dt, 2^l times its level's dt), then commit the step.
__global__ void AmrEndStepKernel(AmrControl* ctrl, const SweepInfo* sweeps, int nsweeps,
                                 LevelDx dx) {
  const double dt = ctrl->dt;
  int failed = 0;
  for (int s = 0; s < nsweeps && !failed; ++s) {
    const int l = sweeps[s].level;
    const double smax = BitsToDouble(ctrl->smax_sweep[s]);
    const double level_dt = dx.dx[l] / smax;
    const double split = sweeps[s].scale * dt;
    if (level_dt < split) {
      failed = 1;
      ctrl->failure_dt = level_dt * double(1 << l);
    }
  }
  ctrl->failed = failed;
  if (!failed) {
    ctrl->t = ctrl->t + dt;
    ctrl->failure_dt = 0.0;
    ctrl->status |= ctrl->step_status;
  }
}

cudaError_t LaunchAmrEndStep(AmrControl* ctrl, const SweepInfo* sweeps, int nsweeps,
                             LevelDx dx, cudaStream_t s) {
  AmrEndStepKernel<<<1, 1, 0, s>>>(ctrl, sweeps, nsweeps, dx);
  return cudaGetLastError();
}

}  // namespace amr
}  // namespace fvs
