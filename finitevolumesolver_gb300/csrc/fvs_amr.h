// fvs_amr.h -- device tables and kernel arguments of the batched AMR patch
// update (2-D, refinement ratio 2, 2 ghost layers).
//
// Storage: every level keeps its patches' ghosted blocks back to back in one
// array per component (structure of arrays over the level):
//   value(c, cell) = level_buffer[c * ncells + cell],
// and a patch block is (nx + 4) x (ny + 4) cells, x fastest.  A sweep reads
// and writes whole rows (x sweeps) or columns (y sweeps) of patches; the work
// of a sweep is the level's list of rows, processed by one persistent launch.
#pragma once

#include <cstdint>

#include "fvs_internal.h"

namespace fvs {
namespace amr {

constexpr int kGhost = 2;
constexpr int kMaxLevels = 4;
constexpr int kComp = 4;  // rho, m_x, m_y, E
// per coarse step at most 4 sweeps on each of 1 + 2 + 4 + 8 level subcycles
constexpr int kMaxSweeps = 4 * 15;

// Where a sweep reads a row's halo cells (positions -2, -1, n, n+1 along the
// row): cell `src` of the same level's current buffer (src >= 0) or cell
// -src-1 of the next coarser level (piecewise-constant injection).  Reading
// them there at sweep time is the ghost fill of the row's two end strips.
// One row (x sweep) or column (y sweep) of one patch.
struct Row {
  int32_t base;     // storage index of the row's first ghost cell (interior -2)
  int32_t stride;   // 1 for x rows, the patch pitch for y columns
  int32_t n;        // interior cells
  int32_t cap_end;  // captures of this row: [previous row's cap_end, cap_end)
  int32_t halo[4];  // sources of the halo cells -2, -1, n, n+1
  int32_t flip;     // bit h: halo cell h is a reflective boundary's image (its
                    // momentum along the row is negated)
};

// A segment [j0, j1) of a row, the work item of a sweep thread: it computes
// the faces j0..j1 and updates the cells j0..j1-1.  A row split into S
// segments gives S threads per row (the autotuner picks S).  The segment's
// register captures are caps[cap_begin, cap_end): faces in [j0, j1), and face
// n for the row's last segment.
struct Seg {
  int32_t base;
  int32_t stride;
  int32_t j0, j1;
  int32_t cap_begin, cap_end;
  int32_t n;        // the row's interior cells
  int32_t halo[4];  // the row's halo sources (Row::halo)
  int32_t flip;     // Row::flip
};

constexpr int kSplits = 4;  // rows are offered split into 1, 2, 4 or 8 segments
constexpr int kSplitOf[kSplits] = {1, 2, 4, 8};

// A flux-register capture: face `face` (0..n, between cells face-1 and face)
// of a row adds dt_split * F to register entry `dst` (K doubles).
struct Cap {
  int32_t face;
  int32_t dst;
};


// Reflux of one coarse cell from `count` register slots starting at
// `first`; the slot's sign is +1 for the cell's low face, -1 for its high face.
struct RefluxCell {
  int32_t cell;
  int32_t first;
  int32_t count;
  int32_t pad;
};

// Average-down of the fine 2 x 2 block whose lower-left cell is `fine`.
struct AvgDown {
  int32_t coarse;
  int32_t fine;
  int32_t pitch;  // fine patch pitch (cells to the next fine row)
  int32_t pad;
};

// Per-run control block (device).
struct AmrControl {
  double t;
  double dt;
  double t_end;
  double cfl;
  double failure_dt;   // > 0: next step uses this instead of the stable dt
  double dt_override;  // > 0: this step uses dt_override, no checks
  unsigned long long smax_stable[kMaxLevels][2];
  unsigned long long smax_sweep[kMaxSweeps];
  int failed;          // this step failed a per-sweep check
  int status;          // StatusBits of the committed steps
  int step_status;
  int nsweeps;
};

// Description of one sweep within the coarse step (device, constant).
struct SweepInfo {
  int level;
  double scale;  // split dt = scale * coarse dt
};

struct PatchSweepArgs {
  const double* in;
  double* out;
  int32_t ncells;  // component stride of the level
  const double* coarse;   // the next coarser level's state (halo injection)
  int32_t coarse_ncells;
  const Seg* segs;
  int32_t nsegs;
  const Cap* caps;
  double* reg;     // register entries of the captures
  double gamma;
  double dx;
  int limiter;
  const double* dt_ptr;  // coarse dt (device)
  double dt_scale;       // split dt = dt_scale * (*dt_ptr)
  unsigned long long* smax_out;  // this sweep's max signal speed (bits)
  AmrControl* ctrl;
  // x sweeps with the lanes of a warp along x (PatchRowWarpKernel): the
  // level's rows (segs, one segment per row) laid end to end as slots,
  // n + 2 per row (cells -1..n); slot_row[s] is slot s's row, row_slot0[r]
  // row r's first slot
  const int32_t* slot_row;
  const int32_t* row_slot0;
  int64_t nslots;
};

// Slots of a row-warp sweep: warp w takes slots kRowWarpStep * w ..
// kRowWarpStep * w + 31 and owns (updates, captures, CFL) the middle 30.
constexpr int kRowWarpStep = 30;

struct MaxSpeedArgs {
  const double* in;
  int32_t ncells;
  const double* coarse;
  int32_t coarse_ncells;
  const Seg* segs;  // the level's rows in this direction, split into segments
  int32_t nsegs;
  double gamma;
  unsigned long long* smax_out;
};

// Launchers (fvs_amr_exact.cu: exact FP64 and the table kernels, compiled
// with -fmad=false; fvs_amr_fast.cu: fast FP64 and mixed).  `grid` is the
// number of persistent blocks.
cudaError_t LaunchPatchSweepExact(int dir, const PatchSweepArgs& a, int grid, int block,
                                  cudaStream_t s);
cudaError_t LaunchPatchSweepFast(int dir, const PatchSweepArgs& a, int grid, int block,
                                 cudaStream_t s);
// occupancy: 0 (registers as needed) or 5 (compiled for 5 resident blocks)
cudaError_t LaunchPatchSweepMixed(int dir, const PatchSweepArgs& a, int grid, int block,
                                  int occupancy, cudaStream_t s);
cudaError_t LaunchPatchMaxSpeedExact(int dir, const MaxSpeedArgs& a, int grid, int block,
                                     cudaStream_t s);
cudaError_t LaunchPatchMaxSpeedFast(int dir, const MaxSpeedArgs& a, int grid, int block,
                                    cudaStream_t s);
cudaError_t LaunchPatchMaxSpeedMixed(int dir, const MaxSpeedArgs& a, int grid, int block,
                                     cudaStream_t s);
cudaError_t LaunchReflux(double* coarse, int32_t n_coarse, const double* reg,
                         const RefluxCell* cells, int32_t ncells, const float* signs, double dx,
                         cudaStream_t s);
cudaError_t LaunchAverageDown(double* coarse, int32_t n_coarse, const double* fine,
                              int32_t n_fine, const AvgDown* e, int32_t count, cudaStream_t s);
struct LevelDx {
  double dx[kMaxLevels];
};
cudaError_t LaunchAmrDt(AmrControl* ctrl, int nlevels, LevelDx dx, cudaStream_t s);
cudaError_t LaunchAmrEndStep(AmrControl* ctrl, const SweepInfo* sweeps, int nsweeps,
                             LevelDx dx, cudaStream_t s);

}  // namespace amr
}  // namespace fvs
