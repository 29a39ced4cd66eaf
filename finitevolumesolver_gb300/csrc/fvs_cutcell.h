// fvs_cutcell.h -- device data of the KBN cut-cell path (2-D), shared by the
// kernels and the C ABI (not part of the C ABI).
#pragma once

#include <cstdint>

#include "fvs_internal.h"

namespace fvs {

// Ghost layers of the cut-cell geometry and the stencil reach of the KBN
// sweep (MUSCL stencil of 2 plus the neighbour faces of the shielding).
constexpr int kCcGhost = 3;

// Geometry over the grid grown by kCcGhost layers (component-major, x
// fastest).  Cells: [NY][NX]; x faces: [NY][NX+1]; y faces: [NY+1][NX].
struct CcGeom {
  int nx, ny;
  double* alpha;
  double* beta[2];
  double* normal;  // [2][NY][NX], into the fluid
  double* center;  // [2][NY][NX], cell units relative to the cell centre
  double* us[2];
  double* sL[2];
  double* sR[2];
  double* us_rel[2];
  double* sL_rel[2];
  double* sR_rel[2];
  signed char* cut;  // IsCutCell
  __host__ __device__ int NX() const { return nx + 2 * kCcGhost; }
  __host__ __device__ int NY() const { return ny + 2 * kCcGhost; }
  __host__ __device__ int64_t CellIndex(int i, int j) const {
    return int64_t(j + kCcGhost) * NX() + (i + kCcGhost);
  }
  // face f (between cells f-1 and f along d) of transverse index t
  __host__ __device__ int64_t FaceIndex(int d, int f, int t) const {
    return d == 0 ? int64_t(t + kCcGhost) * (NX() + 1) + (f + kCcGhost)
                  : int64_t(f + kCcGhost) * NX() + (t + kCcGhost);
  }
  __device__ double Beta(int d, int f, int t) const { return beta[d][FaceIndex(d, f, t)]; }
};

struct CcGeomArgs {
  int nx, ny;
  double x0, y0, dx, dy;
  int ncirc;
  const double* circles;  // device, [ncirc][3]
  double* alpha;
  double* betax;
  double* betay;
  double* normal;
  double* center;
};

struct CcStateArgs {
  CcGeom g;
  const double* in;  // conservative state [4][ny][nx]
  int bc[2];
  double gamma;
  double* refs;      // reference states [6][NY][NX]
};

struct CcSweepArgs {
  CcStateArgs s;
  double* out;
  int dir;
  int limiter;
  int seg_len;
  double dx;
  const double* dt_ptr;
  double dt_scale;
  double dt_value;
  unsigned long long* smax_out;
  Control* ctrl;
  int prev_check;
  double prev_dx;
  int occupancy;  // 0, or resident 128-thread blocks per SM the kernel is compiled for
                  // (FP64: 3, FP32 reconstruction: 4)
  int skip_cfl;   // FP64 flavours: no CFL speeds (a step's first sweep)
};

cudaError_t LaunchCutCellGeometry(const CcGeomArgs& a, const CcGeom& g, cudaStream_t s);
cudaError_t LaunchCutCellReferenceStates(const CcStateArgs& a, cudaStream_t s);
// Plotfile components of rows [j0, j0 + rows): masked Complete (6),
// Boundary_X, Boundary_Y, vfrac; [9][rows][nx].
cudaError_t LaunchCutCellPlotData(const CcGeom& g, const double* cons, double gamma, int j0,
                                  int rows, double* out, cudaStream_t s);
// Fast FP64 (precision 1) and mixed (precision 2) flavours of the KBN kernels.
cudaError_t LaunchCutCellReferenceStatesT(int precision, const CcStateArgs& a, cudaStream_t s);
cudaError_t LaunchCutCellSweepT(int precision, const CcSweepArgs& a, cudaStream_t s);
cudaError_t LaunchCutCellStableDtT(int precision, const CcStateArgs& a,
                                   unsigned long long* smax_out, Control* ctrl, cudaStream_t s);
cudaError_t LaunchCutCellSweep(const CcSweepArgs& a, cudaStream_t s);
cudaError_t LaunchCutCellStableDt(const CcStateArgs& a, unsigned long long* smax_out,
                                  Control* ctrl, cudaStream_t s);

}  // namespace fvs
