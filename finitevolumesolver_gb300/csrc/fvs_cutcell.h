// fvs_cutcell.h -- device data of the KBN cut-cell path (2-D), shared by the
// kernels and the C ABI (not part of the C ABI).
#pragma once

#include <cstdint>

#include "fvs_internal.h"

namespace fvs {

// Ghost layers of the cut-cell geometry and the stencil reach of the KBN
// sweep (MUSCL stencil of 2 plus the neighbour faces of the shielding).
constexpr int kCcGhost = 3;

// Tiles of a KBN sweep in direction d: a group of 32 consecutive grid lines
// along d (one warp) times kCcTile consecutive cells along d.  A tile is
//   regular: every cell of its stencil reach [c0-2, c1+1] has alpha 1, no
//     cell of [c0-1, c1] is cut, and every face of [c0, c1] has beta 1,
//     unshielded fraction 1 and shielded fractions 0 -- there the KBN update
//     is masked MUSCL-Hancock + HLL and U + dt/dx (f_L - f_R), with no
//     geometry to read;
//   covered: its cells have alpha 0 and its faces beta 0 (the cells stay 0
//     and add no CFL speed);
//   cut: everything else, the full KBN arithmetic.
constexpr int kCcTile = 8;
enum CcTileClass : signed char { kCcRegular = 0, kCcCovered = 1, kCcCut = 2 };

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
  // per direction: class of every tile, [NGroups(d)][NTiles(d)], and the
  // ids (group * NTiles(d) + tile) of the cut tiles
  signed char* tile_class[2];
  int* band[2];
  int nband[2];
  __host__ __device__ int NTiles(int d) const { return ((d == 0 ? nx : ny) + kCcTile - 1) / kCcTile; }
  __host__ __device__ int NGroups(int d) const { return ((d == 0 ? ny : nx) + 31) / 32; }
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
// Classifies the tiles of direction d into g.tile_class[d] (CcTileClass).
cudaError_t LaunchCutCellTileClass(const CcGeom& g, int d, cudaStream_t s);
cudaError_t LaunchCutCellReferenceStates(const CcStateArgs& a, cudaStream_t s);
// Plotfile components of rows [j0, j0 + rows): masked Complete (6),
// Boundary_X, Boundary_Y, vfrac; [9][rows][nx].
cudaError_t LaunchCutCellPlotData(const CcGeom& g, const double* cons, double gamma, int j0,
                                  int rows, double* out, cudaStream_t s);
// Fast FP64 (precision 1) and mixed (precision 2) flavours of the KBN kernels.
// A KBN sweep is two launches that write disjoint cells of `out` and feed the
// same CFL maximum: the regular and covered tiles (band = false; threads
// march segments of a.seg_len cells, a multiple of kCcTile) and the cut tiles
// (band = true; one warp per tile of g.band[dir]).  They may run concurrently.
cudaError_t LaunchCutCellReferenceStatesT(int precision, const CcStateArgs& a, cudaStream_t s);
cudaError_t LaunchCutCellSweepT(int precision, const CcSweepArgs& a, bool band, cudaStream_t s);
cudaError_t LaunchCutCellStableDtT(int precision, const CcStateArgs& a,
                                   unsigned long long* smax_out, Control* ctrl, cudaStream_t s);
cudaError_t LaunchCutCellSweep(const CcSweepArgs& a, bool band, cudaStream_t s);
cudaError_t LaunchCutCellStableDt(const CcStateArgs& a, unsigned long long* smax_out,
                                  Control* ctrl, cudaStream_t s);

}  // namespace fvs
