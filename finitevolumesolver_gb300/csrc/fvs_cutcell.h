// fvs_cutcell.h -- device data of the KBN cut-cell path (2-D), shared by the
// kernels and the C ABI (not part of the C ABI).
#pragma once

#include <cstdint>

#include "fvs_internal.h"

namespace fvs {

// Ghost layers of the cut-cell geometry and the stencil reach of the KBN
// sweep (MUSCL stencil of 2 plus the neighbour faces of the shielding).
constexpr int kCcGhost = 3;

// Cells of a KBN sweep in direction d fall into three classes:
//   regular: every cell of its stencil reach j-2 .. j+2 along d has alpha 1,
//     none of j-1 .. j+1 is cut, and its faces j and j+1 have beta 1,
//     unshielded fraction 1 and shielded fractions 0 -- there the KBN update
//     is masked MUSCL-Hancock + HLL with every mask true and
//     U + dt/dx (f_L - f_R), with no geometry to read;
//   covered: alpha 0 (the cell stays 0; its faces have beta 0);
//   band: everything else, the full KBN arithmetic.
// Tiles group 32 consecutive grid lines (one warp) x kCcTile consecutive
// cells along d; a tile is marched by the regular kernels when it holds a
// regular cell.
constexpr int kCcTile = 8;
enum CcCellClass : signed char { kCcRegular = 0, kCcCovered = 1, kCcBand = 2 };

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
  // per direction: the class of every interior cell ([ny][nx], CcCellClass),
  // whether a tile holds a regular cell ([NGroups(d)][NTiles(d)], 0 or 1),
  // and the list of band cells (indices j * nx + i)
  signed char* cell_class[2];
  signed char* tile_regular[2];
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
  int nwords;
  const double* shapes;   // device, shape records (fvs_cutcell_geometry.cuh)
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
// Classifies the cells of direction d into g.cell_class[d] (CcCellClass)
// and marks the tiles with a regular cell in g.tile_regular[d].
cudaError_t LaunchCutCellClasses(const CcGeom& g, int d, cudaStream_t s);
cudaError_t LaunchCutCellReferenceStates(const CcStateArgs& a, cudaStream_t s);
// Plotfile components of rows [j0, j0 + rows): masked Complete (6),
// Boundary_X, Boundary_Y, vfrac; [9][rows][nx].
cudaError_t LaunchCutCellPlotData(const CcGeom& g, const double* cons, double gamma, int j0,
                                  int rows, double* out, cudaStream_t s);
// Fast FP64 (precision 1) and mixed (precision 2) flavours of the KBN kernels.
// A KBN sweep is two launches that write disjoint cells of `out` and feed the
// same CFL maximum: the regular and covered cells (band = false; tiles with a
// regular cell are marched, the FP64 flavours' threads over segments of
// a.seg_len cells, a multiple of kCcTile) and the band cells (band = true;
// one thread per cell of g.band[dir]).  They may run concurrently.
cudaError_t LaunchCutCellReferenceStatesT(int precision, const CcStateArgs& a, cudaStream_t s);
cudaError_t LaunchCutCellSweepT(int precision, const CcSweepArgs& a, bool band, cudaStream_t s);
cudaError_t LaunchCutCellStableDtT(int precision, const CcStateArgs& a,
                                   unsigned long long* smax_out, Control* ctrl, cudaStream_t s);
cudaError_t LaunchCutCellSweep(const CcSweepArgs& a, bool band, cudaStream_t s);
cudaError_t LaunchCutCellStableDt(const CcStateArgs& a, unsigned long long* smax_out,
                                  Control* ctrl, cudaStream_t s);

}  // namespace fvs
