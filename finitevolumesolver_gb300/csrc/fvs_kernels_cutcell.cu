// fvs_kernels_cutcell.cu -- KBN h-box cut-cell update on a uniform 2-D grid:
// geometry, shielded face fractions, and the exact-FP64 instantiation of the
// reference states, the fused cut-cell sweep and the masked stable dt
// (fvs_cutcell_kbn.cuh).  Compiled with -fmad=false: the results are
// bit-identical to the CPU oracle's restatement of the reference.
//
// Reference (maikel/FiniteVolumeSolver):
//   KbnCutCellMethod           include/fub/cutcell_method/KbnStabilisation.hpp:188-450
//   ComputeStableFluxes_Row    src/cutcell_method/KbnStabilisation.cpp:55-105
//   FillCutCellData__          src/AMReX/cutcell/FillCutCellData.cpp:28-118
//   IsCutCell_                 src/CutCellData.cpp:227-246
//   UpdateConservatively_Row   src/AMReX/cutcell/TimeIntegrator.cpp:65-221
//   masked MusclHancock / Hll / Einfeldt / Flux / CompleteFromCons
//       include/fub/flux_method/MusclHancockMethod.hpp:487-571,
//       include/fub/flux_method/HllMethod.hpp:295-365,
//       src/equations/perfect_gas/EinfeldtSignalVelocities.hpp:99-142,
//       src/equations/PerfectGas.cpp:79-93, 126-144
//   HllBase::SolveRiemannProblem (boundary solver)  include/fub/flux_method/HllMethod.hpp:161-184
//   MakeRotation, Reflect      include/fub/ext/Eigen.hpp:104-115, src/equations/PerfectGas.cpp:240-252
#include "fvs_cutcell.h"
#include "fvs_cutcell_geometry.cuh"
#include "fvs_cutcell_kbn.cuh"
#include "fvs_internal.h"
#include "fvs_physics_exact.cuh"
#include "fvs_sweep.cuh"

namespace fvs {
namespace cc {

// ---------------------------------------------------------------------------
// Geometry kernels

__global__ void GeometryCellKernel(CcGeomArgs a) {
  const int NX = a.nx + 2 * kCcGhost, NY = a.ny + 2 * kCcGhost;
  const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (id >= int64_t(NX) * NY) return;
  const int ii = static_cast<int>(id % NX), jj = static_cast<int>(id / NX);
  const double xa = a.x0 + double(ii - kCcGhost) * a.dx;
  const double ya = a.y0 + double(jj - kCcGhost) * a.dy;
  const ccgeom::Cell g = ccgeom::CellGeometry(xa, ya, a.dx, a.dy, a.nwords, a.shapes);
  const int64_t plane = int64_t(NX) * NY;
  a.alpha[id] = g.alpha;
  a.normal[id] = g.nx;
  a.normal[plane + id] = g.ny;
  a.center[id] = g.cx;
  a.center[plane + id] = g.cy;
}

__global__ void GeometryFaceKernel(CcGeomArgs a) {
  const int NX = a.nx + 2 * kCcGhost, NY = a.ny + 2 * kCcGhost;
  const int64_t nxf = int64_t(NX + 1) * NY;
  const int64_t nyf = int64_t(NX) * (NY + 1);
  const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  ccgeom::Iv iv[ccgeom::kMaxIntervals];
  if (id < nxf) {
    const int ii = static_cast<int>(id % (NX + 1)), jj = static_cast<int>(id / (NX + 1));
    const double xf = a.x0 + double(ii - kCcGhost) * a.dx;
    const double ya = a.y0 + double(jj - kCcGhost) * a.dy;
    const int n = ccgeom::Covered(xf, ya, ya + a.dy, true, a.nwords, a.shapes, iv);
    a.betax[id] = ccgeom::FaceFraction(iv, n, ya, ya + a.dy);
  } else if (id < nxf + nyf) {
    const int64_t k = id - nxf;
    const int ii = static_cast<int>(k % NX), jj = static_cast<int>(k / NX);
    const double yf = a.y0 + double(jj - kCcGhost) * a.dy;
    const double xa = a.x0 + double(ii - kCcGhost) * a.dx;
    const int n = ccgeom::Covered(yf, xa, xa + a.dx, false, a.nwords, a.shapes, iv);
    a.betay[k] = ccgeom::FaceFraction(iv, n, xa, xa + a.dx);
  }
}

// Closes the faces next to a cell without volume (a thin fluid gap between
// two circles can leave fluid on a face whose chord polygon has no area).
__global__ void FaceConsistencyKernel(CcGeom g) {
  const int NX = g.NX(), NY = g.NY();
  const int64_t nxf = int64_t(NX + 1) * NY;
  const int64_t nyf = int64_t(NX) * (NY + 1);
  const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (id < nxf) {
    const int ii = static_cast<int>(id % (NX + 1)), jj = static_cast<int>(id / (NX + 1));
    if (ii >= 1 && ii < NX &&
        (g.alpha[int64_t(jj) * NX + ii - 1] <= 0.0 || g.alpha[int64_t(jj) * NX + ii] <= 0.0))
      g.beta[0][id] = 0.0;
  } else if (id < nxf + nyf) {
    const int64_t k = id - nxf;
    const int ii = static_cast<int>(k % NX), jj = static_cast<int>(k / NX);
    if (jj >= 1 && jj < NY &&
        (g.alpha[int64_t(jj - 1) * NX + ii] <= 0.0 || g.alpha[int64_t(jj) * NX + ii] <= 0.0))
      g.beta[1][k] = 0.0;
  }
}

// Shielded fractions of every face with both along-direction neighbours.
__global__ void ShieldedKernel(CcGeom g, int dir) {
  const int NX = g.NX(), NY = g.NY();
  const int nd = dir == 0 ? g.nx : g.ny;
  const int nt = dir == 0 ? g.ny : g.nx;
  const int nf = nd + 2 * kCcGhost - 1;  // faces -G+1 .. nd+G-1
  const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (id >= int64_t(nf) * (nt + 2 * kCcGhost)) return;
  const int f = static_cast<int>(id % nf) - kCcGhost + 1;
  const int t = static_cast<int>(id / nf) - kCcGhost;
  (void)NX;
  (void)NY;
  const double betaL = g.Beta(dir, f - 1, t), betaM0 = g.Beta(dir, f, t), betaR = g.Beta(dir, f + 1, t);
  double betaM = betaM0;
  const double dBetaL = (0.0 < betaM - betaL) ? betaM - betaL : 0.0;  // std::max(0.0, x)
  const double dBetaR = (0.0 < betaM - betaR) ? betaM - betaR : 0.0;
  const double mx = (dBetaL < dBetaR) ? dBetaR : dBetaL;               // std::max(a, b)
  const double us = (0.0 < betaM - mx) ? betaM - mx : 0.0;
  const double ds = (dBetaR < dBetaL) ? dBetaR : dBetaL;               // std::min(a, b)
  const double sL = dBetaL - ds;
  const double sR = dBetaR - ds;
  betaM = betaM > 0 ? betaM : 1.0;
  const int64_t idx = g.FaceIndex(dir, f, t);
  g.us[dir][idx] = us;
  g.sL[dir][idx] = sL;
  g.sR[dir][idx] = sR;
  g.us_rel[dir][idx] = us / betaM;
  g.sL_rel[dir][idx] = sL / betaM;
  g.sR_rel[dir][idx] = sR / betaM;
}

// IsCutCell_ of every cell whose faces exist in the grown box.
__global__ void CutFlagKernel(CcGeom g) {
  const int NX = g.NX(), NY = g.NY();
  const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (id >= int64_t(NX) * NY) return;
  const int i = static_cast<int>(id % NX) - kCcGhost, j = static_cast<int>(id / NX) - kCcGhost;
  const double a = g.alpha[id];
  int cut;
  if (a <= 0.0) {
    cut = 0;
  } else if (a < 1.0) {
    cut = 1;
  } else {
    cut = (g.Beta(0, i, j) < 1.0 || g.Beta(0, i + 1, j) < 1.0 || g.Beta(1, j, i) < 1.0 ||
           g.Beta(1, j + 1, i) < 1.0)
              ? 1
              : 0;
  }
  g.cut[id] = static_cast<signed char>(cut);
}

// Class of interior cell (i, j) for sweeps in direction d (CcCellClass).
__global__ void CellClassKernel(CcGeom g, int d) {
  const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (id >= int64_t(g.nx) * g.ny) return;
  const int i = static_cast<int>(id % g.nx), jj = static_cast<int>(id / g.nx);
  const int t = d == 0 ? jj : i;  // grid line
  const int j = d == 0 ? i : jj;  // cell along d
  auto cell = [&](int c) { return d == 0 ? g.CellIndex(c, t) : g.CellIndex(t, c); };
  signed char k;
  if (g.alpha[cell(j)] == 0.0) {
    k = kCcCovered;
  } else {
    bool regular = true;
    for (int c = j - 2; c <= j + 2; ++c) {
      regular = regular && g.alpha[cell(c)] == 1.0;
      if (c >= j - 1 && c <= j + 1) regular = regular && g.cut[cell(c)] == 0;
    }
    for (int f = j; f <= j + 1; ++f) {
      const int64_t fi = g.FaceIndex(d, f, t);
      regular = regular && g.beta[d][fi] == 1.0 && g.us_rel[d][fi] == 1.0 &&
                g.sL_rel[d][fi] == 0.0 && g.sR_rel[d][fi] == 0.0;
    }
    k = regular ? kCcRegular : kCcBand;
  }
  g.cell_class[d][id] = k;
}

// Whether the tile (group, tile) of direction d holds a regular cell: one
// block of 32 threads, one per line of the group.
__global__ void TileRegularKernel(CcGeom g, int d) {
  const int ntl = g.NTiles(d);
  const int group = blockIdx.x / ntl, tile = blockIdx.x % ntl;
  const int nd = d == 0 ? g.nx : g.ny;
  const int nt = d == 0 ? g.ny : g.nx;
  const int t = group * 32 + static_cast<int>(threadIdx.x);
  const int c0 = tile * kCcTile, c1 = min(nd, c0 + kCcTile);
  bool any = false;
  if (t < nt)
    for (int c = c0; c < c1; ++c) {
      const int64_t id = d == 0 ? int64_t(t) * g.nx + c : int64_t(c) * g.nx + t;
      any = any || g.cell_class[d][id] == kCcRegular;
    }
  any = __any_sync(0xffffffffu, any);
  if (threadIdx.x == 0) g.tile_regular[d][blockIdx.x] = any ? 1 : 0;
}

}  // namespace cc

// ---------------------------------------------------------------------------
// Launchers

cudaError_t LaunchCutCellClasses(const CcGeom& g, int d, cudaStream_t s) {
  const int64_t cells = int64_t(g.nx) * g.ny;
  if (cells > 0) cc::CellClassKernel<<<unsigned((cells + 127) / 128), 128, 0, s>>>(g, d);
  const int64_t n = int64_t(g.NGroups(d)) * g.NTiles(d);
  if (n > 0) cc::TileRegularKernel<<<unsigned(n), 32, 0, s>>>(g, d);
  return cudaGetLastError();
}

cudaError_t LaunchCutCellGeometry(const CcGeomArgs& a, const CcGeom& g, cudaStream_t s) {
  const int NX = a.nx + 2 * kCcGhost, NY = a.ny + 2 * kCcGhost;
  const int block = 128;
  const int64_t cells = int64_t(NX) * NY;
  cc::GeometryCellKernel<<<unsigned((cells + block - 1) / block), block, 0, s>>>(a);
  const int64_t faces = int64_t(NX + 1) * NY + int64_t(NX) * (NY + 1);
  cc::GeometryFaceKernel<<<unsigned((faces + block - 1) / block), block, 0, s>>>(a);
  cc::FaceConsistencyKernel<<<unsigned((faces + block - 1) / block), block, 0, s>>>(g);
  for (int d = 0; d < 2; ++d) {
    const int nd = d == 0 ? a.nx : a.ny;
    const int nt = d == 0 ? a.ny : a.nx;
    const int64_t n = int64_t(nd + 2 * kCcGhost - 1) * (nt + 2 * kCcGhost);
    cc::ShieldedKernel<<<unsigned((n + block - 1) / block), block, 0, s>>>(g, d);
  }
  cc::CutFlagKernel<<<unsigned((cells + block - 1) / block), block, 0, s>>>(g);
  return cudaGetLastError();
}

cudaError_t LaunchCutCellReferenceStates(const CcStateArgs& a, cudaStream_t s) {
  return cc::LaunchKbnStates<double, cc::CcIeee>(a, s);
}

cudaError_t LaunchCutCellSweep(const CcSweepArgs& a, bool band, cudaStream_t s) {
  return cc::LaunchKbnSweep<double, cc::CcIeee>(a, band, s);
}

cudaError_t LaunchCutCellStableDt(const CcStateArgs& a, unsigned long long* smax_out,
                                  Control* ctrl, cudaStream_t s) {
  return cc::LaunchKbnStableDt<double, cc::CcIeee>(a, smax_out, ctrl, s);
}

namespace cc {

// Plotfile data of rows [j0, j0 + rows) of the cut-cell grid, component-major
// over the nx x rows box: the Complete state masked by alpha > 0
// (include/fub/AMReX/cutcell/Reconstruction.hpp:76-157), Boundary_X and
// Boundary_Y (AMReX's boundary normal of cut cells, 0 < alpha < 1, the
// negative of fub's GetBoundaryNormal, src/CutCellData.cpp:90-105; 0
// elsewhere), and vfrac, the components the reference's cut-cell
// WritePlotFile (include/fub/AMReX/cutcell/PatchHierarchy.hpp:265-314) and
// AMReX's EB plotfile writer put out.
__global__ void PlotDataKernel(CcGeom g, const double* __restrict__ in, double gamma, int j0,
                               int rows, double* __restrict__ out) {
  const int64_t n = int64_t(g.nx) * rows;
  const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (id >= n) return;
  const int i = static_cast<int>(id % g.nx);
  const int j = j0 + static_cast<int>(id / g.nx);
  const int64_t cs = int64_t(g.nx) * g.ny;
  const int64_t cell = int64_t(j) * g.nx + i;
  double u[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) u[c] = in[c * cs + cell];
  const int64_t gi = g.CellIndex(i, j);
  const double alpha = g.alpha[gi];
  const GasT<double> eq = MakeGasT<double>(gamma);
  C2T<double> q;
  CompleteMasked(eq, q, u, alpha > 0.0);
  const bool cut = alpha > 0.0 && alpha < 1.0;
  const int64_t gc = int64_t(g.NX()) * g.NY();
  const double v[9] = {q.rho, q.m[0], q.m[1], q.E, q.p, q.c,
                       cut ? -g.normal[gi] : 0.0, cut ? -g.normal[gc + gi] : 0.0, alpha};
#pragma unroll
  for (int c = 0; c < 9; ++c) out[c * n + id] = v[c];
}

}  // namespace cc

cudaError_t LaunchCutCellPlotData(const CcGeom& g, const double* cons, double gamma, int j0,
                                  int rows, double* out, cudaStream_t s) {
  const int64_t n = int64_t(g.nx) * rows;
  if (n == 0) return cudaSuccess;
  const int block = 256;
  cc::PlotDataKernel<<<unsigned((n + block - 1) / block), block, 0, s>>>(g, cons, gamma, j0,
                                                                         rows, out);
  return cudaGetLastError();
}

}  // namespace fvs
