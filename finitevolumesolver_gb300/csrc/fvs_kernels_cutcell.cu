// fvs_kernels_cutcell.cu -- KBN h-box cut-cell update on a uniform 2-D grid:
// geometry, shielded face fractions, reference states, the fused cut-cell
// sweep and the masked stable dt.  Compiled with -fmad=false: the results are
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
#include "fvs_internal.h"
#include "fvs_physics_exact.cuh"
#include "fvs_sweep.cuh"

namespace fvs {
namespace cc {

using exact::Complete;
using exact::Gas;
using exact::PMax;
using exact::PMin;
using C2 = Complete<2>;

__device__ __forceinline__ Gas MakeGas(double gamma) {
  Gas g;
  g.gamma = gamma;
  g.gamma_minus_1_inv = 1.0 / (gamma - 1.0);
  return g;
}

// CompleteFromCons masked by `mask && rho > 0` (PerfectGas.cpp:126-144).
__device__ __forceinline__ void CompleteMasked(const Gas& eq, C2& q, const double* u, bool mask) {
  if (!(mask && u[0] > 0.0)) {
    q.rho = 0.0;
    q.m[0] = 0.0;
    q.m[1] = 0.0;
    q.E = 0.0;
    q.p = 0.0;
    q.c = 0.0;
    return;
  }
  exact::CompleteFromCons<2>(eq, q, u);
}

// Flux masked by `rho > 0` (PerfectGas.cpp:79-93, mask true).
__device__ __forceinline__ void FluxMasked(double* f, const C2& q, int dir) {
  const double rho = (q.rho > 0.0) ? q.rho : 1.0;
  const double velocity = q.m[dir] / rho;
  f[0] = q.m[dir];
  f[1] = velocity * q.m[0];
  f[2] = velocity * q.m[1];
  f[1 + dir] += q.p;
  f[3] = velocity * (q.E + q.p);
}

// Masked Einfeldt speeds with mask true (EinfeldtSignalVelocities.hpp:99-142).
__device__ __forceinline__ void EinfeldtMasked(const Gas& eq, const C2& L, const C2& R, int dir,
                                               double& sL, double& sR) {
  const double rhoL = L.rho, rhoR = R.rho;
  const double sqRhoL = sqrt(rhoL);
  const double sqRhoR = sqrt(rhoR);
  const double sqRho = sqRhoL + sqRhoR;
  const double uL = L.m[dir] / rhoL;
  const double uR = R.m[dir] / rhoR;
  const double wL = sqRhoL / sqRho;
  const double wR = sqRhoR / sqRho;
  const double roeU = uL * wL + uR * wR;
  const double hL = (L.E + L.p) / rhoL;
  const double hR = (R.E + R.p) / rhoR;
  const double roeH = hL * wL + hR * wR;
  const double roeA2 = (eq.gamma - 1.0) * (roeH - 0.5 * roeU * roeU);
  const double roeA = sqrt(roeA2);
  sL = PMin(uL - L.c, roeU - roeA);
  sR = PMax(roeU + roeA, uR + R.c);
}

// Masked MUSCL-Hancock predictor of one cell (both face states); the slope
// is zeroed unless the three cells of its window have volume.
__device__ __forceinline__ void PredictMasked(const Gas& eq, C2& recL, C2& recR, const double* q0,
                                              const double* q1, const double* q2, bool smask,
                                              int limiter, double lambda_half, int dir) {
  double uL[4], uR[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const double sL = smask ? q1[k] - q0[k] : 0.0;
    const double sR = smask ? q2[k] - q1[k] : 0.0;
    double slope;
    if (limiter == exact::kVanLeer) {
      const double c = 2.0 * sL * sR;
      slope = (c > 0.0) ? c / (sL + sR) : 0.0;
    } else if (limiter == exact::kMinMod) {
      slope = (sR > 0) ? PMax(0.0, PMin(sL, sR)) : PMin(0.0, PMax(sL, sR));
    } else {
      slope = 0.0;
    }
    uL[k] = q1[k] - 0.5 * slope;
    uR[k] = q1[k] + 0.5 * slope;
  }
  C2 qL, qR;
  CompleteMasked(eq, qL, uL, true);
  CompleteMasked(eq, qR, uR, true);
  double fL[4], fR[4];
  FluxMasked(fL, qL, dir);
  FluxMasked(fR, qR, dir);
  double a[4], b[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const double df = fL[k] - fR[k];
    b[k] = uR[k] + lambda_half * df;
    a[k] = uL[k] + lambda_half * df;
  }
  CompleteMasked(eq, recR, b, true);
  CompleteMasked(eq, recL, a, true);
}

// Masked HLL flux of a face with beta > 0 (HllMethod.hpp:295-335).
__device__ __forceinline__ void HllMasked(const Gas& eq, double* nf, const C2& L, const C2& R,
                                          int dir) {
  double s0, s1;
  EinfeldtMasked(eq, L, R, dir, s0, s1);
  double fL[4], fR[4];
  FluxMasked(fL, L, dir);
  FluxMasked(fR, R, dir);
  const double qL[4] = {L.rho, L.m[0], L.m[1], L.E};
  const double qR[4] = {R.rho, R.m[0], R.m[1], R.E};
  const double sL = PMin(s0, 0.0);
  const double sR = PMax(s1, 0.0);
  const double sLsR = sL * sR;
  const double ds = sR - sL;
#pragma unroll
  for (int k = 0; k < 4; ++k) nf[k] = (sR * fL[k] - sL * fR[k] + sLsR * (qR[k] - qL[k])) / ds;
}

// HllBase::SolveRiemannProblem (scalar, HllMethod.hpp:161-184), direction x.
__device__ __forceinline__ void HllRiemannState(const Gas& eq, C2& sol, const C2& L, const C2& R) {
  double sL, sR;
  exact::Einfeldt<2>(eq, L, R, 0, sL, sR);
  double fL[4], fR[4];
  exact::Flux<2>(fL, L, 0);
  exact::Flux<2>(fR, R, 0);
  const double qL[4] = {L.rho, L.m[0], L.m[1], L.E};
  const double qR[4] = {R.rho, R.m[0], R.m[1], R.E};
  const double ds = sL != sR ? sR - sL : 1.0;
  if (0.0 < sL) {
    sol = L;
  } else if (sR < 0.0) {
    sol = R;
  } else {
    double u[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) u[k] = (sR * qR[k] - sL * qL[k] + fL[k] - fR[k]) / ds;
    exact::CompleteFromCons<2>(eq, sol, u);
  }
}

// Rotation taking unit vector a to b applied to the momentum (MakeRotation).
__device__ __forceinline__ void RotateMomentum(C2& q, double a0, double a1, double b0, double b1) {
  if (a0 == -b0 && a1 == -b1) {
    q.m[0] = -q.m[0];
    q.m[1] = -q.m[1];
    return;
  }
  const double s = a0 * b1 - a1 * b0;
  const double c = a0 * b0 + a1 * b1;
  const double m0 = q.m[0], m1 = q.m[1];
  q.m[0] = c * m0 + (-s) * m1;
  q.m[1] = s * m0 + c * m1;
}

// Wall state: HLL solution of (reflected | state) in the frame of the
// boundary normal, rotated back (KbnStabilisation.hpp:188-210, 229-238).
__device__ __forceinline__ C2 WallSolution(const Gas& eq, const C2& state, double n0, double n1) {
  C2 rot = state;
  RotateMomentum(rot, n0, n1, 1.0, 0.0);
  C2 refl = rot;
  const double dot = rot.m[0] * 1.0 + rot.m[1] * 0.0;
  const double p0 = dot * 1.0, p1 = dot * 0.0;
  refl.m[0] = rot.m[0] - 2 * p0;
  refl.m[1] = rot.m[1] - 2 * p1;
  C2 sol;
  HllRiemannState(eq, sol, refl, rot);
  RotateMomentum(sol, 1.0, 0.0, n0, n1);
  return sol;
}

__device__ __forceinline__ double Clamp01(double x) {
  x = x < 0.0 ? 0.0 : x;
  return 1.0 < x ? 1.0 : x;
}

// ---------------------------------------------------------------------------
// Geometry kernels

__global__ void GeometryCellKernel(CcGeomArgs a) {
  const int NX = a.nx + 2 * kCcGhost, NY = a.ny + 2 * kCcGhost;
  const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (id >= int64_t(NX) * NY) return;
  const int ii = static_cast<int>(id % NX), jj = static_cast<int>(id / NX);
  const double xa = a.x0 + double(ii - kCcGhost) * a.dx;
  const double ya = a.y0 + double(jj - kCcGhost) * a.dy;
  const ccgeom::Cell g = ccgeom::CellGeometry(xa, ya, a.dx, a.dy, a.ncirc, a.circles);
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
  ccgeom::Iv iv[16];
  if (id < nxf) {
    const int ii = static_cast<int>(id % (NX + 1)), jj = static_cast<int>(id / (NX + 1));
    const double xf = a.x0 + double(ii - kCcGhost) * a.dx;
    const double ya = a.y0 + double(jj - kCcGhost) * a.dy;
    const int n = ccgeom::Covered(xf, ya, ya + a.dy, true, a.ncirc, a.circles, iv);
    a.betax[id] = ccgeom::FaceFraction(iv, n, ya, ya + a.dy);
  } else if (id < nxf + nyf) {
    const int64_t k = id - nxf;
    const int ii = static_cast<int>(k % NX), jj = static_cast<int>(k / NX);
    const double yf = a.y0 + double(jj - kCcGhost) * a.dy;
    const double xa = a.x0 + double(ii - kCcGhost) * a.dx;
    const int n = ccgeom::Covered(yf, xa, xa + a.dx, false, a.ncirc, a.circles, iv);
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

// ---------------------------------------------------------------------------
// State helpers

__device__ __forceinline__ void LoadCons(const CcStateArgs& a, int i, int j, double* u) {
  const int si = BcIndex(i, a.g.nx, a.bc[0]);
  const int sj = BcIndex(j, a.g.ny, a.bc[1]);
  const int64_t cs = int64_t(a.g.nx) * a.g.ny;
  const int64_t off = int64_t(sj) * a.g.nx + si;
#pragma unroll
  for (int k = 0; k < 4; ++k) u[k] = __ldg(a.in + k * cs + off);
}

// KbnCutCellMethod::PreAdvanceHierarchy for the cut cells of [-1, n+1)^2.
__global__ void ReferenceStatesKernel(CcStateArgs a) {
  const int w = a.g.nx + 2, h = a.g.ny + 2;
  const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (id >= int64_t(w) * h) return;
  const int i = static_cast<int>(id % w) - 1, j = static_cast<int>(id / w) - 1;
  const int64_t c = a.g.CellIndex(i, j);
  if (!a.g.cut[c]) return;
  const Gas eq = MakeGas(a.gamma);
  double u[4];
  LoadCons(a, i, j, u);
  C2 q;
  CompleteMasked(eq, q, u, a.g.alpha[c] > 0.0);
  const int64_t plane = int64_t(a.g.NX()) * a.g.NY();
  C2 r;
  if (q.rho > 0.0) {
    r = WallSolution(eq, q, a.g.normal[c], a.g.normal[plane + c]);
  } else {
    r = C2{0.0, {0.0, 0.0}, 0.0, 0.0, 0.0};
  }
  a.refs[c] = r.rho;
  a.refs[plane + c] = r.m[0];
  a.refs[2 * plane + c] = r.m[1];
  a.refs[3 * plane + c] = r.E;
  a.refs[4 * plane + c] = r.p;
  a.refs[5 * plane + c] = r.c;
}

// ---------------------------------------------------------------------------
// The fused KBN sweep: one thread marches one grid line (segment) along
// `dir`, evaluating per cell the masked predictor and the boundary flux, per
// face the masked HLLE flux, the h-box stabilised fluxes and the CFL speed,
// and per cell the cut-cell update.

struct FaceData {
  double f[4], fs[4], fsL[4], fsR[4];
  double beta, us, sL, sR;
};

__global__ void __launch_bounds__(128) KbnSweepKernel(CcSweepArgs a) {
  const CcGeom& g = a.s.g;
  const int dir = a.dir;
  const int nd = dir == 0 ? g.nx : g.ny;
  const int nt = dir == 0 ? g.ny : g.nx;
  const int64_t t64 = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int j0 = blockIdx.y * a.seg_len;
  const int j1 = min(nd, j0 + a.seg_len);
  const double split_dt = a.dt_ptr ? a.dt_scale * (*a.dt_ptr) : a.dt_value;
  if (a.ctrl) {
    if (a.ctrl->abort || a.ctrl->done) return;
    if (a.prev_check >= 0) {
      const double smax = BitsToDouble(a.ctrl->smax_check[a.prev_check]);
      if (a.prev_dx / smax < split_dt) return;
    }
  }
  double smax = 0.0;
  int status = 0;
  if (t64 < nt) {
    const int t = static_cast<int>(t64);
    const Gas eq = MakeGas(a.s.gamma);
    const double dx = a.dx;
    const double lambda_half = 0.5 * split_dt / dx;
    const double dt_dx = split_dt / dx;
    const int64_t plane = int64_t(g.NX()) * g.NY();
    const int64_t cs = int64_t(g.nx) * g.ny;
    auto cell_ij = [&](int c, int& i, int& j) {
      if (dir == 0) {
        i = c;
        j = t;
      } else {
        i = t;
        j = c;
      }
    };
    // masked complete state (alpha > 0 and rho > 0) of cell c
    auto load_cell = [&](int c, double* u, double& alpha) {
      int i, j;
      cell_ij(c, i, j);
      double v[4];
      LoadCons(a.s, i, j, v);
      alpha = g.alpha[g.CellIndex(i, j)];
      C2 q;
      CompleteMasked(eq, q, v, alpha > 0.0);
      u[0] = q.rho;
      u[1] = q.m[0];
      u[2] = q.m[1];
      u[3] = q.E;
    };
    // boundary flux of cell c (0 unless it is a cut cell)
    auto boundary_flux = [&](int c, const double* u, double* fb) {
      int i, j;
      cell_ij(c, i, j);
      const int64_t ci = g.CellIndex(i, j);
#pragma unroll
      for (int k = 0; k < 4; ++k) fb[k] = 0.0;
      if (!g.cut[ci]) return;
      C2 ref;
      ref.rho = a.s.refs[ci];
      ref.m[0] = a.s.refs[plane + ci];
      ref.m[1] = a.s.refs[2 * plane + ci];
      ref.E = a.s.refs[3 * plane + ci];
      ref.p = a.s.refs[4 * plane + ci];
      ref.c = a.s.refs[5 * plane + ci];
      C2 q;
      CompleteMasked(eq, q, u, g.alpha[ci] > 0.0);
      exact::Flux<2>(fb, ref, dir);
      const C2 sol = WallSolution(eq, q, g.normal[ci], g.normal[plane + ci]);
      fb[1 + dir] += sol.p - ref.p;
    };
    auto center_of = [&](int c) {
      int i, j;
      cell_ij(c, i, j);
      return g.center[int64_t(dir) * plane + g.CellIndex(i, j)];
    };
    double um[4], uc[4], up[4];
    double am, ac, ap;
    load_cell(j0 - 2, um, am);
    load_cell(j0 - 1, uc, ac);
    C2 recR_prev;
    double fb_prev[4];
    double xb_prev = 0.0;
    C2 q_prev;
    FaceData F_prev;
    for (int j = j0 - 1; j <= j1; ++j) {
      load_cell(j + 1, up, ap);
      const bool smask = am > 0.0 && ac > 0.0 && ap > 0.0;
      C2 recL, recR;
      PredictMasked(eq, recL, recR, um, uc, up, smask, a.limiter, lambda_half, dir);
      double fb[4];
      boundary_flux(j, uc, fb);
      const double xb = center_of(j);
      C2 q;
      CompleteMasked(eq, q, uc, true);  // uc is already masked by alpha
      if (j >= j0) {
        FaceData F;
        const int64_t fi = g.FaceIndex(dir, j, t);
        F.beta = g.beta[dir][fi];
        F.us = g.us[dir][fi];
        F.sL = g.sL[dir][fi];
        F.sR = g.sR[dir][fi];
        const double us_rel = g.us_rel[dir][fi];
        const double sL_rel = g.sL_rel[dir][fi];
        const double sR_rel = g.sR_rel[dir][fi];
        if (F.beta > 0.0) {
          HllMasked(eq, F.f, recR_prev, recL, dir);
          double s0, s1;
          EinfeldtMasked(eq, q_prev, q, dir, s0, s1);
          const double mx = PMax(PMax(0.0, fabs(s0)), fabs(s1));
          smax = mx > smax ? mx : smax;
        } else {
#pragma unroll
          for (int k = 0; k < 4; ++k) F.f[k] = 0.0;
        }
        const double dL = Clamp01(0.5 - xb_prev);
        const double dR = Clamp01(0.5 + xb);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const double fk = F.f[k];
          const double sLk = dL * fk + (1.0 - dL) * fb_prev[k];
          const double sRk = dR * fk + (1.0 - dR) * fb[k];
          F.fsL[k] = sLk;
          F.fsR[k] = sRk;
          F.fs[k] = us_rel * fk + sL_rel * sLk + sR_rel * sRk;
        }
        if (j > j0) {
          // cut-cell update of cell j-1 (faces j-1 and j)
          const int c = j - 1;
          int i, jj;
          cell_ij(c, i, jj);
          const int64_t out = int64_t(jj) * g.nx + i;
          const double alpha = am;  // alpha of cell j-1
          const double betaL = F_prev.beta, betaR = F.beta;
          const double center = xb_prev;
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            double next;
            if (alpha == 0.0) {
              next = 0.0;
            } else {
              const double prev = __ldg(a.s.in + k * cs + out);
              const double fLs = F_prev.fs[k], fRs = F.fs[k];
              const double fLu = F_prev.f[k], fRu = F.f[k];
              if (betaL == betaR) {
                next = prev + dt_dx * (fLs - fRs);
              } else if (betaL > betaR) {
                const double bus = F_prev.us / alpha;
                const double bsL = F_prev.sL / alpha;
                const double dist = 0.5 + center;
                const double dBeta = Clamp01((F_prev.sR * dist) / alpha);
                const double dF_us = fLu - fRs;
                const double dF_sL = F_prev.fsL[k] - fRs;
                const double dB = fLu - fb_prev[k];
                next = prev + dt_dx * bus * dF_us + dt_dx * bsL * dF_sL + dt_dx * dBeta * dB;
              } else {
                const double bus = F.us / alpha;
                const double bsR = F.sR / alpha;
                const double dist = 0.5 - center;
                const double dBeta = Clamp01((F.sL * dist) / alpha);
                const double dF_us = fLs - fRu;
                const double dF_sR = fLs - F.fsR[k];
                const double dB = fb_prev[k] - fRu;
                next = prev + dt_dx * bus * dF_us + dt_dx * bsR * dF_sR + dt_dx * dBeta * dB;
              }
            }
            a.out[k * cs + out] = next;
          }
          if (alpha > 0.0 && __double_as_longlong(a.out[out]) <= 0)
            status |= kStatusNonPositiveDensity;
        }
        F_prev = F;
      }
      recR_prev = recR;
#pragma unroll
      for (int k = 0; k < 4; ++k) fb_prev[k] = fb[k];
      xb_prev = xb;
      q_prev = q;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        um[k] = uc[k];
        uc[k] = up[k];
      }
      am = ac;
      ac = ap;
    }
  }
  const double m = WarpMax(smax);
  if ((threadIdx.x & 31) == 0 && a.smax_out && m > 0.0) AtomicMaxPositive(a.smax_out, m);
  if (status && a.ctrl) atomicOr(&a.ctrl->step_status, status);
}

// Masked stable dt over both directions: faces 0..n with beta > 0
// (KbnStabilisation.hpp:275-345).
__global__ void KbnStableDtKernel(CcStateArgs a, unsigned long long* smax_out, Control* ctrl) {
  if (ctrl && (ctrl->abort || ctrl->done)) return;
  const CcGeom& g = a.g;
  const int w = g.nx + 1, h = g.ny + 1;
  const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  double sm[2] = {0.0, 0.0};
  if (id < int64_t(w) * h) {
    const int i = static_cast<int>(id % w), j = static_cast<int>(id / w);
    const Gas eq = MakeGas(a.gamma);
    for (int d = 0; d < 2; ++d) {
      const int f = d == 0 ? i : j;
      const int t = d == 0 ? j : i;
      const int nt = d == 0 ? g.ny : g.nx;
      if (t >= nt) continue;
      if (!(g.beta[d][g.FaceIndex(d, f, t)] > 0.0)) continue;
      const int il = d == 0 ? f - 1 : t, jl = d == 0 ? t : f - 1;
      const int ir = d == 0 ? f : t, jr = d == 0 ? t : f;
      double ul[4], ur[4];
      LoadCons(a, il, jl, ul);
      LoadCons(a, ir, jr, ur);
      C2 L, R;
      CompleteMasked(eq, L, ul, g.alpha[g.CellIndex(il, jl)] > 0.0);
      CompleteMasked(eq, R, ur, g.alpha[g.CellIndex(ir, jr)] > 0.0);
      double s0, s1;
      EinfeldtMasked(eq, L, R, d, s0, s1);
      const double mx = PMax(PMax(0.0, fabs(s0)), fabs(s1));
      sm[d] = mx > sm[d] ? mx : sm[d];
    }
  }
  for (int d = 0; d < 2; ++d) {
    const double m = WarpMax(sm[d]);
    if ((threadIdx.x & 31) == 0 && m > 0.0) AtomicMaxPositive(smax_out + d, m);
  }
}

}  // namespace cc

// ---------------------------------------------------------------------------
// Launchers

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
  const int64_t n = int64_t(a.g.nx + 2) * (a.g.ny + 2);
  const int block = 128;
  cc::ReferenceStatesKernel<<<unsigned((n + block - 1) / block), block, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t LaunchCutCellSweep(const CcSweepArgs& a, cudaStream_t s) {
  const int nd = a.dir == 0 ? a.s.g.nx : a.s.g.ny;
  const int nt = a.dir == 0 ? a.s.g.ny : a.s.g.nx;
  const int block = 128;
  const int seg = a.seg_len > 0 ? a.seg_len : nd;
  CcSweepArgs b = a;
  b.seg_len = seg;
  dim3 grid(unsigned((nt + block - 1) / block), unsigned((nd + seg - 1) / seg));
  cc::KbnSweepKernel<<<grid, block, 0, s>>>(b);
  return cudaGetLastError();
}

cudaError_t LaunchCutCellStableDt(const CcStateArgs& a, unsigned long long* smax_out,
                                  Control* ctrl, cudaStream_t s) {
  const int64_t n = int64_t(a.g.nx + 1) * (a.g.ny + 1);
  const int block = 128;
  cc::KbnStableDtKernel<<<unsigned((n + block - 1) / block), block, 0, s>>>(a, smax_out, ctrl);
  return cudaGetLastError();
}

}  // namespace fvs
