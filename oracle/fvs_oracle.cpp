// fvs_oracle.cpp -- CPU oracle: patch-level flux / dt / update functions and
// a uniform-grid split time stepper, exported with a C ABI for the tests.
//
// TEST INFRASTRUCTURE ONLY (see fvs_oracle.hpp).  Restates:
//   include/fub/flux_method/FluxMethod.hpp:200-215, 295-382 (face loop, dt)
//   src/HyperbolicPatchIntegrator.cpp:88-105 (conservative update)
//   include/fub/solver/DimensionalSplitLevelIntegrator.hpp:204-276 (sweeps)
//   src/split_method/StrangSplitting.cpp:25-69 (Strang order)
//   include/fub/split_method/SplittingMethod.hpp:115-126 (direction order)
//   include/fub/RunSimulation.hpp:97-160 (dt selection, restart on failure)
//   src/AMReX/boundary_condition/TransmissiveBoundary.cpp:31-93 (ghost fill)
//   include/fub/AMReX/FluxMethodAdapter.hpp:69-114 (dt over MFIter tiles)
#include "fvs_oracle.hpp"
#include "fvs_oracle_riemann.hpp"

#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

using namespace fvs_oracle;

extern "C" {
// Method description shared with the Python test helpers.
struct orc_method {
  int32_t method;   // kMusclHlle, kHlle, kGodunov, kMusclGodunov, kHllem, kMusclHllem,
                    // kMusclChar, kMusclPrim
  int32_t limiter;  // kVanLeer, kMinMod, kNoLimiter
  int32_t guess;    // kGuessMean, kGuessPvrsTr
  int32_t max_iterations;
  double tol;
};
}

namespace {

// A box view in the FArrayBox layout: component-major, x fastest,
// element (c, i, j, k) at ((c*n2 + k-lo2)*n1 + j-lo1)*n0 + i-lo0
// (include/fub/AMReX/ViewFArrayBox.hpp:73-82).
struct BoxView {
  double* data;
  int lo[3];
  int n[3];
  int64_t Index(int c, int i, int j, int k) const {
    return ((int64_t(c) * n[2] + (k - lo[2])) * n[1] + (j - lo[1])) * int64_t(n[0]) +
           (i - lo[0]);
  }
  double& operator()(int c, int i, int j, int k) const { return data[Index(c, i, j, k)]; }
};

BoxView MakeView(const double* data, const int32_t* lo, const int32_t* hi) {
  BoxView v;
  v.data = const_cast<double*>(data);
  for (int d = 0; d < 3; ++d) {
    v.lo[d] = lo[d];
    v.n[d] = hi[d] - lo[d];
  }
  return v;
}

template <int D>
Complete<D> LoadComplete(const BoxView& v, int i, int j, int k) {
  Complete<D> q;
  q.rho = v(0, i, j, k);
  for (int d = 0; d < D; ++d) q.m[d] = v(1 + d, i, j, k);
  q.E = v(1 + D, i, j, k);
  q.p = v(2 + D, i, j, k);
  q.c = v(3 + D, i, j, k);
  return q;
}

template <int D>
void LoadCons(double* u, const BoxView& v, int i, int j, int k) {
  for (int c = 0; c < D + 2; ++c) u[c] = v(c, i, j, k);
}

inline void Shift(int* idx, int dir, int s) { idx[dir] += s; }

int StencilWidth(int method) {
  return (method == kHlle || method == kGodunov || method == kHllem) ? 1 : 2;
}

// The numeric flux of one face from the 2w cells of its stencil.
// MusclHancock: include/fub/flux_method/MusclHancockMethod.hpp:419-485,
// Hll: include/fub/flux_method/HllMethod.hpp:260-293,
// Godunov: include/fub/flux_method/GodunovMethod.hpp:129-135.
template <int D>
void FaceFlux(const Gas& eq, const orc_method& m, double* nf,
              const Complete<D>* st, double dt, double dx, int dir,
              int* iters, int* converged) {
  ExactOptions opt;
  opt.guess = m.guess;
  opt.tol = m.tol;
  opt.max_iterations = m.max_iterations;
  if (iters) *iters = 0;
  if (converged) *converged = 1;
  if (m.method == kHlle) {
    HllFlux<D>(eq, nf, st[0], st[1], dir);
    return;
  }
  if (m.method == kHllem) {
    HllemFlux<D>(eq, nf, st[0], st[1], dir);
    return;
  }
  if (m.method == kGodunov) {
    int it = GodunovFlux<D>(eq, nf, st[0], st[1], dir, opt, 0.0, converged);
    if (iters) *iters = it;
    return;
  }
  if (m.method == kMusclChar || m.method == kMusclPrim) {
    // MusclHancockCharacteristic / MusclHancockPrim: reconstruct the two
    // inner cells, then Hllem (MusclHancockCharacteristicMethod.hpp:303-317,
    // MusclHancockPrimMethod.hpp:59-182); the stable dt is Hllem's on the
    // inner pair (:354-358, :35-40).
    const double lambda = dt / dx;
    Complete<D> rec0, rec1;
    if (m.method == kMusclChar) {
      CharPredict<D>(eq, rec0, st, lambda, dir, 1.0);
      CharPredict<D>(eq, rec1, st + 1, lambda, dir, -1.0);
    } else {
      PrimPredict<D>(eq, rec0, st, lambda, dir, +1);
      PrimPredict<D>(eq, rec1, st + 1, lambda, dir, -1);
    }
    HllemFlux<D>(eq, nf, rec0, rec1, dir);
    return;
  }
  const double lambda_half = 0.5 * dt / dx;
  double u[4][D + 2];
  for (int s = 0; s < 4; ++s) AsCons<D>(u[s], st[s]);
  Complete<D> rec0, rec1;
  MusclPredict<D>(eq, rec0, u[0], u[1], u[2], m.limiter, lambda_half, dir, +1);
  MusclPredict<D>(eq, rec1, u[1], u[2], u[3], m.limiter, lambda_half, dir, -1);
  if (m.method == kMusclHlle) {
    HllFlux<D>(eq, nf, rec0, rec1, dir);
  } else if (m.method == kMusclHllem) {
    HllemFlux<D>(eq, nf, rec0, rec1, dir);
  } else {
    int it = GodunovFlux<D>(eq, nf, rec0, rec1, dir, opt, 0.0, converged);
    if (iters) *iters = it;
  }
}

// Stable dt of one window of 2w cells: MusclHancock uses the middle pair
// (include/fub/flux_method/MusclHancockMethod.hpp:214-218).
template <int D>
double WindowDt(const Gas& eq, const orc_method& m, const Complete<D>* st,
                double dx, int dir) {
  const int w = StencilWidth(m.method);
  const Complete<D>& L = st[w - 1];
  const Complete<D>& R = st[w];
  if (m.method == kGodunov || m.method == kMusclGodunov) {
    ExactOptions opt;
    opt.guess = m.guess;
    opt.tol = m.tol;
    opt.max_iterations = m.max_iterations;
    return GodunovStableDt<D>(eq, L, R, dx, dir, opt);
  }
  if (m.method == kHllem || m.method == kMusclHllem || m.method == kMusclChar ||
      m.method == kMusclPrim)
    return HllemStableDt<D>(eq, L, R, dx, dir);
  return HllStableDt<D>(eq, L, R, dx, dir);
}

// FluxMethod<Base>::ComputeNumericFluxes, sequential face loop
// include/fub/flux_method/FluxMethod.hpp:200-215.
template <int D>
void ComputeNumericFluxes(const orc_method& m, const BoxView& fluxes,
                          const BoxView& states, double dt, double dx, int dir,
                          int64_t* total_iters, int64_t* failures) {
  const Gas eq;
  const int w = StencilWidth(m.method);
  const int n_outer = fluxes.n[2] * fluxes.n[1];
  int64_t it_sum = 0, fail_sum = 0;
#pragma omp parallel for schedule(static) reduction(+ : it_sum, fail_sum)
  for (int o = 0; o < n_outer; ++o) {
    const int k = fluxes.lo[2] + o / fluxes.n[1];
    const int j = fluxes.lo[1] + o % fluxes.n[1];
    Complete<D> st[4];
    double nf[D + 2];
    for (int i = fluxes.lo[0]; i < fluxes.lo[0] + fluxes.n[0]; ++i) {
      int face[3] = {i, j, k};
      for (int s = 0; s < 2 * w; ++s) {
        int cell[3] = {face[0], face[1], face[2]};
        Shift(cell, dir, s - w);
        st[s] = LoadComplete<D>(states, cell[0], cell[1], cell[2]);
      }
      int iters = 0, conv = 1;
      FaceFlux<D>(eq, m, nf, st, dt, dx, dir, &iters, &conv);
      it_sum += iters;
      fail_sum += conv ? 0 : 1;
      for (int c = 0; c < D + 2; ++c) fluxes(c, i, j, k) = nf[c];
    }
  }
  if (total_iters) *total_iters = it_sum;
  if (failures) *failures = fail_sum;
}

// FluxMethod<Base>::ComputeStableDt.  window_rule 0: sequential tag, windows
// starting in Shrink(box, dir, {0, 2w}) (FluxMethod.hpp:295-314); 1: simd tag,
// windows starting in Shrink(box, dir, {0, 2w-1}) (FluxMethod.hpp:341-382).
template <int D>
double ComputeStableDt(const orc_method& m, const BoxView& states, double dx,
                       int dir, int window_rule) {
  const Gas eq;
  const int w = StencilWidth(m.method);
  const int S = 2 * w;
  int lo[3] = {states.lo[0], states.lo[1], states.lo[2]};
  int hi[3] = {states.lo[0] + states.n[0], states.lo[1] + states.n[1],
               states.lo[2] + states.n[2]};
  hi[dir] -= (window_rule == 0) ? S : (S - 1);
  double min_dt = std::numeric_limits<double>::infinity();
  for (int k = lo[2]; k < hi[2]; ++k) {
    for (int j = lo[1]; j < hi[1]; ++j) {
      for (int i = lo[0]; i < hi[0]; ++i) {
        Complete<D> st[4];
        for (int s = 0; s < S; ++s) {
          int cell[3] = {i, j, k};
          Shift(cell, dir, s);
          st[s] = LoadComplete<D>(states, cell[0], cell[1], cell[2]);
        }
        const double dt = WindowDt<D>(eq, m, st, dx, dir);
        // std::min(dt, min_dt) of the reference for every non-NaN dt.  A NaN
        // window dt (a NaN face speed: negative pressure, outside the pinned
        // domain) is skipped, the one NaN rule of the library's CFL maxima;
        // the reference's std::min would instead forget every window before
        // the NaN one.
        if (dt < min_dt) min_dt = dt;
      }
    }
  }
  return min_dt;
}

// HyperbolicPatchIntegrator<seq>::UpdateConservatively
// src/HyperbolicPatchIntegrator.cpp:88-105.
void UpdateConservatively(const BoxView& next, const BoxView& prev,
                          const BoxView& fluxes, int ncomp, double dt,
                          double dx, int dir) {
  const double dt_dx = dt / dx;
#pragma omp parallel for collapse(3) schedule(static)
  for (int c = 0; c < ncomp; ++c) {
    for (int k = next.lo[2]; k < next.lo[2] + next.n[2]; ++k) {
      for (int j = next.lo[1]; j < next.lo[1] + next.n[1]; ++j) {
        for (int i = next.lo[0]; i < next.lo[0] + next.n[0]; ++i) {
          int fR[3] = {i, j, k};
          Shift(fR, dir, 1);
          const double U_prev = prev(c, i, j, k);
          const double f_left = fluxes(c, i, j, k);
          const double f_right = fluxes(c, fR[0], fR[1], fR[2]);
          next(c, i, j, k) = U_prev + dt_dx * (f_left - f_right);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Uniform single-patch grid: interior cons arrays without ghosts, ghost cells
// materialised per sweep (2 layers), exactly as the reference's scratch.

struct Grid {
  int D;
  int n[3];
  int bc[3];  // 0 periodic, 1 transmissive, 2 reflective
  double dx[3];
  int64_t cells() const { return int64_t(n[0]) * n[1] * n[2]; }
};

Grid MakeGrid(int rank, const int32_t* n, const int32_t* bc, const double* dx) {
  Grid g;
  g.D = rank;
  for (int d = 0; d < 3; ++d) {
    g.n[d] = d < rank ? n[d] : 1;
    g.bc[d] = d < rank ? bc[d] : 0;
    g.dx[d] = d < rank ? dx[d] : 1.0;
  }
  return g;
}

// Index of the cell supplying the value of (possibly ghost) index i in a
// direction of extent n: periodic image, the boundary cell (transmissive,
// TransmissiveBoundary.cpp:31-42 copies the boundary cell, no mirroring) or
// the mirror cell (reflective, ReflectIndex of
// src/boundary_condition/ReflectiveBoundary.cpp:24-36 with the ghost strip as
// the fill box: lower side i -> -1 - i, upper side i -> 2n - 1 - i).
inline int SourceIndex(int i, int n, int bc) {
  if (i >= 0 && i < n) return i;
  if (bc == 0) return ((i % n) + n) % n;
  if (bc == 2) return i < 0 ? -1 - i : 2 * n - 1 - i;
  return i < 0 ? 0 : n - 1;
}

// Build the ghosted Complete-state scratch for a sweep in `dir` with `G`
// ghost layers in that direction, then CompleteFromCons on every cell.
template <int D>
std::vector<double> BuildScratch(const Grid& g, const double* cons, int dir,
                                 int G, int lo[3], int hi[3]) {
  for (int d = 0; d < 3; ++d) {
    lo[d] = 0;
    hi[d] = g.n[d];
  }
  lo[dir] -= G;
  hi[dir] += G;
  const int sn[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
  const int64_t ncell = int64_t(sn[0]) * sn[1] * sn[2];
  std::vector<double> scratch(size_t(ncell) * (D + 4));
  BoxView sv{scratch.data(), {lo[0], lo[1], lo[2]}, {sn[0], sn[1], sn[2]}};
  BoxView cv{const_cast<double*>(cons), {0, 0, 0}, {g.n[0], g.n[1], g.n[2]}};
  const Gas eq;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = lo[2]; k < hi[2]; ++k) {
    for (int j = lo[1]; j < hi[1]; ++j) {
      for (int i = lo[0]; i < hi[0]; ++i) {
        int src[3] = {i, j, k};
        src[dir] = SourceIndex(src[dir], g.n[dir], g.bc[dir]);
        double u[D + 2];
        LoadCons<D>(u, cv, src[0], src[1], src[2]);
        Complete<D> q;
        CompleteFromCons<D>(eq, q, u);
        // ReflectiveBoundary::FillBoundary: the ghost is Reflect of the mirror
        // cell's complete state (ReflectiveBoundary.hpp:61-75)
        const int at[3] = {i, j, k};
        if (g.bc[dir] == 2 && (at[dir] < 0 || at[dir] >= g.n[dir])) ReflectMomentum<D>(q.m, dir);
        sv(0, i, j, k) = q.rho;
        for (int d = 0; d < D; ++d) sv(1 + d, i, j, k) = q.m[d];
        sv(1 + D, i, j, k) = q.E;
        sv(2 + D, i, j, k) = q.p;
        sv(3 + D, i, j, k) = q.c;
      }
    }
  }
  return scratch;
}

// One directional sweep: ghost fill -> fluxes -> conservative update
// (DimensionalSplitLevelIntegrator.hpp:227-263).  cons_out may equal cons_in.
template <int D>
void GridSweep(const Grid& g, const orc_method& m, const double* cons_in,
               double* cons_out, double dt, int dir, int64_t* iters,
               int64_t* failures) {
  const int G = 2;
  int lo[3], hi[3];
  std::vector<double> scratch = BuildScratch<D>(g, cons_in, dir, G, lo, hi);
  BoxView sv{scratch.data(), {lo[0], lo[1], lo[2]},
             {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]}};
  int fn[3] = {g.n[0], g.n[1], g.n[2]};
  fn[dir] += 1;
  std::vector<double> flux(size_t(fn[0]) * fn[1] * fn[2] * (D + 2));
  BoxView fv{flux.data(), {0, 0, 0}, {fn[0], fn[1], fn[2]}};
  ComputeNumericFluxes<D>(m, fv, sv, dt, g.dx[dir], dir, iters, failures);
  BoxView prev{const_cast<double*>(cons_in), {0, 0, 0}, {g.n[0], g.n[1], g.n[2]}};
  BoxView next{cons_out, {0, 0, 0}, {g.n[0], g.n[1], g.n[2]}};
  UpdateConservatively(next, prev, fv, D + 2, dt, g.dx[dir], dir);
}

// Stable dt in `dir`.  rule 0: every face of the level, including the two
// boundary faces (the GPU fused reduction).  rule 1: the reference's
// FluxMethodAdapter tiling of a single-box level, MFIter tiles of
// (1024000, 8, 8) cells grown by the 2 scratch ghost layers where they touch
// the box boundary, simd windows inside each tile (FluxMethodAdapter.hpp:85-96,
// FluxMethod.hpp:341-382).
template <int D>
double GridStableDt(const Grid& g, const orc_method& m, const double* cons,
                    int dir, int rule) {
  const int G = 2;
  int lo[3], hi[3];
  std::vector<double> scratch = BuildScratch<D>(g, cons, dir, G, lo, hi);
  BoxView sv{scratch.data(), {lo[0], lo[1], lo[2]},
             {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]}};
  const Gas eq;
  const int w = StencilWidth(m.method);
  const double dx = g.dx[dir];
  double min_dt = std::numeric_limits<double>::infinity();
  if (rule == 0 || dir == 0) {
    // faces f in [0, n]: cells (f-1, f).  For dir 0 with 2 ghosts the simd
    // window rule covers exactly these faces as well.
    int fhi[3] = {g.n[0], g.n[1], g.n[2]};
    fhi[dir] += 1;
#pragma omp parallel for collapse(2) schedule(static) reduction(min : min_dt)
    for (int k = 0; k < fhi[2]; ++k) {
      for (int j = 0; j < fhi[1]; ++j) {
        for (int i = 0; i < fhi[0]; ++i) {
          Complete<D> st[4];
          for (int s = 0; s < 2 * w; ++s) {
            int cell[3] = {i, j, k};
            Shift(cell, dir, s - w);
            int c2[3] = {cell[0], cell[1], cell[2]};
            c2[dir] = std::max(lo[dir], std::min(hi[dir] - 1, c2[dir]));
            st[s] = LoadComplete<D>(sv, c2[0], c2[1], c2[2]);
          }
          min_dt = std::min(min_dt, WindowDt<D>(eq, m, st, dx, dir));
        }
      }
    }
    return min_dt;
  }
  // rule 1, dir = y or z: tiles of 8 cells along dir over the interior,
  // grown by G at the box boundary; windows of 2w cells inside each tile.
  const int n = g.n[dir];
  for (int t0 = 0; t0 < n; t0 += 8) {
    const int t1 = std::min(n, t0 + 8);
    const int a = (t0 == 0) ? -G : t0;
    const int b = (t1 == n) ? n + G : t1;
    // windows start s in [a, b - (2w - 1)); the window uses cells s+w-1, s+w
    for (int s = a; s < b - (2 * w - 1); ++s) {
      const int f = s + w;  // face between cells f-1 and f
      int cnt[3] = {g.n[0], g.n[1], g.n[2]};
      cnt[dir] = 1;
      for (int k = 0; k < cnt[2]; ++k) {
        for (int j = 0; j < cnt[1]; ++j) {
          for (int i = 0; i < cnt[0]; ++i) {
            Complete<D> st[4];
            for (int q = 0; q < 2 * w; ++q) {
              int cell[3] = {i, j, k};
              cell[dir] = f - w + q;
              st[q] = LoadComplete<D>(sv, cell[0], cell[1], cell[2]);
            }
            min_dt = std::min(min_dt, WindowDt<D>(eq, m, st, dx, dir));
          }
        }
      }
    }
  }
  return min_dt;
}

// MakeSplitDirections  include/fub/split_method/SplittingMethod.hpp:115-126.
void SplitDirections(int rank, int cycle, int* dirs) {
  const int is_odd = (cycle % 2) % 2;
  for (int i = 0; i < rank; ++i) dirs[i] = is_odd ? rank - 1 - i : i;
}

// One split step of size dt.  Returns 0 on success or 1 with *fail_dt set
// when the per-sweep dt check fails (DimensionalSplitLevelIntegrator.hpp:240-245).
template <int D>
int AdvanceStep(const Grid& g, const orc_method& m, double* cons, double dt,
                int cycle, int dt_rule, int check, double* fail_dt,
                int64_t* iters, int64_t* failures) {
  int dirs[3];
  SplitDirections(D, cycle, dirs);
  // Strang sequence of (direction, fraction of dt): StrangSplitting.cpp:25-69.
  int seq[6];
  int nseq = 0;
  double frac = 0.5;
  if (D == 1) {
    seq[nseq++] = dirs[0];
    frac = 1.0;
  } else if (D == 2) {
    const int s[4] = {dirs[0], dirs[1], dirs[1], dirs[0]};
    for (int i = 0; i < 4; ++i) seq[nseq++] = s[i];
  } else {
    const int s[6] = {dirs[0], dirs[1], dirs[2], dirs[2], dirs[1], dirs[0]};
    for (int i = 0; i < 6; ++i) seq[nseq++] = s[i];
  }
  const double split_dt = frac * dt;
  for (int s = 0; s < nseq; ++s) {
    const int dir = seq[s];
    if (check) {
      const double level_dt = GridStableDt<D>(g, m, cons, dir, dt_rule);
      if (level_dt < split_dt) {
        *fail_dt = level_dt;
        return 1;
      }
    }
    int64_t it = 0, fl = 0;
    GridSweep<D>(g, m, cons, cons, split_dt, dir, &it, &fl);
    if (iters) *iters += it;
    if (failures) *failures += fl;
  }
  return 0;
}

template <int D>
double GridStableDtAllDirs(const Grid& g, const orc_method& m,
                           const double* cons, int rule) {
  double dt = std::numeric_limits<double>::max();
  for (int d = 0; d < D; ++d) dt = std::min(dt, GridStableDt<D>(g, m, cons, d, rule));
  return dt;
}

// RunSimulation loop without outputs: dt = min(t_end - t, cfl * stable_dt),
// the step restarts from a backup with the failure dt when a sweep's check
// fails (RunSimulation.hpp:97-160).  When dt_override is given, step s uses
// dt_override[s] instead and the checks are skipped.
template <int D>
int Run(const Grid& g, const orc_method& m, double* cons, double cfl,
        double t_end, int max_steps, int dt_rule, const double* dt_override,
        int n_override, double* dt_log, int* restarts, int64_t* iters,
        int64_t* failures) {
  const double eps = 1e-12;
  double t = 0.0;
  int step = 0;
  int n_restarts = 0;
  std::vector<double> backup(size_t(g.cells()) * (D + 2));
  bool have_failure = false;
  double failure_dt = 0.0;
  while (t + eps < t_end && (max_steps < 0 || step < max_steps)) {
    double dt;
    const bool fixed = dt_override && step < n_override;
    if (fixed) {
      dt = dt_override[step];
    } else {
      const double stable_dt =
          have_failure ? failure_dt : GridStableDtAllDirs<D>(g, m, cons, dt_rule);
      dt = std::min(t_end - t, cfl * stable_dt);
    }
    std::memcpy(backup.data(), cons, backup.size() * sizeof(double));
    double fail_dt = 0.0;
    const int err = AdvanceStep<D>(g, m, cons, dt, step, dt_rule, !fixed,
                                   &fail_dt, iters, failures);
    if (err) {
      std::memcpy(cons, backup.data(), backup.size() * sizeof(double));
      have_failure = true;
      failure_dt = fail_dt;
      ++n_restarts;
      continue;
    }
    have_failure = false;
    if (dt_log) dt_log[step] = dt;
    t = t + dt;
    ++step;
  }
  if (restarts) *restarts = n_restarts;
  return step;
}

template <typename F> auto DispatchRank(int rank, F&& f) {
  switch (rank) {
  case 1:
    return f(std::integral_constant<int, 1>{});
  case 2:
    return f(std::integral_constant<int, 2>{});
  default:
    return f(std::integral_constant<int, 3>{});
  }
}

void SetThreads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

}  // namespace

extern "C" {

int orc_abi_version(void) { return 1; }

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// PerfectGas<D>::CompleteFromCons over n states (SoA, component-major).
void orc_complete_from_cons(int rank, int64_t n, const double* cons,
                            double* complete) {
  DispatchRank(rank, [&](auto R) {
    constexpr int D = decltype(R)::value;
    const Gas eq;
    for (int64_t i = 0; i < n; ++i) {
      double u[D + 2];
      for (int c = 0; c < D + 2; ++c) u[c] = cons[c * n + i];
      Complete<D> q;
      CompleteFromCons<D>(eq, q, u);
      complete[0 * n + i] = q.rho;
      for (int d = 0; d < D; ++d) complete[(1 + d) * n + i] = q.m[d];
      complete[(1 + D) * n + i] = q.E;
      complete[(2 + D) * n + i] = q.p;
      complete[(3 + D) * n + i] = q.c;
    }
    return 0;
  });
}

// Patch-level FluxMethod::ComputeNumericFluxes over box views.
int orc_compute_numeric_fluxes(const orc_method* m, int rank, double* fluxes,
                               const int32_t* face_lo, const int32_t* face_hi,
                               const double* states, const int32_t* cell_lo,
                               const int32_t* cell_hi, double dt, double dx,
                               int dir, int64_t* iters, int64_t* failures) {
  BoxView fv = MakeView(fluxes, face_lo, face_hi);
  BoxView sv = MakeView(states, cell_lo, cell_hi);
  return DispatchRank(rank, [&](auto R) {
    constexpr int D = decltype(R)::value;
    ComputeNumericFluxes<D>(*m, fv, sv, dt, dx, dir, iters, failures);
    return 0;
  });
}

double orc_compute_stable_dt(const orc_method* m, int rank,
                             const double* states, const int32_t* cell_lo,
                             const int32_t* cell_hi, double dx, int dir,
                             int window_rule) {
  BoxView sv = MakeView(states, cell_lo, cell_hi);
  return DispatchRank(rank, [&](auto R) {
    constexpr int D = decltype(R)::value;
    return ComputeStableDt<D>(*m, sv, dx, dir, window_rule);
  });
}

void orc_update_conservatively(double* next, const int32_t* next_lo,
                               const int32_t* next_hi, const double* prev,
                               const int32_t* prev_lo, const int32_t* prev_hi,
                               const double* fluxes, const int32_t* face_lo,
                               const int32_t* face_hi, int ncomp, double dt,
                               double dx, int dir) {
  UpdateConservatively(MakeView(next, next_lo, next_hi),
                       MakeView(prev, prev_lo, prev_hi),
                       MakeView(fluxes, face_lo, face_hi), ncomp, dt, dx, dir);
}

// One directional sweep of a uniform grid (cons in/out, no ghosts).
void orc_grid_sweep(const orc_method* m, int rank, const int32_t* n,
                    const int32_t* bc, const double* dx, const double* cons_in,
                    double* cons_out, double dt, int dir, int nthreads,
                    int64_t* iters, int64_t* failures) {
  SetThreads(nthreads);
  const Grid g = MakeGrid(rank, n, bc, dx);
  DispatchRank(rank, [&](auto R) {
    constexpr int D = decltype(R)::value;
    GridSweep<D>(g, *m, cons_in, cons_out, dt, dir, iters, failures);
    return 0;
  });
}

double orc_grid_stable_dt(const orc_method* m, int rank, const int32_t* n,
                          const int32_t* bc, const double* dx,
                          const double* cons, int dir, int rule, int nthreads) {
  SetThreads(nthreads);
  const Grid g = MakeGrid(rank, n, bc, dx);
  return DispatchRank(rank, [&](auto R) {
    constexpr int D = decltype(R)::value;
    if (dir < 0) return GridStableDtAllDirs<D>(g, *m, cons, rule);
    return GridStableDt<D>(g, *m, cons, dir, rule);
  });
}

// One split step (Strang for rank >= 2) with a given dt and cycle parity.
int orc_grid_step(const orc_method* m, int rank, const int32_t* n,
                  const int32_t* bc, const double* dx, double* cons, double dt,
                  int cycle, int nthreads) {
  SetThreads(nthreads);
  const Grid g = MakeGrid(rank, n, bc, dx);
  return DispatchRank(rank, [&](auto R) {
    constexpr int D = decltype(R)::value;
    double fail_dt = 0.0;
    return AdvanceStep<D>(g, *m, cons, dt, cycle, 0, 0, &fail_dt, nullptr,
                          nullptr);
  });
}

int orc_run(const orc_method* m, int rank, const int32_t* n, const int32_t* bc,
            const double* dx, double* cons, double cfl, double t_end,
            int max_steps, int dt_rule, const double* dt_override,
            int n_override, double* dt_log, int* restarts, int nthreads,
            int64_t* iters, int64_t* failures) {
  SetThreads(nthreads);
  const Grid g = MakeGrid(rank, n, bc, dx);
  return DispatchRank(rank, [&](auto R) {
    constexpr int D = decltype(R)::value;
    return Run<D>(g, *m, cons, cfl, t_end, max_steps, dt_rule, dt_override,
                  n_override, dt_log, restarts, iters, failures);
  });
}

// Exact Riemann star state for n 1-D problems given as primitive states.
void orc_exact_star(int64_t n, const double* rhoL, const double* uL,
                    const double* pL, const double* rhoR, const double* uR,
                    const double* pR, int guess, const double* given,
                    double tol, int max_iterations, double* pstar,
                    double* ustar, int32_t* iterations, int32_t* converged) {
  const Gas eq;
  for (int64_t i = 0; i < n; ++i) {
    Complete<1> L, R;
    L.rho = rhoL[i];
    L.m[0] = rhoL[i] * uL[i];
    L.p = pL[i];
    L.E = pL[i] * eq.gamma_minus_1_inv + 0.5 * L.m[0] * L.m[0] / L.rho;
    L.c = std::sqrt(eq.gamma * L.p / L.rho);
    R.rho = rhoR[i];
    R.m[0] = rhoR[i] * uR[i];
    R.p = pR[i];
    R.E = pR[i] * eq.gamma_minus_1_inv + 0.5 * R.m[0] * R.m[0] / R.rho;
    R.c = std::sqrt(eq.gamma * R.p / R.rho);
    const StarState st = ComputeMiddleState<1>(eq, L, R, 0, guess,
                                               given ? given[i] : 0.0, tol,
                                               max_iterations);
    pstar[i] = st.pM;
    ustar[i] = st.uM;
    if (iterations) iterations[i] = st.iterations;
    if (converged) converged[i] = st.converged;
  }
}

}  // extern "C"
