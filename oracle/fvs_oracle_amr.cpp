// fvs_oracle_amr.cpp -- CPU oracle of the batched AMR patch update (2-D).
//
// TEST INFRASTRUCTURE ONLY (see fvs_oracle.hpp).  A plain restatement of a
// subcycled, refluxed block-structured AMR step, written independently of
// the library's table-driven implementation: every ghost cell's source is
// found by a geometric search at fill time.
//
// What it follows in the reference:
//  - SubcycleFineFirstSolver::AdvanceLevel: finer levels first, `ratio`
//    subcycles of dt/ratio, then this level, then the flux correction and
//    the conservative average-down (include/fub/solver/
//    SubcycleFineFirstSolver.hpp:114-175); the coarse step dt is
//    min over levels of ratio^l * stable dt of level l, times the CFL number
//    (SubcycleFineFirstSolver.hpp:100-112, RunSimulation.hpp:126-131);
//  - DimensionalSplitLevelIntegrator::AdvanceLevelNonRecursively with
//    StrangSplitting (x, y, y, x half steps) and the direction order of
//    MakeSplitDirections(coarse cycle, subcycle index)
//    (DimensionalSplitLevelIntegrator.hpp:221-276, SplittingMethod.hpp:115-126);
//  - the per-sweep stable-dt check and the restart of the coarse step with
//    ratio^l times the failing level's dt (DimensionalSplitLevelIntegrator.hpp:
//    240-245, SubcycleFineFirstSolver.hpp:121-127, RunSimulation.hpp:141-151);
//  - the per-patch MUSCL-Hancock + HLLE flux and conservative update of the
//    uniform oracle (FluxMethod.hpp:200-215, HyperbolicPatchIntegrator.cpp:
//    88-105);
//  - AMReX's FluxRegister (FineAdd / CrseInit / Reflux) and average_down as
//    called from src/AMReX/IntegratorContext.cpp:451-533, restated
//    arithmetically below (AMReX itself is not part of the reference tree).
//
// Design rules of this project (the library implements the same):
//  - ghost cells (2 layers, the side strips of each patch; corners are never
//    read by a split sweep) are refilled before every sweep: the boundary
//    condition maps the ghost position into the domain (periodic: wrap,
//    transmissive: clamp), then the value is copied from the level's patch
//    that owns that cell, or, where no patch of the level owns it, injected
//    (piecewise constant) from the coarser level's cell under it.  Fine
//    levels advance first, so the coarser data is the coarse step's start
//    state, as AMReX's FillPatchTwoLevels uses the single coarse time level;
//  - a coarse cell next to a coarse-fine face is corrected by
//    U += s * (0.5 * (F1 + F2) - Fc) / dx_c, with Fc the sum over the coarse
//    sweeps of dt_split * F at that face, F1 and F2 those of its two fine
//    sub-faces over all fine sweeps, s = +1 when the face is the cell's low
//    face and -1 when it is its high face; corrections of one cell are
//    applied in the order of (direction, side);
//  - average-down: U_c = (((f(2i,2j) + f(2i+1,2j)) + f(2i,2j+1)) + f(2i+1,2j+1)) * 0.25.
#include "fvs_oracle.hpp"

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <limits>
#include <set>
#include <tuple>
#include <unordered_map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

using namespace fvs_oracle;

namespace {

constexpr int kD = 2;
constexpr int kK = kD + 2;
constexpr int kG = 2;  // ghost layers

struct Patch {
  int level;
  int lo[2], hi[2];
  int n[2];
  std::vector<double> u;  // [K][n1 + 4][n0 + 4]
  int Pitch() const { return n[0] + 2 * kG; }
  int64_t Cs() const { return int64_t(n[0] + 2 * kG) * (n[1] + 2 * kG); }
  // local interior coordinates, ghosts at -2, -1, n, n+1
  double& At(int c, int i, int j) {
    return u[size_t(c * Cs() + int64_t(j + kG) * Pitch() + (i + kG))];
  }
  double At(int c, int i, int j) const {
    return u[size_t(c * Cs() + int64_t(j + kG) * Pitch() + (i + kG))];
  }
};

struct Level {
  int n[2];
  double dx;
  std::vector<int> patches;
  std::vector<int> owner;  // dense map cell -> patch index, -1 if none
  int Owner(int i, int j) const { return owner[size_t(int64_t(j) * n[0] + i)]; }
};

// one coarse-fine face: coarse cell C (level lc = fine level - 1) and its side
struct Slot {
  int ci, cj;   // coarse cell
  int dir;      // face normal
  int side;     // 0: low face of C (s = +1), 1: high face of C (s = -1)
  double coarse[kK];
  double fine[2][kK];
};

struct Hier {
  int nlevels;
  int bc[2];
  std::vector<Patch> patches;
  std::vector<Level> levels;
  std::vector<std::vector<Slot>> slots;  // slots[l]: faces between level l and l-1 (l >= 1)
  Gas eq;
  int limiter = 0;  // van Leer

  // periodic wrap, transmissive clamp, reflective mirror (ReflectIndex,
  // src/boundary_condition/ReflectiveBoundary.cpp:24-36)
  int MapCoord(int x, int n, int d) const {
    if (bc[d] == 0) return ((x % n) + n) % n;
    if (bc[d] == 2) return x < 0 ? -1 - x : (x >= n ? 2 * n - 1 - x : x);
    return x < 0 ? 0 : (x >= n ? n - 1 : x);
  }

  // value of cell (i, j) (already inside the domain) at level l
  void Value(int l, int i, int j, double* out) const {
    const int p = levels[size_t(l)].Owner(i, j);
    if (p >= 0) {
      const Patch& P = patches[size_t(p)];
      for (int c = 0; c < kK; ++c) out[c] = P.At(c, i - P.lo[0], j - P.lo[1]);
      return;
    }
    Value(l - 1, i >> 1, j >> 1, out);
  }

  void FillGhosts(int l) {
    const Level& L = levels[size_t(l)];
    const int np = int(L.patches.size());
#pragma omp parallel for schedule(dynamic, 4)
    for (int q = 0; q < np; ++q) {
      Patch& P = patches[size_t(L.patches[size_t(q)])];
      auto fill = [&](int li, int lj) {
        const int gi = P.lo[0] + li, gj = P.lo[1] + lj;
        const int si = MapCoord(gi, L.n[0], 0);
        const int sj = MapCoord(gj, L.n[1], 1);
        double v[kK];
        Value(l, si, sj, v);
        // a reflective wall's ghost: Reflect of the mirror cell's state
        if (bc[0] == 2 && (gi < 0 || gi >= L.n[0])) ReflectMomentum<2>(v + 1, 0);
        if (bc[1] == 2 && (gj < 0 || gj >= L.n[1])) ReflectMomentum<2>(v + 1, 1);
        for (int c = 0; c < kK; ++c) P.At(c, li, lj) = v[c];
      };
      for (int lj = 0; lj < P.n[1]; ++lj)
        for (int g = 1; g <= kG; ++g) {
          fill(-g, lj);
          fill(P.n[0] - 1 + g, lj);
        }
      for (int li = 0; li < P.n[0]; ++li)
        for (int g = 1; g <= kG; ++g) {
          fill(li, -g);
          fill(li, P.n[1] - 1 + g);
        }
    }
  }

  // Max signal speed over the faces 0..n of every patch row of level l in
  // direction d (ghosts filled): the level's stable dt is dx / max.
  double MaxSpeed(int l, int d) const {
    const Level& L = levels[size_t(l)];
    double smax = 0.0;
    for (int q : L.patches) {
      const Patch& P = patches[size_t(q)];
      const int nd = P.n[d], nt = P.n[1 - d];
      for (int t = 0; t < nt; ++t) {
        for (int f = 0; f <= nd; ++f) {
          Complete<kD> a, b;
          double ua[kK], ub[kK];
          for (int c = 0; c < kK; ++c) {
            ua[c] = d == 0 ? P.At(c, f - 1, t) : P.At(c, t, f - 1);
            ub[c] = d == 0 ? P.At(c, f, t) : P.At(c, t, f);
          }
          CompleteFromCons<kD>(eq, a, ua);
          CompleteFromCons<kD>(eq, b, ub);
          // the face speed of HllStableDt (fvs_oracle.hpp; HllMethod.hpp:
          // 337-347) with its NaN rule: a NaN sound speed (negative
          // pressure) gives either |sR| or NaN, and NaN face speeds are
          // skipped by the max, as in the uniform-grid restatement
          double sL, sR;
          Einfeldt<kD>(eq, a, b, d, sL, sR);
          const double s = PMax(PMax(0.0, std::abs(sL)), std::abs(sR));
          smax = s > smax ? s : smax;
        }
      }
    }
    return smax;
  }

  double StableDt(int l, int d) const { return levels[size_t(l)].dx / MaxSpeed(l, d); }

  // One sweep of every patch of level l in direction d with step dt_split.
  void Sweep(int l, int d, double dt_split) {
    const Level& L = levels[size_t(l)];
    const double dx = L.dx;
    const double lambda_half = 0.5 * dt_split / dx;
    const double dt_dx = dt_split / dx;
    const int np = int(L.patches.size());
#pragma omp parallel for schedule(dynamic, 2)
    for (int q = 0; q < np; ++q) {
      Patch& P = patches[size_t(L.patches[size_t(q)])];
      const int nd = P.n[d], nt = P.n[1 - d];
      std::vector<double> F(size_t(nd + 1) * kK);
      std::vector<double> next(size_t(nd) * kK);
      for (int t = 0; t < nt; ++t) {
        auto load = [&](double* u, int x) {
          for (int c = 0; c < kK; ++c) u[c] = d == 0 ? P.At(c, x, t) : P.At(c, t, x);
        };
        for (int f = 0; f <= nd; ++f) {
          double u[4][kK];
          for (int s = 0; s < 4; ++s) load(u[s], f - 2 + s);
          Complete<kD> rec0, rec1;
          MusclPredict<kD>(eq, rec0, u[0], u[1], u[2], limiter, lambda_half, d, +1);
          MusclPredict<kD>(eq, rec1, u[1], u[2], u[3], limiter, lambda_half, d, -1);
          HllFlux<kD>(eq, &F[size_t(f) * kK], rec0, rec1, d);
        }
        for (int x = 0; x < nd; ++x) {
          for (int c = 0; c < kK; ++c) {
            const double U = d == 0 ? P.At(c, x, t) : P.At(c, t, x);
            next[size_t(x) * kK + c] =
                U + dt_dx * (F[size_t(x) * kK + c] - F[size_t(x + 1) * kK + c]);
          }
        }
        // coarse-fine register contributions of this row
        Capture(l, P, d, t, F, dt_split);
        for (int x = 0; x < nd; ++x)
          for (int c = 0; c < kK; ++c) {
            if (d == 0)
              P.At(c, x, t) = next[size_t(x) * kK + c];
            else
              P.At(c, t, x) = next[size_t(x) * kK + c];
          }
      }
    }
  }

  // Register contributions of one swept row: the coarse faces of level l's
  // rows (slots of level l+1) and the fine faces (slots of level l).
  void Capture(int l, const Patch& P, int d, int t, const std::vector<double>& F,
               double dt_split) {
    (void)l;
    const auto it = caps.find(CapKey(&P - patches.data(), d, t));
    if (it == caps.end()) return;
    for (const Cap& c : it->second) {
      double* dst = c.sub < 0 ? c.slot->coarse : c.slot->fine[c.sub];
      for (int k = 0; k < kK; ++k) dst[k] += dt_split * F[size_t(c.face) * kK + k];
    }
  }

  struct Cap {
    int face;  // face index in the row (0..n)
    int sub;   // -1: coarse face, 0/1: fine sub-face
    Slot* slot;
  };
  std::unordered_map<int64_t, std::vector<Cap>> caps;
  static int64_t CapKey(int64_t patch, int d, int t) { return ((patch * 2 + d) << 24) | t; }

  void BuildSlots() {
    slots.assign(size_t(nlevels), {});
    for (int l = 1; l < nlevels; ++l) {
      const Level& L = levels[size_t(l)];
      std::vector<Slot>& S = slots[size_t(l)];
      std::set<std::tuple<int64_t, int, int>> seen;
      const int ncx = levels[size_t(l - 1)].n[0];
      for (int q : L.patches) {
        const Patch& P = patches[size_t(q)];
        for (int d = 0; d < 2; ++d) {
          const int nt = P.n[1 - d];
          for (int t = 0; t < nt; ++t) {
            for (int end = 0; end < 2; ++end) {
              const int x_in = end == 0 ? 0 : P.n[d] - 1;
              const int step = end == 0 ? -1 : 1;
              const int gi = P.lo[0] + (d == 0 ? x_in : t);
              const int gj = P.lo[1] + (d == 0 ? t : x_in);
              int oi = gi + (d == 0 ? step : 0);
              int oj = gj + (d == 0 ? 0 : step);
              const int on = d == 0 ? oi : oj;
              if (bc[d] != 0 && (on < 0 || on >= L.n[d])) continue;  // physical boundary
              oi = MapCoord(oi, L.n[0], 0);
              oj = MapCoord(oj, L.n[1], 1);
              if (L.Owner(oi, oj) >= 0) continue;  // same-level neighbour
              const int ci = oi >> 1, cj = oj >> 1;
              // the fine region lies on C's low side when the fine cell steps up
              const int side = step > 0 ? 0 : 1;
              if (seen.insert({int64_t(cj) * ncx + ci, d, side}).second) {
                Slot sl{};
                sl.ci = ci;
                sl.cj = cj;
                sl.dir = d;
                sl.side = side;
                S.push_back(sl);
              }
            }
          }
        }
      }
      std::sort(S.begin(), S.end(), [ncx](const Slot& a, const Slot& b) {
        const int64_t ka = int64_t(a.cj) * ncx + a.ci, kb = int64_t(b.cj) * ncx + b.ci;
        if (ka != kb) return ka < kb;
        if (a.dir != b.dir) return a.dir < b.dir;
        return a.side < b.side;
      });
    }
    // where each slot's fluxes are computed
    for (int l = 1; l < nlevels; ++l) {
      const Level& C = levels[size_t(l - 1)];
      const Level& Fl = levels[size_t(l)];
      for (Slot& sl : slots[size_t(l)]) {
        const int d = sl.dir;
        const int cp = C.Owner(sl.ci, sl.cj);
        const Patch& CP = patches[size_t(cp)];
        const int cx = (d == 0 ? sl.ci : sl.cj) - CP.lo[d];
        const int ct = (d == 0 ? sl.cj : sl.ci) - CP.lo[1 - d];
        caps[CapKey(cp, d, ct)].push_back({sl.side == 0 ? cx : cx + 1, -1, &sl});
        // fine cells across the face: the covered coarse neighbour's cells next to it
        const int cn = (d == 0 ? sl.ci : sl.cj) + (sl.side == 0 ? -1 : 1);
        const int cnw = MapCoord(cn, C.n[d], d);
        const int fx = sl.side == 0 ? 2 * cnw + 1 : 2 * cnw;
        for (int sub = 0; sub < 2; ++sub) {
          const int ft = 2 * (d == 0 ? sl.cj : sl.ci) + sub;
          const int fi = d == 0 ? fx : ft, fj = d == 0 ? ft : fx;
          const int fp = Fl.Owner(fi, fj);
          const Patch& FP = patches[size_t(fp)];
          const int lx = (d == 0 ? fi : fj) - FP.lo[d];
          const int lt = (d == 0 ? fj : fi) - FP.lo[1 - d];
          caps[CapKey(fp, d, lt)].push_back({sl.side == 0 ? lx + 1 : lx, sub, &sl});
        }
      }
    }
  }

  void ResetSlots(int l) {
    for (Slot& s : slots[size_t(l)]) {
      std::memset(s.coarse, 0, sizeof s.coarse);
      std::memset(s.fine, 0, sizeof s.fine);
    }
  }

  void Reflux(int l) {  // slots of level l correct level l-1
    const Level& C = levels[size_t(l - 1)];
    for (const Slot& s : slots[size_t(l)]) {
      const int p = C.Owner(s.ci, s.cj);
      Patch& P = patches[size_t(p)];
      const double sign = s.side == 0 ? 1.0 : -1.0;
      for (int c = 0; c < kK; ++c) {
        const double delta = 0.5 * (s.fine[0][c] + s.fine[1][c]) - s.coarse[c];
        double& U = P.At(c, s.ci - P.lo[0], s.cj - P.lo[1]);
        U = U + sign * delta / C.dx;
      }
    }
  }

  void AverageDown(int l) {  // level l onto level l-1
    const Level& F = levels[size_t(l)];
    for (int q : F.patches) {
      const Patch& P = patches[size_t(q)];
      for (int j = P.lo[1]; j < P.hi[1]; j += 2) {
        for (int i = P.lo[0]; i < P.hi[0]; i += 2) {
          const int ci = i >> 1, cj = j >> 1;
          const int cp = levels[size_t(l - 1)].Owner(ci, cj);
          Patch& Q = patches[size_t(cp)];
          for (int c = 0; c < kK; ++c) {
            const double a = P.At(c, i - P.lo[0], j - P.lo[1]);
            const double b = P.At(c, i + 1 - P.lo[0], j - P.lo[1]);
            const double e = P.At(c, i - P.lo[0], j + 1 - P.lo[1]);
            const double f = P.At(c, i + 1 - P.lo[0], j + 1 - P.lo[1]);
            Q.At(c, ci - Q.lo[0], cj - Q.lo[1]) = (((a + b) + e) + f) * 0.25;
          }
        }
      }
    }
  }

  // AdvanceLevelNonRecursively; returns 1 and the scaled failing dt on a
  // failed per-sweep check.
  int AdvanceLevelOnly(int l, double dt, int cycle, int sub, int check, double* fail_dt) {
    const int is_odd = (cycle % 2 + sub) % 2;
    const int d0 = is_odd ? 1 : 0, d1 = 1 - d0;
    const int seq[4] = {d0, d1, d1, d0};
    const double split_dt = 0.5 * dt;
    for (int s = 0; s < 4; ++s) {
      const int d = seq[s];
      FillGhosts(l);
      if (check) {
        const double level_dt = StableDt(l, d);
        if (level_dt < split_dt) {
          *fail_dt = level_dt * double(1 << l);
          return 1;
        }
      }
      Sweep(l, d, split_dt);
    }
    return 0;
  }

  int AdvanceLevel(int l, double dt, int cycle, int sub, int check, double* fail_dt) {
    if (l + 1 < nlevels) {
      ResetSlots(l + 1);
      for (int r = 0; r < 2; ++r)
        if (AdvanceLevel(l + 1, 0.5 * dt, cycle, r, check, fail_dt)) return 1;
    }
    if (AdvanceLevelOnly(l, dt, cycle, sub, check, fail_dt)) return 1;
    if (l + 1 < nlevels) {
      Reflux(l + 1);
      AverageDown(l + 1);
    }
    return 0;
  }

  double CoarseStableDt() {
    double dt = std::numeric_limits<double>::max();
    for (int l = 0; l < nlevels; ++l) {
      FillGhosts(l);
      for (int d = 0; d < 2; ++d) dt = std::min(dt, double(1 << l) * StableDt(l, d));
    }
    return dt;
  }
};

}  // namespace

extern "C" {

// Runs the AMR hierarchy.  Patches: level plevel[p], box pbox[4p..4p+3] =
// (lo0, lo1, hi0, hi1) in that level's index space.  cons: the patches'
// interiors concatenated in patch order, each [4][ny][nx]; advanced in place.
// dt_override (n_override entries) replaces the CFL step for the first steps
// and disables the checks there.  Returns the number of coarse steps, or -1
// on an invalid hierarchy.
int orc_amr_run(int nlevels, const int32_t* n0, const int32_t* bc, double dx0, int npatch,
                const int32_t* plevel, const int32_t* pbox, double* cons, double cfl,
                double t_end, int max_steps, const double* dt_override, int n_override,
                double* dt_log, int* restarts, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  Hier h;
  h.nlevels = nlevels;
  h.bc[0] = bc[0];
  h.bc[1] = bc[1];
  h.levels.resize(size_t(nlevels));
  for (int l = 0; l < nlevels; ++l) {
    Level& L = h.levels[size_t(l)];
    L.n[0] = n0[0] << l;
    L.n[1] = n0[1] << l;
    L.dx = dx0 / double(1 << l);
    L.owner.assign(size_t(int64_t(L.n[0]) * L.n[1]), -1);
  }
  h.patches.resize(size_t(npatch));
  int64_t off = 0;
  for (int p = 0; p < npatch; ++p) {
    Patch& P = h.patches[size_t(p)];
    P.level = plevel[p];
    if (P.level < 0 || P.level >= nlevels) return -1;
    for (int d = 0; d < 2; ++d) {
      P.lo[d] = pbox[4 * p + d];
      P.hi[d] = pbox[4 * p + 2 + d];
      P.n[d] = P.hi[d] - P.lo[d];
    }
    P.u.assign(size_t(kK * P.Cs()), 0.0);
    Level& L = h.levels[size_t(P.level)];
    L.patches.push_back(p);
    for (int j = P.lo[1]; j < P.hi[1]; ++j)
      for (int i = P.lo[0]; i < P.hi[0]; ++i) {
        if (L.owner[size_t(int64_t(j) * L.n[0] + i)] >= 0) return -1;
        L.owner[size_t(int64_t(j) * L.n[0] + i)] = p;
      }
    for (int c = 0; c < kK; ++c)
      for (int j = 0; j < P.n[1]; ++j)
        for (int i = 0; i < P.n[0]; ++i) P.At(c, i, j) = cons[off++];
  }
  h.BuildSlots();

  const double eps = 1e-12;
  double t = 0.0;
  int step = 0, n_restarts = 0;
  bool have_failure = false;
  double failure_dt = 0.0;
  std::vector<std::vector<double>> backup(static_cast<size_t>(npatch));
  while (t + eps < t_end && (max_steps < 0 || step < max_steps)) {
    double dt;
    const bool fixed = dt_override && step < n_override;
    if (fixed) {
      dt = dt_override[step];
    } else {
      const double stable = have_failure ? failure_dt : h.CoarseStableDt();
      dt = std::min(t_end - t, cfl * stable);
    }
    for (int p = 0; p < npatch; ++p) backup[size_t(p)] = h.patches[size_t(p)].u;
    double fail_dt = 0.0;
    if (h.AdvanceLevel(0, dt, step, 0, !fixed, &fail_dt)) {
      for (int p = 0; p < npatch; ++p) h.patches[size_t(p)].u = backup[size_t(p)];
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
  off = 0;
  for (int p = 0; p < npatch; ++p) {
    const Patch& P = h.patches[size_t(p)];
    for (int c = 0; c < kK; ++c)
      for (int j = 0; j < P.n[1]; ++j)
        for (int i = 0; i < P.n[0]; ++i) cons[off++] = P.At(c, i, j);
  }
  if (restarts) *restarts = n_restarts;
  return step;
}

}  // extern "C"
