// fvs_amr.cu -- host side of the batched AMR patch update (2-D, ratio 2).
//
// Builds, once per hierarchy, every table the device needs: the rows of the
// patches per level and direction (the work of one persistent sweep launch)
// with the sources of their halo cells (same-level cells after the boundary
// condition's mapping, or piecewise-constant injection from the coarser
// level), the flux-register captures, the reflux lists and the average-down
// lists.  A coarse step -- stable dt of every level, dt selection, the
// fine-first subcycled Strang sweeps of all levels, refluxing, average-down
// and the per-sweep CFL checks -- is one CUDA graph (one per parity of the
// cycle counter, which fixes the direction order).  The semantics follow
// SubcycleFineFirstSolver (include/fub/solver/SubcycleFineFirstSolver.hpp:
// 100-191) and DimensionalSplitLevelIntegrator (include/fub/solver/
// DimensionalSplitLevelIntegrator.hpp:204-276) with these rules of this
// library: every sweep sees its level's ghost cells as they are at that
// sweep (it reads a row's halo from the neighbouring patch's current cells,
// so a level split into patches advances exactly like one uniform grid), and
// a fine level's ghost cells outside that level are injected from the
// coarser level's state at the start of the coarse step (fine levels advance
// first).
#include "../../include/fvs_gpu.h"
#include "fvs_amr.h"
#include "fvs_internal.h"
#include "fvs_plotfile.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <tuple>
#include <vector>

using namespace fvs::amr;

namespace {

struct PatchHost {
  int level;
  int lo[2], hi[2], n[2];
  int32_t block_start;
  int32_t pitch;
  int32_t row_offset[2];  // first row id of this patch per direction
};

struct LevelHost {
  int n[2];
  double dx;
  std::vector<int> patches;
  std::vector<int32_t> owner;
  int64_t ncells = 0;
  double* A = nullptr;
  double* B = nullptr;
  double* backup = nullptr;
  int32_t nrows[2] = {0, 0};
  Seg* segs[2][kSplits] = {};
  int32_t nsegs[2][kSplits] = {};
  int split[2] = {0, 0};  // index into kSplitOf; kSplits: x rows with lanes along x
  // slots of the x sweep with lanes along x (PatchSweepArgs::slot_row)
  int32_t* slot_row = nullptr;
  int32_t* row_slot0 = nullptr;
  int64_t nslots = 0;
  Cap* caps[2] = {nullptr, nullptr};
  RefluxCell* reflux = nullptr;
  int32_t nreflux = 0;
  AvgDown* avg = nullptr;
  int32_t navg = 0;
  int32_t slot_begin = 0, slot_end = 0;
  int block[2] = {128, 128};
  int grid[2] = {0, 0};
  int occ[2] = {0, 0};  // occupancy variant of the mixed sweep
  std::string hist;
  int32_t Owner(int i, int j) const { return owner[size_t(int64_t(j) * n[0] + i)]; }
};

std::mutex g_tune_mutex;
struct Tuned {
  int block, grid, occ, split;
};
std::map<std::string, Tuned> g_tuned;  // key -> launch shape

}  // namespace

struct fvs_amr {
  int nlevels = 0;
  int bc[2] = {1, 1};
  int n0[2] = {0, 0};
  double dx0 = 0.0;
  fvs_method m{};
  std::vector<PatchHost> patches;
  std::vector<LevelHost> L;
  std::vector<std::vector<int>> level_patch_order;
  double* reg = nullptr;
  int32_t nslots = 0;
  float* signs = nullptr;
  AmrControl* ctrl = nullptr;
  AmrControl* ctrl_host = nullptr;
  SweepInfo* sweeps = nullptr;
  int nsweeps = 0;
  double* tune_dt = nullptr;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  int64_t cycle = 0;
  double t = 0.0;
  int sms = 152;
  std::vector<void*> allocations;

  ~fvs_amr() {
    if (stream) cudaStreamSynchronize(stream);
    for (auto& g : graph)
      if (g) cudaGraphExecDestroy(g);
    for (void* p : allocations) cudaFree(p);
    if (ctrl_host) cudaFreeHost(ctrl_host);
    if (stream) cudaStreamDestroy(stream);
  }
  template <class T> cudaError_t Alloc(T** p, size_t count) {
    void* v = nullptr;
    cudaError_t e = cudaMalloc(&v, std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) {
      allocations.push_back(v);
      e = cudaMemset(v, 0, std::max<size_t>(count, 1) * sizeof(T));
    }
    *p = static_cast<T*>(v);
    return e;
  }
  template <class T> cudaError_t Upload(T** p, const std::vector<T>& h) {
    cudaError_t e = Alloc(p, h.size());
    if (e == cudaSuccess && !h.empty())
      e = cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
    return e;
  }
  int32_t SI(int p, int i, int j) const {  // storage index of cell (i, j) of patch p
    const PatchHost& P = patches[size_t(p)];
    return P.block_start + (j - P.lo[1] + kGhost) * P.pitch + (i - P.lo[0] + kGhost);
  }
  // level coordinate x of a direction of n cells mapped into the domain:
  // periodic wrap, transmissive clamp, reflective mirror (ReflectIndex)
  int MapCoord(int x, int n, int d) const {
    if (bc[d] == 0) return ((x % n) + n) % n;
    if (bc[d] == 2) return x < 0 ? -1 - x : (x >= n ? 2 * n - 1 - x : x);
    return x < 0 ? 0 : (x >= n ? n - 1 : x);
  }
};

namespace {

int Fail(int code, const std::string& msg) {
  fvs::SetLastError(msg);
  return code;
}

int CudaFail(cudaError_t e, const char* what) {
  fvs::SetLastError(std::string(what) + ": " + cudaGetErrorString(e));
  return FVS_ERR_CUDA;
}

#define AMR_CUDA(call)                                 \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return CudaFail(e_, #call); \
  } while (0)

struct SlotHost {
  int ci, cj, dir, side;
};

int Build(fvs_amr* a) {
  const int nl = a->nlevels;
  a->L.resize(size_t(nl));
  for (int l = 0; l < nl; ++l) {
    LevelHost& L = a->L[size_t(l)];
    L.n[0] = a->n0[0] << l;
    L.n[1] = a->n0[1] << l;
    L.dx = a->dx0 / double(1 << l);
    const int64_t cells = int64_t(L.n[0]) * L.n[1];
    if (cells > (int64_t(1) << 28)) return Fail(FVS_ERR_INVALID, "level index space too large");
    L.owner.assign(size_t(cells), -1);
  }
  // storage blocks and owner maps
  for (size_t p = 0; p < a->patches.size(); ++p) {
    PatchHost& P = a->patches[p];
    LevelHost& L = a->L[size_t(P.level)];
    P.pitch = P.n[0] + 2 * kGhost;
    const int64_t blk = int64_t(P.pitch) * (P.n[1] + 2 * kGhost);
    if (L.ncells + blk > (int64_t(1) << 31) - 1)
      return Fail(FVS_ERR_INVALID, "level storage exceeds 2^31 cells");
    P.block_start = static_cast<int32_t>(L.ncells);
    L.ncells += blk;
    L.patches.push_back(int(p));
    for (int j = P.lo[1]; j < P.hi[1]; ++j)
      for (int i = P.lo[0]; i < P.hi[0]; ++i) {
        int32_t& o = L.owner[size_t(int64_t(j) * L.n[0] + i)];
        if (o >= 0) return Fail(FVS_ERR_INVALID, "patches of one level overlap");
        o = int32_t(p);
      }
  }
  for (int32_t o : a->L[0].owner)
    if (o < 0) return Fail(FVS_ERR_INVALID, "level-0 patches must cover the domain");

  // rows per level and direction
  std::vector<std::vector<Row>> rows_h[2];
  for (int d = 0; d < 2; ++d) rows_h[d].resize(size_t(nl));
  for (int l = 0; l < nl; ++l) {
    LevelHost& L = a->L[size_t(l)];
    for (int d = 0; d < 2; ++d) {
      std::vector<Row>& R = rows_h[d][size_t(l)];
      for (int p : L.patches) {
        PatchHost& P = a->patches[size_t(p)];
        P.row_offset[d] = int32_t(R.size());
        const int nt = P.n[1 - d];
        for (int t = 0; t < nt; ++t) {
          Row r{};
          if (d == 0) {
            r.base = P.block_start + (t + kGhost) * P.pitch;
            r.stride = 1;
            r.n = P.n[0];
          } else {
            r.base = P.block_start + (t + kGhost);
            r.stride = P.pitch;
            r.n = P.n[1];
          }
          R.push_back(r);
        }
      }
      L.nrows[d] = int32_t(R.size());
    }
  }

  // halo sources of every row end: the cell a ghost fill would copy into the
  // halo (same level after the boundary condition's mapping, else the
  // coarser cell under it); also checks the nesting of the patches
  for (int l = 0; l < nl; ++l) {
    const LevelHost& L = a->L[size_t(l)];
    for (int p : L.patches) {
      const PatchHost& P = a->patches[size_t(p)];
      auto src_of = [&](int li, int lj, int32_t& src) -> int {
        const int gi = P.lo[0] + li, gj = P.lo[1] + lj;
        const int si = a->MapCoord(gi, L.n[0], 0), sj = a->MapCoord(gj, L.n[1], 1);
        const int32_t o = L.Owner(si, sj);
        if (o >= 0) {
          src = a->SI(o, si, sj);
          return FVS_OK;
        }
        if (l == 0) return Fail(FVS_ERR_INVALID, "level 0 does not cover the domain");
        const LevelHost& C = a->L[size_t(l - 1)];
        const int32_t co = C.Owner(si >> 1, sj >> 1);
        if (co < 0)
          return Fail(FVS_ERR_INVALID,
                      "patches are not properly nested: a ghost cell of level " +
                          std::to_string(l) + " has no coarser cell under it");
        src = -a->SI(co, si >> 1, sj >> 1) - 1;
        return FVS_OK;
      };
      for (int d = 0; d < 2; ++d) {
        const int nt = P.n[1 - d], nd = P.n[d];
        for (int t = 0; t < nt; ++t) {
          Row& r = rows_h[d][size_t(l)][size_t(P.row_offset[d] + t)];
          const int pos[4] = {-2, -1, nd, nd + 1};
          r.flip = 0;
          for (int h = 0; h < 4; ++h) {
            const int li = d == 0 ? pos[h] : t, lj = d == 0 ? t : pos[h];
            if (int e = src_of(li, lj, r.halo[h])) return e;
            const int g = P.lo[d] + pos[h];
            if (a->bc[d] == FVS_BC_REFLECTIVE && (g < 0 || g >= L.n[d])) r.flip |= 1 << h;
          }
        }
      }
    }
  }

  // coarse-fine faces (register slots), captures, reflux and average-down
  std::vector<std::vector<std::vector<Cap>>> caps_h[2];  // [d][l][row]
  for (int d = 0; d < 2; ++d) {
    caps_h[d].resize(size_t(nl));
    for (int l = 0; l < nl; ++l) caps_h[d][size_t(l)].resize(size_t(a->L[size_t(l)].nrows[d]));
  }
  std::vector<float> signs_h;
  std::vector<std::vector<RefluxCell>> reflux_h(static_cast<size_t>(nl));
  std::vector<std::vector<AvgDown>> avg_h(static_cast<size_t>(nl));
  int32_t gslot = 0;
  for (int l = 1; l < nl; ++l) {
    LevelHost& F = a->L[size_t(l)];
    const LevelHost& C = a->L[size_t(l - 1)];
    std::set<std::tuple<int64_t, int, int>> seen;
    std::vector<SlotHost> S;
    for (int p : F.patches) {
      const PatchHost& P = a->patches[size_t(p)];
      for (int d = 0; d < 2; ++d) {
        for (int t = 0; t < P.n[1 - d]; ++t) {
          for (int end = 0; end < 2; ++end) {
            const int x_in = end == 0 ? 0 : P.n[d] - 1;
            const int step = end == 0 ? -1 : 1;
            const int gi = P.lo[0] + (d == 0 ? x_in : t);
            const int gj = P.lo[1] + (d == 0 ? t : x_in);
            int oi = gi + (d == 0 ? step : 0), oj = gj + (d == 0 ? 0 : step);
            const int on = d == 0 ? oi : oj;
            if (a->bc[d] != FVS_BC_PERIODIC && (on < 0 || on >= F.n[d])) continue;
            oi = a->MapCoord(oi, F.n[0], 0);
            oj = a->MapCoord(oj, F.n[1], 1);
            if (F.Owner(oi, oj) >= 0) continue;
            const int ci = oi >> 1, cj = oj >> 1;
            const int side = step > 0 ? 0 : 1;
            if (seen.insert({int64_t(cj) * C.n[0] + ci, d, side}).second)
              S.push_back({ci, cj, d, side});
          }
        }
      }
    }
    std::sort(S.begin(), S.end(), [&C](const SlotHost& x, const SlotHost& y) {
      const int64_t kx = int64_t(x.cj) * C.n[0] + x.ci, ky = int64_t(y.cj) * C.n[0] + y.ci;
      if (kx != ky) return kx < ky;
      if (x.dir != y.dir) return x.dir < y.dir;
      return x.side < y.side;
    });
    F.slot_begin = gslot;
    for (size_t k = 0; k < S.size(); ++k) {
      const SlotHost& s = S[k];
      const int32_t gs = gslot + int32_t(k);
      const int d = s.dir;
      const int32_t cp = C.Owner(s.ci, s.cj);
      if (cp < 0) return Fail(FVS_ERR_INVALID, "coarse-fine face without a coarse cell");
      const PatchHost& CP = a->patches[size_t(cp)];
      const int cx = (d == 0 ? s.ci : s.cj) - CP.lo[d];
      const int ct = (d == 0 ? s.cj : s.ci) - CP.lo[1 - d];
      caps_h[d][size_t(l - 1)][size_t(CP.row_offset[d] + ct)].push_back(
          {s.side == 0 ? cx : cx + 1, 3 * gs});
      const int cn = a->MapCoord((d == 0 ? s.ci : s.cj) + (s.side == 0 ? -1 : 1), C.n[d], d);
      const int fx = s.side == 0 ? 2 * cn + 1 : 2 * cn;
      for (int sub = 0; sub < 2; ++sub) {
        const int ft = 2 * (d == 0 ? s.cj : s.ci) + sub;
        const int fi = d == 0 ? fx : ft, fj = d == 0 ? ft : fx;
        const int32_t fp = F.Owner(fi, fj);
        if (fp < 0) return Fail(FVS_ERR_INVALID, "coarse-fine face without its fine cells");
        const PatchHost& FP = a->patches[size_t(fp)];
        const int lx = (d == 0 ? fi : fj) - FP.lo[d];
        const int lt = (d == 0 ? fj : fi) - FP.lo[1 - d];
        caps_h[d][size_t(l)][size_t(FP.row_offset[d] + lt)].push_back(
            {s.side == 0 ? lx + 1 : lx, 3 * gs + 1 + sub});
      }
      signs_h.push_back(s.side == 0 ? 1.0f : -1.0f);
      const int32_t cell = a->SI(cp, s.ci, s.cj);
      if (!reflux_h[size_t(l)].empty() && reflux_h[size_t(l)].back().cell == cell) {
        reflux_h[size_t(l)].back().count += 1;
      } else {
        reflux_h[size_t(l)].push_back({cell, gs, 1, 0});
      }
    }
    gslot += int32_t(S.size());
    F.slot_end = gslot;
    for (int p : F.patches) {
      const PatchHost& P = a->patches[size_t(p)];
      for (int j = P.lo[1]; j < P.hi[1]; j += 2)
        for (int i = P.lo[0]; i < P.hi[0]; i += 2) {
          const int32_t co = C.Owner(i >> 1, j >> 1);
          if (co < 0) return Fail(FVS_ERR_INVALID, "fine patch outside the coarser level");
          avg_h[size_t(l)].push_back({a->SI(co, i >> 1, j >> 1), a->SI(p, i, j), P.pitch, 0});
        }
    }
  }
  a->nslots = gslot;

  // flatten captures per row (sorted by face), checking one capture per face
  std::vector<std::vector<Cap>> caps_flat[2];
  for (int d = 0; d < 2; ++d) {
    caps_flat[d].resize(size_t(nl));
    for (int l = 0; l < nl; ++l) {
      std::vector<Row>& R = rows_h[d][size_t(l)];
      std::vector<Cap>& flat = caps_flat[d][size_t(l)];
      for (size_t r = 0; r < R.size(); ++r) {
        std::vector<Cap>& c = caps_h[d][size_t(l)][r];
        std::sort(c.begin(), c.end(), [](const Cap& x, const Cap& y) { return x.face < y.face; });
        for (size_t k = 1; k < c.size(); ++k)
          if (c[k].face == c[k - 1].face)
            return Fail(FVS_ERR_INVALID, "a face is both a coarse and a fine register face");
        flat.insert(flat.end(), c.begin(), c.end());
        R[r].cap_end = int32_t(flat.size());
      }
    }
  }

  // device allocations
  for (int l = 0; l < nl; ++l) {
    LevelHost& Lv = a->L[size_t(l)];
    const size_t n = size_t(Lv.ncells) * kComp;
    AMR_CUDA(a->Alloc(&Lv.A, n));
    AMR_CUDA(a->Alloc(&Lv.B, n));
    AMR_CUDA(a->Alloc(&Lv.backup, n));
    for (int d = 0; d < 2; ++d) {
      const std::vector<Row>& R = rows_h[d][size_t(l)];
      const std::vector<Cap>& flat = caps_flat[d][size_t(l)];
      AMR_CUDA(a->Upload(&Lv.caps[d], flat));
      // the rows split into 1, 2 or 4 segments (threads per row)
      for (int si = 0; si < kSplits; ++si) {
        std::vector<Seg> segs;
        for (size_t r = 0; r < R.size(); ++r) {
          const int nn = R[r].n;
          const int parts = std::max(1, std::min(kSplitOf[si], nn));
          const int32_t cb = r > 0 ? R[r - 1].cap_end : 0, ce = R[r].cap_end;
          int32_t c = cb;
          for (int k = 0; k < parts; ++k) {
            Seg sg{};
            sg.base = R[r].base;
            sg.stride = R[r].stride;
            sg.n = nn;
            for (int h = 0; h < 4; ++h) sg.halo[h] = R[r].halo[h];
            sg.flip = R[r].flip;
            sg.j0 = int32_t(int64_t(k) * nn / parts);
            sg.j1 = int32_t(int64_t(k + 1) * nn / parts);
            sg.cap_begin = c;
            if (k + 1 < parts) {
              while (c < ce && flat[size_t(c)].face < sg.j1) ++c;
            } else {
              c = ce;
            }
            sg.cap_end = c;
            segs.push_back(sg);
          }
        }
        Lv.nsegs[d][si] = int32_t(segs.size());
        AMR_CUDA(a->Upload(&Lv.segs[d][si], segs));
      }
      if (d == 0) {
        // x rows end to end as slots, cells -1..n of each
        std::vector<int32_t> slot_row, row_slot0(R.size());
        for (size_t r = 0; r < R.size(); ++r) {
          row_slot0[r] = int32_t(slot_row.size());
          slot_row.insert(slot_row.end(), size_t(R[r].n) + 2, int32_t(r));
        }
        Lv.nslots = int64_t(slot_row.size());
        AMR_CUDA(a->Upload(&Lv.slot_row, slot_row));
        AMR_CUDA(a->Upload(&Lv.row_slot0, row_slot0));
      }
    }
    AMR_CUDA(a->Upload(&Lv.reflux, reflux_h[size_t(l)]));
    Lv.nreflux = int32_t(reflux_h[size_t(l)].size());
    AMR_CUDA(a->Upload(&Lv.avg, avg_h[size_t(l)]));
    Lv.navg = int32_t(avg_h[size_t(l)].size());
    // patch-size histogram (the autotuner's key)
    std::map<std::pair<int, int>, int> h;
    for (int p : Lv.patches) h[{a->patches[size_t(p)].n[0], a->patches[size_t(p)].n[1]}] += 1;
    for (auto& kv : h)
      Lv.hist += std::to_string(kv.first.first) + "x" + std::to_string(kv.first.second) + ":" +
                 std::to_string(kv.second) + ",";
    for (int d = 0; d < 2; ++d)
      Lv.grid[d] = std::max(1, std::min((Lv.nsegs[d][0] + 127) / 128, a->sms * 4));
  }
  AMR_CUDA(a->Alloc(&a->reg, size_t(std::max(a->nslots, 1)) * 3 * kComp));
  AMR_CUDA(a->Upload(&a->signs, signs_h));
  AMR_CUDA(a->Alloc(&a->ctrl, 1));
  AMR_CUDA(a->Alloc(&a->tune_dt, 1));
  AMR_CUDA(cudaMallocHost(&a->ctrl_host, sizeof(AmrControl)));
  std::memset(a->ctrl_host, 0, sizeof(AmrControl));
  // sweep list in execution order (fine-first recursion, 4 sweeps per advance)
  std::vector<SweepInfo> sw;
  struct Rec {
    static void Go(int l, int nl, std::vector<SweepInfo>& sw) {
      if (l + 1 < nl)
        for (int r = 0; r < 2; ++r) Go(l + 1, nl, sw);
      for (int k = 0; k < 4; ++k) sw.push_back({l, 0.5 / double(1 << l)});
    }
  };
  Rec::Go(0, nl, sw);
  if (int(sw.size()) > kMaxSweeps) return Fail(FVS_ERR_INVALID, "too many levels");
  a->nsweeps = int(sw.size());
  AMR_CUDA(a->Upload(&a->sweeps, sw));
  return FVS_OK;
}

cudaError_t LaunchSweep(fvs_amr* a, int l, int d, const double* in, double* out,
                        double scale, const double* dt_ptr, unsigned long long* smax, int block,
                        int grid, int occ, int split) {
  const LevelHost& Lv = a->L[size_t(l)];
  PatchSweepArgs s{};
  s.in = in;
  s.out = out;
  s.ncells = int32_t(Lv.ncells);
  // halo cells injected from the coarser level's state at the start of the
  // coarse step (finer levels advance first, so its A buffer still holds it)
  if (l > 0) {
    s.coarse = a->L[size_t(l - 1)].A;
    s.coarse_ncells = int32_t(a->L[size_t(l - 1)].ncells);
  }
  if (split == kSplits) {  // x rows with the lanes of a warp along x
    s.segs = Lv.segs[d][0];
    s.nsegs = Lv.nsegs[d][0];
    s.slot_row = Lv.slot_row;
    s.row_slot0 = Lv.row_slot0;
    s.nslots = Lv.nslots;
    occ += 10;
  } else {
    s.segs = Lv.segs[d][split];
    s.nsegs = Lv.nsegs[d][split];
  }
  s.caps = Lv.caps[d];
  s.reg = a->reg;
  s.gamma = a->m.gamma;
  s.dx = Lv.dx;
  s.limiter = a->m.limiter;
  s.dt_ptr = dt_ptr;
  s.dt_scale = scale;
  s.smax_out = smax;
  s.ctrl = a->ctrl;
  switch (a->m.precision) {
  case FVS_FP64_EXACT:
    return LaunchPatchSweepExact(d, s, grid, block, a->stream);
  case FVS_FP64_FAST:
    return LaunchPatchSweepFast(d, s, grid, block, a->stream);
  default:
    return LaunchPatchSweepMixed(d, s, grid, block, occ, a->stream);
  }
}

cudaError_t LaunchMaxSpeed(fvs_amr* a, int l, int d) {
  const LevelHost& Lv = a->L[size_t(l)];
  MaxSpeedArgs s{};
  s.in = Lv.A;
  s.ncells = int32_t(Lv.ncells);
  if (l > 0) {
    s.coarse = a->L[size_t(l - 1)].A;
    s.coarse_ncells = int32_t(a->L[size_t(l - 1)].ncells);
  }
  s.segs = Lv.segs[d][kSplits - 1];  // rows in 8 segments
  s.nsegs = Lv.nsegs[d][kSplits - 1];
  s.gamma = a->m.gamma;
  s.smax_out = &a->ctrl->smax_stable[l][d];
  const int block = 128;
  const int grid = static_cast<int>(std::max<int64_t>(
      1, std::min<int64_t>((int64_t(s.nsegs) + block - 1) / block, int64_t(a->sms) * 16)));
  switch (a->m.precision) {
  case FVS_FP64_EXACT:
    return LaunchPatchMaxSpeedExact(d, s, grid, block, a->stream);
  case FVS_FP64_FAST:
    return LaunchPatchMaxSpeedFast(d, s, grid, block, a->stream);
  default:
    return LaunchPatchMaxSpeedMixed(d, s, grid, block, a->stream);
  }
}

LevelDx Dx(const fvs_amr* a) {
  LevelDx dx{};
  for (int l = 0; l < a->nlevels; ++l) dx.dx[l] = a->L[size_t(l)].dx;
  return dx;
}

cudaError_t AdvanceLevel(fvs_amr* a, int l, int parity, int sub, int& counter) {
  cudaError_t e;
  const int nl = a->nlevels;
  if (l + 1 < nl) {
    const LevelHost& F = a->L[size_t(l + 1)];
    const size_t n = size_t(F.slot_end - F.slot_begin) * 3 * kComp;
    if (n) {
      e = cudaMemsetAsync(a->reg + size_t(F.slot_begin) * 3 * kComp, 0, n * sizeof(double),
                          a->stream);
      if (e != cudaSuccess) return e;
    }
    for (int r = 0; r < 2; ++r)
      if ((e = AdvanceLevel(a, l + 1, parity, r, counter)) != cudaSuccess) return e;
  }
  LevelHost& Lv = a->L[size_t(l)];
  // MakeSplitDirections(cycle, subcycle) and StrangSplitting (x, y, y, x)
  const int is_odd = (parity + sub) % 2;
  const int d0 = is_odd ? 1 : 0;
  const int seq[4] = {d0, 1 - d0, 1 - d0, d0};
  double* bufs[2] = {Lv.A, Lv.B};
  int cur = 0;
  for (int k = 0; k < 4; ++k) {
    const int d = seq[k];
    if ((e = LaunchSweep(a, l, d, bufs[cur], bufs[1 - cur], 0.5 / double(1 << l), &a->ctrl->dt,
                         &a->ctrl->smax_sweep[counter++], Lv.block[d], Lv.grid[d], Lv.occ[d],
                         Lv.split[d])) !=
        cudaSuccess)
      return e;
    cur ^= 1;
  }
  if (l + 1 < nl) {
    const LevelHost& F = a->L[size_t(l + 1)];
    if ((e = LaunchReflux(Lv.A, int32_t(Lv.ncells), a->reg, F.reflux, F.nreflux, a->signs,
                          Lv.dx, a->stream)) != cudaSuccess)
      return e;
    if ((e = LaunchAverageDown(Lv.A, int32_t(Lv.ncells), F.A, int32_t(F.ncells), F.avg, F.navg,
                               a->stream)) != cudaSuccess)
      return e;
  }
  return cudaSuccess;
}

cudaError_t EnqueueStep(fvs_amr* a, int parity) {
  cudaError_t e;
  for (int l = 0; l < a->nlevels; ++l) {
    const LevelHost& Lv = a->L[size_t(l)];
    e = cudaMemcpyAsync(Lv.backup, Lv.A, size_t(Lv.ncells) * kComp * sizeof(double),
                        cudaMemcpyDeviceToDevice, a->stream);
    if (e != cudaSuccess) return e;
  }
  e = cudaMemsetAsync(&a->ctrl->smax_stable[0][0], 0,
                      sizeof(a->ctrl->smax_stable) + sizeof(a->ctrl->smax_sweep), a->stream);
  if (e != cudaSuccess) return e;
  for (int l = 0; l < a->nlevels; ++l)
    for (int d = 0; d < 2; ++d)
      if ((e = LaunchMaxSpeed(a, l, d)) != cudaSuccess) return e;
  if ((e = LaunchAmrDt(a->ctrl, a->nlevels, Dx(a), a->stream)) != cudaSuccess) return e;
  int counter = 0;
  if ((e = AdvanceLevel(a, 0, parity, 0, counter)) != cudaSuccess) return e;
  return LaunchAmrEndStep(a->ctrl, a->sweeps, a->nsweeps, Dx(a), a->stream);
}

void DropGraphs(fvs_amr* a) {
  for (auto& g : a->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

int EnsureGraph(fvs_amr* a, int parity) {
  if (a->graph[parity]) return FVS_OK;
  cudaGraph_t g;
  AMR_CUDA(cudaStreamBeginCapture(a->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = EnqueueStep(a, parity);
  cudaError_t e2 = cudaStreamEndCapture(a->stream, &g);
  if (e != cudaSuccess) return CudaFail(e, "capture AMR step");
  if (e2 != cudaSuccess) return CudaFail(e2, "end capture");
  e = cudaGraphInstantiate(&a->graph[parity], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return CudaFail(e, "instantiate AMR graph");
  return FVS_OK;
}

}  // namespace

extern "C" {

int fvs_amr_create(const fvs_amr_desc* d, const fvs_method* m, fvs_amr** out) {
  if (!d || !out || !d->patch_level || !d->patch_box) return Fail(FVS_ERR_INVALID, "NULL argument");
  *out = nullptr;
  if (d->rank != 2) return Fail(FVS_ERR_UNSUPPORTED, "AMR patch sets are rank 2");
  if (d->nlevels < 1 || d->nlevels > kMaxLevels)
    return Fail(FVS_ERR_INVALID, "1 to 4 levels");
  if (d->n0[0] < 1 || d->n0[1] < 1 || !(d->dx0 > 0.0) || d->npatches < 1)
    return Fail(FVS_ERR_INVALID, "bad level-0 size, dx or patch count");
  for (int k = 0; k < 2; ++k) {
    if (d->bc[k] != FVS_BC_PERIODIC && d->bc[k] != FVS_BC_TRANSMISSIVE &&
        d->bc[k] != FVS_BC_REFLECTIVE)
      return Fail(FVS_ERR_INVALID, "bad boundary condition");
    if (d->bc[k] == FVS_BC_REFLECTIVE && d->n0[k] < 2)
      return Fail(FVS_ERR_INVALID, "a reflective direction needs at least 2 cells");
  }
  fvs_method mm;
  if (m) {
    mm = *m;
  } else {
    fvs_method_default(&mm);
  }
  if (mm.flux_method != FVS_MUSCL_HLLE)
    return Fail(FVS_ERR_UNSUPPORTED, "AMR patch sets run MUSCL-Hancock + HLLE");
  if (mm.precision < FVS_FP64_EXACT || mm.precision > FVS_MIXED)
    return Fail(FVS_ERR_UNSUPPORTED, "AMR patch sets run in exact FP64, fast FP64 or mixed");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return Fail(FVS_ERR_NO_DEVICE, "no CUDA device available");
  }
  fvs_amr* a = new fvs_amr();
  a->nlevels = d->nlevels;
  a->n0[0] = d->n0[0];
  a->n0[1] = d->n0[1];
  a->bc[0] = d->bc[0];
  a->bc[1] = d->bc[1];
  a->dx0 = d->dx0;
  a->m = mm;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&a->sms, cudaDevAttrMultiProcessorCount, dev);
  a->patches.resize(size_t(d->npatches));
  for (int p = 0; p < d->npatches; ++p) {
    PatchHost& P = a->patches[size_t(p)];
    P.level = d->patch_level[p];
    const fvs_box& b = d->patch_box[p];
    bool ok = P.level >= 0 && P.level < d->nlevels;
    for (int k = 0; k < 2 && ok; ++k) {
      P.lo[k] = b.lo[k];
      P.hi[k] = b.hi[k];
      P.n[k] = b.hi[k] - b.lo[k];
      const int n = d->n0[k] << P.level;
      ok = P.n[k] >= 1 && P.lo[k] >= 0 && P.hi[k] <= n &&
           (P.level == 0 || (P.lo[k] % 2 == 0 && P.hi[k] % 2 == 0));
    }
    if (!ok) {
      delete a;
      return Fail(FVS_ERR_INVALID, "patch " + std::to_string(p) +
                                       " has a bad level or box (fine boxes need even corners)");
    }
  }
  cudaError_t e = cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete a;
    return CudaFail(e, "cudaStreamCreate");
  }
  if (int r = Build(a)) {
    delete a;
    return r;
  }
  *out = a;
  return FVS_OK;
}

int fvs_amr_destroy(fvs_amr* a) {
  delete a;
  return FVS_OK;
}

int fvs_amr_upload(fvs_amr* a, const double* host) {
  if (!a || !host) return Fail(FVS_ERR_INVALID, "NULL argument");
  std::vector<std::vector<double>> lv(static_cast<size_t>(a->nlevels));
  for (int l = 0; l < a->nlevels; ++l)
    lv[size_t(l)].assign(size_t(a->L[size_t(l)].ncells) * kComp, 0.0);
  size_t off = 0;
  for (size_t p = 0; p < a->patches.size(); ++p) {
    const PatchHost& P = a->patches[p];
    const int64_t N = a->L[size_t(P.level)].ncells;
    std::vector<double>& v = lv[size_t(P.level)];
    for (int c = 0; c < kComp; ++c)
      for (int j = 0; j < P.n[1]; ++j)
        for (int i = 0; i < P.n[0]; ++i)
          v[size_t(c * N + a->SI(int(p), P.lo[0] + i, P.lo[1] + j))] = host[off++];
  }
  for (int l = 0; l < a->nlevels; ++l)
    AMR_CUDA(cudaMemcpy(a->L[size_t(l)].A, lv[size_t(l)].data(),
                        lv[size_t(l)].size() * sizeof(double), cudaMemcpyHostToDevice));
  a->t = 0.0;
  a->cycle = 0;
  return FVS_OK;
}

int fvs_amr_download(fvs_amr* a, double* host) {
  if (!a || !host) return Fail(FVS_ERR_INVALID, "NULL argument");
  AMR_CUDA(cudaStreamSynchronize(a->stream));
  std::vector<std::vector<double>> lv(static_cast<size_t>(a->nlevels));
  for (int l = 0; l < a->nlevels; ++l) {
    lv[size_t(l)].resize(size_t(a->L[size_t(l)].ncells) * kComp);
    AMR_CUDA(cudaMemcpy(lv[size_t(l)].data(), a->L[size_t(l)].A,
                        lv[size_t(l)].size() * sizeof(double), cudaMemcpyDeviceToHost));
  }
  size_t off = 0;
  for (size_t p = 0; p < a->patches.size(); ++p) {
    const PatchHost& P = a->patches[p];
    const int64_t N = a->L[size_t(P.level)].ncells;
    const std::vector<double>& v = lv[size_t(P.level)];
    for (int c = 0; c < kComp; ++c)
      for (int j = 0; j < P.n[1]; ++j)
        for (int i = 0; i < P.n[0]; ++i)
          host[off++] = v[size_t(c * N + a->SI(int(p), P.lo[0] + i, P.lo[1] + j))];
  }
  return FVS_OK;
}

int fvs_amr_write_plotfile(fvs_amr* a, const char* dir) {
  if (!a || !dir || !*dir) return Fail(FVS_ERR_INVALID, "NULL argument");
  fvs::plot::Plotfile pf;
  pf.dir = dir;
  pf.dim = 2;
  pf.time = a->t;
  pf.vars = fvs::plot::CompleteNames(2);
  for (int d = 0; d < 2; ++d) pf.prob_hi[d] = a->n0[d] * a->dx0;
  std::vector<std::vector<int>> members(static_cast<size_t>(a->nlevels));
  for (size_t p = 0; p < a->patches.size(); ++p)
    members[size_t(a->patches[p].level)].push_back(int(p));
  for (int l = 0; l < a->nlevels; ++l) {
    const LevelHost& LH = a->L[size_t(l)];
    fvs::plot::Level L{};
    for (int d = 0; d < 3; ++d) {
      L.domain.lo[d] = 0;
      L.domain.hi[d] = d < 2 ? LH.n[d] - 1 : 0;
      L.dx[d] = d < 2 ? LH.dx : 1.0;
    }
    L.step = static_cast<int>(a->cycle << l);
    L.ratio_to_next = 2;
    for (int p : members[size_t(l)]) {
      const PatchHost& P = a->patches[size_t(p)];
      fvs::plot::Box b{};
      for (int d = 0; d < 2; ++d) {
        b.lo[d] = P.lo[d];
        b.hi[d] = P.lo[d] + P.n[d] - 1;
      }
      L.boxes.push_back(b);
    }
    pf.levels.push_back(L);
  }
  if (std::string e = fvs::plot::WriteHeader(pf); !e.empty()) return Fail(FVS_ERR_IO, e);
  constexpr int kOut = 6;  // Complete components in 2-D
  for (int l = 0; l < a->nlevels; ++l) {
    const LevelHost& LH = a->L[size_t(l)];
    const int64_t N = LH.ncells;
    double* dq = nullptr;
    AMR_CUDA(cudaMallocAsync(&dq, size_t(N) * kOut * sizeof(double), a->stream));
    // Complete state of every storage cell of the level (the level arrays are
    // component-major over N cells, read here as an N x 1 x 1 box)
    fvs::BoxDesc box{{0, 0, 0}, {static_cast<int>(N), 1, 1}};
    cudaError_t ce =
        fvs::LaunchPatchCompleteFromCons(2, a->m.gamma, dq, box, LH.A, box, box, a->stream);
    std::vector<double> q(size_t(N) * kOut);
    if (ce == cudaSuccess)
      ce = cudaMemcpyAsync(q.data(), dq, q.size() * sizeof(double), cudaMemcpyDeviceToHost,
                           a->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(a->stream);
    cudaFreeAsync(dq, a->stream);
    if (ce != cudaSuccess) return Fail(FVS_ERR_CUDA, cudaGetErrorString(ce));
    fvs::plot::LevelWriter w(pf, l);
    std::vector<double> fab;
    int bi = 0;
    for (int p : members[size_t(l)]) {
      const PatchHost& P = a->patches[size_t(p)];
      const int64_t n = int64_t(P.n[0]) * P.n[1];
      fab.resize(size_t(n) * kOut);
      size_t off = 0;
      for (int c = 0; c < kOut; ++c)
        for (int j = 0; j < P.n[1]; ++j)
          for (int i = 0; i < P.n[0]; ++i)
            fab[off++] = q[size_t(c * N + a->SI(p, P.lo[0] + i, P.lo[1] + j))];
      if (std::string e = w.Append(bi++, fab.data()); !e.empty()) return Fail(FVS_ERR_IO, e);
    }
    if (std::string e = w.Finish(); !e.empty()) return Fail(FVS_ERR_IO, e);
  }
  return FVS_OK;
}

int fvs_amr_info(fvs_amr* a, int64_t* cells_per_level, int64_t* storage_per_level,
                 int32_t* nslots) {
  if (!a) return Fail(FVS_ERR_INVALID, "NULL argument");
  for (int l = 0; l < a->nlevels; ++l) {
    int64_t c = 0;
    for (int p : a->L[size_t(l)].patches)
      c += int64_t(a->patches[size_t(p)].n[0]) * a->patches[size_t(p)].n[1];
    if (cells_per_level) cells_per_level[l] = c;
    if (storage_per_level) storage_per_level[l] = a->L[size_t(l)].ncells;
  }
  if (nslots) *nslots = a->nslots;
  return FVS_OK;
}

int fvs_amr_stream(fvs_amr* a, void** stream) {
  if (!a || !stream) return Fail(FVS_ERR_INVALID, "NULL argument");
  *stream = a->stream;
  return FVS_OK;
}

int fvs_amr_stable_dt(fvs_amr* a, double* dt) {
  if (!a || !dt) return Fail(FVS_ERR_INVALID, "NULL argument");
  AMR_CUDA(cudaMemsetAsync(&a->ctrl->smax_stable[0][0], 0, sizeof(a->ctrl->smax_stable),
                           a->stream));
  for (int l = 0; l < a->nlevels; ++l)
    for (int d = 0; d < 2; ++d) AMR_CUDA(LaunchMaxSpeed(a, l, d));
  unsigned long long bits[kMaxLevels][2];
  AMR_CUDA(cudaMemcpyAsync(bits, a->ctrl->smax_stable, sizeof bits, cudaMemcpyDeviceToHost,
                           a->stream));
  AMR_CUDA(cudaStreamSynchronize(a->stream));
  double stable = 1.7976931348623157e308;
  for (int l = 0; l < a->nlevels; ++l)
    for (int d = 0; d < 2; ++d) {
      double s;
      std::memcpy(&s, &bits[l][d], sizeof s);
      const double v = double(1 << l) * (a->L[size_t(l)].dx / s);
      stable = v < stable ? v : stable;
    }
  *dt = stable;
  return FVS_OK;
}

int fvs_amr_run(fvs_amr* a, double cfl, double t_end, int max_steps, double* dt_log,
                int log_len, fvs_run_stats* stats) {
  if (!a) return Fail(FVS_ERR_INVALID, "NULL argument");
  if (!(cfl > 0.0)) return Fail(FVS_ERR_INVALID, "cfl must be positive");
  for (int p = 0; p < 2; ++p)
    if (int r = EnsureGraph(a, p)) return r;
  AmrControl& h = *a->ctrl_host;
  std::memset(&h, 0, sizeof h);
  h.t = a->t;
  h.t_end = t_end;
  h.cfl = cfl;
  AMR_CUDA(cudaMemcpyAsync(a->ctrl, &h, sizeof h, cudaMemcpyHostToDevice, a->stream));
  const double eps = 1e-12;
  int steps = 0, restarts = 0, retries = 0;
  double last_dt = 0.0;
  while (a->t + eps < t_end && (max_steps < 0 || steps < max_steps)) {
    AMR_CUDA(cudaGraphLaunch(a->graph[a->cycle % 2], a->stream));
    AMR_CUDA(cudaMemcpyAsync(&h, a->ctrl, sizeof h, cudaMemcpyDeviceToHost, a->stream));
    AMR_CUDA(cudaStreamSynchronize(a->stream));
    if (h.failed) {
      for (int l = 0; l < a->nlevels; ++l) {
        const LevelHost& Lv = a->L[size_t(l)];
        AMR_CUDA(cudaMemcpyAsync(Lv.A, Lv.backup, size_t(Lv.ncells) * kComp * sizeof(double),
                                 cudaMemcpyDeviceToDevice, a->stream));
      }
      ++restarts;
      if (++retries > 64) return Fail(FVS_ERR_DT_TOO_LARGE, "AMR step keeps failing its checks");
      continue;
    }
    retries = 0;
    last_dt = h.dt;
    if (dt_log && steps < log_len) dt_log[steps] = h.dt;
    a->t = h.t;
    ++steps;
    ++a->cycle;
  }
  if (stats) {
    stats->time = a->t;
    stats->steps = steps;
    stats->restarts = restarts;
    stats->status = h.status;
    stats->last_dt = last_dt;
  }
  return FVS_OK;
}

int fvs_amr_set_launch(fvs_amr* a, int level, int dir, int block, int grid,
                       int threads_per_row) {
  if (!a || level < 0 || level >= a->nlevels || dir < 0 || dir > 1)
    return Fail(FVS_ERR_INVALID, "bad level or direction");
  if (block != 32 && block != 64 && block != 128)
    return Fail(FVS_ERR_INVALID, "block must be 32, 64 or 128");
  if (grid < 1) return Fail(FVS_ERR_INVALID, "grid must be positive");
  int si = -1;
  for (int k = 0; k < kSplits; ++k)
    if (kSplitOf[k] == threads_per_row) si = k;
  if (threads_per_row == 32 && dir == 0 && a->m.precision == FVS_MIXED) si = kSplits;
  if (si < 0)
    return Fail(FVS_ERR_INVALID,
                "threads per row must be 1, 2, 4 or 8 (or 32: x rows with lanes along x, mixed)");
  a->L[size_t(level)].block[dir] = block;
  a->L[size_t(level)].grid[dir] = grid;
  a->L[size_t(level)].split[dir] = si;
  DropGraphs(a);
  return FVS_OK;
}

int fvs_amr_autotune(fvs_amr* a, int32_t* configs) {
  if (!a) return Fail(FVS_ERR_INVALID, "NULL argument");
  const double dt_small = 1e-9;
  AMR_CUDA(cudaMemcpy(a->tune_dt, &dt_small, sizeof dt_small, cudaMemcpyHostToDevice));
  cudaEvent_t e0, e1;
  AMR_CUDA(cudaEventCreate(&e0));
  AMR_CUDA(cudaEventCreate(&e1));
  for (int l = 0; l < a->nlevels; ++l) {
    LevelHost& Lv = a->L[size_t(l)];
    for (int d = 0; d < 2; ++d) {
      const std::string key = std::to_string(a->m.precision) + "/" + std::to_string(d) + "/" +
                              Lv.hist;
      {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end()) {
          Lv.block[d] = it->second.block;
          Lv.grid[d] = it->second.grid;
          Lv.occ[d] = it->second.occ;
          Lv.split[d] = it->second.split;
          continue;
        }
      }
      float best = 1e30f;
      Tuned bt{128, Lv.grid[d], 0, 0};
      const bool mixed = a->m.precision == FVS_MIXED;
      // splits of the marching kernel, and (mixed x sweeps) the kernel with
      // the lanes of a warp along x
      for (int si = 0; si <= kSplits; ++si) {
        if (si == kSplits && !(mixed && d == 0)) continue;
        if (si > 0 && si < kSplits && Lv.nsegs[d][si] == Lv.nsegs[d][si - 1])
          continue;  // rows too short
        const int64_t threads =
            si == kSplits
                ? 32 * std::max<int64_t>(1, (Lv.nslots - 1 + kRowWarpStep - 1) / kRowWarpStep)
                : int64_t(Lv.nsegs[d][si]);
        for (int occ : {0, 5}) {
          if (occ && !mixed) continue;
          for (int block : {64, 128}) {
            const int full = int(std::max<int64_t>(1, (threads + block - 1) / block));
            for (int bps : {1, 2, 4, 8, 16, 64}) {
              const int grid = std::min(full, a->sms * bps);
              float sum = 0.f;
              for (int rep = 0; rep < 3; ++rep) {
                // the sweep's max slot starts at zero, as in a step
                AMR_CUDA(cudaMemsetAsync(&a->ctrl->smax_sweep[0], 0, sizeof(unsigned long long),
                                         a->stream));
                AMR_CUDA(cudaEventRecord(e0, a->stream));
                AMR_CUDA(LaunchSweep(a, l, d, Lv.A, Lv.B, 0.5, a->tune_dt,
                                     &a->ctrl->smax_sweep[0], block, grid, occ, si));
                AMR_CUDA(cudaEventRecord(e1, a->stream));
                AMR_CUDA(cudaEventSynchronize(e1));
                float ms = 0.f;
                AMR_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                if (rep > 0) sum += ms;
              }
              if (sum < best) {
                best = sum;
                bt = {block, grid, occ, si};
              }
              if (grid == full) break;
            }
          }
        }
      }
      Lv.block[d] = bt.block;
      Lv.grid[d] = bt.grid;
      Lv.occ[d] = bt.occ;
      Lv.split[d] = bt.split;
      std::lock_guard<std::mutex> lock(g_tune_mutex);
      g_tuned[key] = bt;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (configs)
    for (int l = 0; l < a->nlevels; ++l)
      for (int d = 0; d < 2; ++d) {
        configs[(l * 2 + d) * 3] = a->L[size_t(l)].block[d];
        configs[(l * 2 + d) * 3 + 1] = a->L[size_t(l)].grid[d];
        configs[(l * 2 + d) * 3 + 2] =
            a->L[size_t(l)].split[d] == kSplits ? 32 : kSplitOf[a->L[size_t(l)].split[d]];
      }
  DropGraphs(a);
  return FVS_OK;
}

}  // extern "C"
