// fvs_capi.cu -- the C ABI of libfvs_gb300 (include/fvs_gpu.h): argument
// checking, the patch-level entry points, and the uniform-grid solver
// context with its device-resident time stepping and CUDA graphs.
#include "../../include/fvs_gpu.h"
#include "fvs_cutcell.h"
#include "fvs_internal.h"
#include "fvs_plotfile.h"
#include "fvs_tma.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

namespace {

thread_local std::string g_last_error;

int Fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int CudaFail(cudaError_t e, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return FVS_ERR_CUDA;
}

#define FVS_CUDA(call)                                  \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return CudaFail(e_, #call);  \
  } while (0)

fvs::BoxDesc ToDesc(const fvs_box& b) {
  fvs::BoxDesc d;
  for (int i = 0; i < 3; ++i) {
    d.lo[i] = b.lo[i];
    d.n[i] = b.hi[i] - b.lo[i];
  }
  return d;
}

bool ValidBox(const fvs_box& b) {
  for (int i = 0; i < 3; ++i)
    if (b.hi[i] < b.lo[i]) return false;
  return true;
}

bool Contains(const fvs_box& outer, const int* lo, const int* hi) {
  for (int i = 0; i < 3; ++i)
    if (lo[i] < outer.lo[i] || hi[i] > outer.hi[i]) return false;
  return true;
}

int64_t Volume(const fvs_box& b) {
  return int64_t(b.hi[0] - b.lo[0]) * (b.hi[1] - b.lo[1]) * (b.hi[2] - b.lo[2]);
}

bool IsGodunov(int method) { return method == FVS_GODUNOV || method == FVS_MUSCL_GODUNOV; }

int StencilWidth(int method) {
  return (method == FVS_HLLE || method == FVS_GODUNOV || method == FVS_HLLEM) ? 1 : 2;
}

// Methods whose face flux is Hllem: none, conservative, characteristic or
// primitive reconstruction in front of it (-1 for the others).
int HllemRecon(int method) {
  switch (method) {
  case FVS_HLLEM:
    return 0;
  case FVS_MUSCL_HLLEM:
    return 1;
  case FVS_MUSCL_CHAR:
    return 2;
  case FVS_MUSCL_PRIM:
    return 3;
  default:
    return -1;
  }
}

double BitsToDouble(unsigned long long b) {
  double d;
  std::memcpy(&d, &b, sizeof d);
  return d;
}

}  // namespace

// ---------------------------------------------------------------------------
// Control kernels of the device-resident time loop.

namespace fvs {

void SetLastError(const std::string& msg) { g_last_error = msg; }

int CheckDevice() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return Fail(FVS_ERR_NO_DEVICE, "no CUDA device available");
  }
  return FVS_OK;
}

int CheckMethod(const fvs_method* m, int rank) {
  if (!m) return Fail(FVS_ERR_INVALID, "method is NULL");
  if (rank < 1 || rank > 3) return Fail(FVS_ERR_INVALID, "rank must be 1, 2 or 3");
  if (m->flux_method < 0 || m->flux_method > 7)
    return Fail(FVS_ERR_INVALID, "unknown flux method");
  if (m->limiter < 0 || m->limiter > 3) return Fail(FVS_ERR_INVALID, "unknown limiter");
  // the characteristic method limits with VanLeer's two-slope functor only,
  // the primitive one with its own fixed limiter
  if ((m->flux_method == FVS_MUSCL_CHAR || m->flux_method == FVS_MUSCL_PRIM) &&
      m->limiter != FVS_VAN_LEER)
    return Fail(FVS_ERR_UNSUPPORTED, "the characteristic and primitive reconstructions "
                                     "take no limiter choice (FVS_VAN_LEER)");
  if (m->precision < 0 || m->precision > 3)
    return Fail(FVS_ERR_INVALID, "unknown precision");
  if (!(m->gamma > 1.0)) return Fail(FVS_ERR_INVALID, "gamma must exceed 1");
  return FVS_OK;
}

__device__ __forceinline__ double BitsToDoubleDev(unsigned long long b) {
  return __longlong_as_double(static_cast<long long>(b));
}

struct StepPlan {
  int nsweeps;
  int dir[6];
  double dx[6];
  double frac;  // split dt = frac * dt
  int rank;
  double dxd[3];
  int skip0;    // sweep 0 takes its check's speed from the stable-dt pass
};

// RunSimulation's dt selection (include/fub/RunSimulation.hpp:125-131):
// dt = min(t_end - t, cfl * stable_dt), or the failed check's dt after a
// restart; stops when t + 1e-12 >= t_end.
__global__ void BeginStepKernel(Control* c, StepPlan plan) {
  if (c->abort || c->done) return;
  const double eps = 1e-12;
  if (!(c->t + eps < c->t_end)) {
    c->done = 1;
    return;
  }
  double stable;
  if (c->have_failure) {
    stable = c->fail_dt;
    c->have_failure = 0;
  } else {
    stable = 1.7976931348623157e308;
    for (int d = 0; d < plan.rank; ++d) {
      const double s = BitsToDoubleDev(c->smax_stable[d]);
      const double dtd = plan.dxd[d] / s;
      stable = dtd < stable ? dtd : stable;
    }
  }
  double dt;
  if (c->dt_override > 0.0) {
    dt = c->dt_override;
  } else {
    const double a = c->t_end - c->t;
    const double b = c->cfl * stable;
    dt = a < b ? a : b;
  }
  c->dt = dt;
  for (int q = 0; q < 6; ++q) c->smax_check[q] = 0ull;
  // the first sweep's input is the state the stable-dt pass just measured,
  // over the same faces: its check uses that pass's speed in its direction
  if (plan.skip0) c->smax_check[0] = c->smax_stable[plan.dir[0]];
  c->step_status = 0;
}

// The per-sweep checks (DimensionalSplitLevelIntegrator.hpp:240-245), in
// sweep order; commits the step or records the first failure.
__global__ void EndStepKernel(Control* c, StepPlan plan, int step_in_batch,
                              double* dt_log, int dt_log_len) {
  if (c->abort || c->done) return;
  const double split_dt = plan.frac * c->dt;
  for (int q = 0; q < plan.nsweeps; ++q) {
    const double level_dt = plan.dx[q] / BitsToDoubleDev(c->smax_check[q]);
    if (level_dt < split_dt) {
      c->abort = 1;
      c->failed_step = step_in_batch;
      c->fail_dt = level_dt;
      c->have_failure = 1;
      return;
    }
  }
  if (dt_log && c->steps_done < dt_log_len) dt_log[c->steps_done] = c->dt;  // cumulative index
  c->t = c->t + c->dt;
  c->steps_done += 1;
  c->status |= c->step_status;
  for (int d = 0; d < 3; ++d) c->smax_stable[d] = 0ull;
}

}  // namespace fvs

using fvs::CheckDevice;
using fvs::CheckMethod;

// ---------------------------------------------------------------------------

struct fvs_solver {
  fvs_grid_desc g;
  fvs_method m;
  cudaStream_t stream = nullptr;
  double* buf[3] = {nullptr, nullptr, nullptr};
  int cur = 0;
  fvs::Control* ctrl = nullptr;
  fvs::Control* ctrl_host = nullptr;  // pinned
  unsigned long long* scratch_words = nullptr;  // [8]
  unsigned long long* newton_words = nullptr;   // [3] host-driven sweeps
  double* dt_log_dev = nullptr;
  int dt_log_cap = 0;
  int seg_len = 0;
  int seg_tuned[3] = {0, 0, 0};  // autotuned cells per thread segment, per direction
  int occ_tuned[3] = {0, 0, 0};  // autotuned occupancy variant (mixed), per direction
  int64_t cycle = 0;
  double t = 0.0;
  int64_t cells = 0;
  int ncons = 0;
  std::map<std::tuple<int, int, int>, cudaGraphExec_t> graphs;
  // embedded boundary (KBN cut cells, rank 2)
  bool cc = false;
  fvs::CcGeom ccg{};
  double* cc_refs = nullptr;
  std::vector<void*> cc_allocs;
  // the cut tiles of a KBN sweep run on `side`, forked from and joined back
  // into `stream` by the two events
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // tensor maps of the three state buffers for the TMA-staged y and z
  // sweeps of the mixed flavour ([buffer][dir - 1]); built on first use
  CUtensorMap tmap[3][2];  // aligned as the type requires (new of an over-aligned type, C++17)
  int tmap_state = 0;  // 0 not tried, 1 built, -1 not available
  // host-resident steps (fvs_solver_step_host): the copies of the last
  // sweep's slabs run on `copy`, each after its slab's event
  cudaStream_t copy = nullptr, slab = nullptr;
  cudaEvent_t slab_ev[fvs::kHostSlabs + 1] = {};
  cudaEvent_t slab_fork = nullptr;
  ~fvs_solver() {
    for (cudaEvent_t e : slab_ev)
      if (e) cudaEventDestroy(e);
    if (slab_fork) cudaEventDestroy(slab_fork);
    if (copy) cudaStreamDestroy(copy);
    if (slab) cudaStreamDestroy(slab);
    for (void* p : cc_allocs) cudaFree(p);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (side) cudaStreamDestroy(side);
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    for (double* b : buf)
      if (b) cudaFree(b);
    if (ctrl) cudaFree(ctrl);
    if (ctrl_host) cudaFreeHost(ctrl_host);
    if (scratch_words) cudaFree(scratch_words);
    if (newton_words) cudaFree(newton_words);
    if (dt_log_dev) cudaFree(dt_log_dev);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

// The tensor maps of the TMA-staged sweep: each state buffer as
// [K][nz][ny][nx] (rank 3) or [K][ny][nx] (rank 2) FP64 with boxes of
// 32 x-cells by kTmaRows cells along y or z by all K components.  Available
// for the mixed flavour's MUSCL-HLLE / HLLE sweeps of grids of rank >= 2
// with an even nx (TMA's row pitch must be a multiple of 16 bytes).
bool TmaMapsReady(fvs_solver* s) {
  if (s->tmap_state != 0) return s->tmap_state > 0;
  s->tmap_state = -1;
  const int rank = s->g.rank;
  if (s->cc || s->m.precision != FVS_MIXED || s->m.flux_method > FVS_HLLE || rank < 2 ||
      (s->g.n[0] % 2) != 0)
    return false;
  const fvs::tma::EncodeTiledFn fn = fvs::tma::EncodeTiled();
  if (!fn) return false;
  const int K = rank + 2;
  const cuuint64_t nx = cuuint64_t(s->g.n[0]), ny = cuuint64_t(s->g.n[1]),
                   nz = cuuint64_t(rank == 3 ? s->g.n[2] : 1);
  for (int b = 0; b < 3; ++b) {
    for (int d = 1; d < rank; ++d) {
      CUresult r;
      const cuuint32_t estr[4] = {1u, 1u, 1u, 1u};
      if (rank == 3) {
        const cuuint64_t dims[4] = {nx, ny, nz, cuuint64_t(K)};
        const cuuint64_t strides[3] = {nx * 8, nx * ny * 8, nx * ny * nz * 8};
        const cuuint32_t box[4] = {32u, d == 1 ? cuuint32_t(fvs::kTmaRows) : 1u,
                                   d == 2 ? cuuint32_t(fvs::kTmaRows) : 1u, cuuint32_t(K)};
        r = fn(&s->tmap[b][d - 1], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, s->buf[b], dims,
               strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      } else {
        const cuuint64_t dims[3] = {nx, ny, cuuint64_t(K)};
        const cuuint64_t strides[2] = {nx * 8, nx * ny * 8};
        const cuuint32_t box[3] = {32u, cuuint32_t(fvs::kTmaRows), cuuint32_t(K)};
        r = fn(&s->tmap[b][d - 1], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, s->buf[b], dims,
               strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      }
      if (r != CUDA_SUCCESS) return false;
    }
  }
  s->tmap_state = 1;
  return true;
}

// The tensor map of `in` (one of the state buffers) for a sweep in `dir`.
const void* TmaMapOf(const fvs_solver* s, const double* in, int dir) {
  if (s->tmap_state <= 0 || dir < 1) return nullptr;
  for (int b = 0; b < 3; ++b)
    if (s->buf[b] == in) return &s->tmap[b][dir - 1];
  return nullptr;
}

int SegLen(const fvs_solver* s, int dir) {
  if (s->seg_len > 0) return s->seg_len;
  if (s->seg_tuned[dir] > 0) return s->seg_tuned[dir];
  const int nd = s->g.n[dir];
  int64_t ntrans = s->cells / nd;
  // Enough threads for several waves of resident blocks on 152 SMs
  // (~60K threads per wave at 150 registers per thread); never shorter than
  // 16 cells (the 2-cell halo of a segment is recomputed).
  const int64_t target = 262144;
  int seg = nd;
  while (seg > 16 && ntrans * ((nd + seg - 1) / seg) < target) seg = (seg + 1) / 2;
  return seg;
}

fvs::CcStateArgs MakeCcState(const fvs_solver* s, const double* in) {
  fvs::CcStateArgs a{};
  a.g = s->ccg;
  a.in = in;
  a.bc[0] = s->g.bc[0];
  a.bc[1] = s->g.bc[1];
  a.gamma = s->m.gamma;
  a.refs = s->cc_refs;
  return a;
}

cudaError_t CcReferenceStates(const fvs_solver* s, const double* in) {
  const fvs::CcStateArgs a = MakeCcState(s, in);
  return s->m.precision == FVS_FP64_EXACT
             ? fvs::LaunchCutCellReferenceStates(a, s->stream)
             : fvs::LaunchCutCellReferenceStatesT(s->m.precision, a, s->stream);
}

cudaError_t LaunchSweep(const fvs_solver* s, const double* in, double* out,
                        int dir, const double* dt_ptr, double dt_scale,
                        double dt_value, unsigned long long* smax_out,
                        fvs::Control* ctrl, int prev_check, double prev_dx,
                        bool skip_cfl = false, int64_t t_lo = 0, int64_t t_hi = 0,
                        cudaStream_t stream = nullptr) {
  if (s->cc) {
    fvs::CcSweepArgs c{};
    c.s = MakeCcState(s, in);
    c.out = out;
    c.dir = dir;
    c.limiter = s->m.limiter;
    c.seg_len = SegLen(s, dir);
    c.dx = s->g.dx[dir];
    c.dt_ptr = dt_ptr;
    c.dt_scale = dt_scale;
    c.dt_value = dt_value;
    c.smax_out = smax_out;
    c.ctrl = ctrl;
    c.prev_check = prev_check;
    c.prev_dx = prev_dx;
    c.occupancy = s->occ_tuned[dir];
    c.skip_cfl = skip_cfl ? 1 : 0;
    auto launch = [&](bool band, cudaStream_t st) {
      return s->m.precision == FVS_FP64_EXACT
                 ? fvs::LaunchCutCellSweep(c, band, st)
                 : fvs::LaunchCutCellSweepT(s->m.precision, c, band, st);
    };
    // the cut tiles on the side stream, concurrent with the regular and
    // covered tiles (disjoint output cells, one CFL maximum)
    cudaError_t e = cudaSuccess;
    const bool fork = s->ccg.nband[dir] > 0;
    if (fork) {
      e = cudaEventRecord(s->ev_fork, s->stream);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s->side, s->ev_fork, 0);
      if (e == cudaSuccess) e = launch(true, s->side);
      if (e == cudaSuccess) e = cudaEventRecord(s->ev_join, s->side);
    }
    if (e == cudaSuccess) e = launch(false, s->stream);
    if (fork && e == cudaSuccess) e = cudaStreamWaitEvent(s->stream, s->ev_join, 0);
    return e;
  }
  fvs::SweepArgs a{};
  a.in = in;
  a.out = out;
  for (int d = 0; d < 3; ++d) a.n[d] = s->g.n[d];
  a.rank = s->g.rank;
  a.dir = dir;
  a.bc = s->g.bc[dir];
  a.limiter = s->m.limiter;
  a.seg_len = SegLen(s, dir);
  a.occupancy = s->occ_tuned[dir];
  a.gamma = s->m.gamma;
  a.dx = s->g.dx[dir];
  a.dt_ptr = dt_ptr;
  a.dt_scale = dt_scale;
  a.dt_value = dt_value;
  a.smax_out = smax_out;
  a.ctrl = ctrl;
  a.prev_check = prev_check;
  a.prev_dx = prev_dx;
  a.guess = s->m.guess;
  a.max_iterations = s->m.max_iterations;
  a.tolerance = s->m.tolerance;
  a.mlp = s->m.mlp_params;
  a.stats_out = ctrl ? ctrl->newton : s->newton_words;
  a.skip_cfl = skip_cfl ? 1 : 0;
  a.tmap = a.occupancy >= 20 ? TmaMapOf(s, in, dir) : nullptr;
  a.t_lo = t_lo;
  a.t_hi = t_hi;
  cudaStream_t st = stream ? stream : s->stream;
  if (s->m.flux_method == FVS_GODUNOV || s->m.flux_method == FVS_MUSCL_GODUNOV)
    return fvs::LaunchSweepGodunov(a, s->m.flux_method == FVS_MUSCL_GODUNOV, st);
  if (HllemRecon(s->m.flux_method) >= 0)
    return fvs::LaunchSweepHllem(a, HllemRecon(s->m.flux_method), st);
  switch (s->m.precision) {
  case FVS_FP64_EXACT:
    return fvs::LaunchSweepExact(a, st);
  case FVS_FP64_FAST:
    return fvs::LaunchSweepFast(a, st);
  case FVS_FP64_DF:
    return fvs::LaunchSweepDf64(a, st);
  default:
    return fvs::LaunchSweepMixed(a, st);
  }
}

// k_hi > 0: the faces of planes [k_lo, k_hi) only (3-D HLLE methods without
// a reflective direction: StablePlanesOk).
cudaError_t LaunchStable(const fvs_solver* s, const double* in,
                         unsigned long long* smax_out, fvs::Control* ctrl, int k_lo = 0,
                         int k_hi = 0) {
  if (s->cc)
    return s->m.precision == FVS_FP64_EXACT
               ? fvs::LaunchCutCellStableDt(MakeCcState(s, in), smax_out, ctrl, s->stream)
               : fvs::LaunchCutCellStableDtT(s->m.precision, MakeCcState(s, in), smax_out, ctrl,
                                             s->stream);
  fvs::StableDtArgs a{};
  a.in = in;
  for (int d = 0; d < 3; ++d) {
    a.n[d] = s->g.n[d];
    a.bc[d] = s->g.bc[d];
  }
  a.rank = s->g.rank;
  a.rule = s->g.dt_rule;
  a.width = StencilWidth(s->m.flux_method);
  a.gamma = s->m.gamma;
  a.smax_out = smax_out;
  a.ctrl = ctrl;
  a.k_lo = k_lo;
  a.k_hi = k_hi;
  if (k_hi > 0 && (s->m.flux_method > FVS_HLLE || s->g.rank != 3)) return cudaErrorNotSupported;
  if (s->m.flux_method == FVS_GODUNOV || s->m.flux_method == FVS_MUSCL_GODUNOV)
    return fvs::LaunchStableDtGodunov(a, s->m.guess, s->m.max_iterations, s->m.tolerance,
                                      s->m.mlp_params, s->stream);
  if (HllemRecon(s->m.flux_method) >= 0) return fvs::LaunchStableDtHllem(a, s->stream);
  switch (s->m.precision) {
  case FVS_FP64_EXACT:
    return fvs::LaunchStableDtExact(a, s->stream);
  case FVS_FP64_FAST:
    return fvs::LaunchStableDtFast(a, s->stream);
  case FVS_FP64_DF:
    return fvs::LaunchStableDtDf64(a, s->stream);
  default:
    return fvs::LaunchStableDtMixed(a, s->stream);
  }
}

fvs::StepPlan MakePlan(const fvs_solver* s, int64_t cycle) {
  fvs::StepPlan p{};
  const int D = s->g.rank;
  // MakeSplitDirections (SplittingMethod.hpp:115-126)
  int dirs[3];
  const int odd = static_cast<int>(cycle % 2);
  for (int i = 0; i < D; ++i) dirs[i] = odd ? D - 1 - i : i;
  // StrangSplitting::Advance (StrangSplitting.cpp:25-69)
  if (D == 1) {
    p.nsweeps = 1;
    p.dir[0] = dirs[0];
    p.frac = 1.0;
  } else if (D == 2) {
    const int q[4] = {dirs[0], dirs[1], dirs[1], dirs[0]};
    p.nsweeps = 4;
    for (int i = 0; i < 4; ++i) p.dir[i] = q[i];
    p.frac = 0.5;
  } else {
    const int q[6] = {dirs[0], dirs[1], dirs[2], dirs[2], dirs[1], dirs[0]};
    p.nsweeps = 6;
    for (int i = 0; i < 6; ++i) p.dir[i] = q[i];
    p.frac = 0.5;
  }
  for (int i = 0; i < p.nsweeps; ++i) p.dx[i] = s->g.dx[p.dir[i]];
  p.rank = D;
  // HLL and HLLEM sweeps (and the KBN cut-cell sweeps, faces of beta > 0)
  // measure the same face speeds as the stable-dt pass when that pass takes
  // every face (dt rule 0); the exact Riemann solver's sweeps and the mixed
  // flavour keep their own
  p.skip0 = (s->g.dt_rule == 0 && !IsGodunov(s->m.flux_method) &&
             s->m.precision != FVS_MIXED)
                ? 1
                : 0;
  for (int d = 0; d < 3; ++d) p.dxd[d] = s->g.dx[d];
  return p;
}

int NextBuffer(int start, int nsweeps) { return (start + (nsweeps % 2 ? 1 : 2)) % 3; }

// The lines of the last sweep of a step split into fvs::kHostSlabs slabs
// along the slowest transverse direction, and the host copies of a slab's
// cells: per component one contiguous run or one 2-D copy (pitch, width,
// rows) in doubles.
struct SlabCopy {
  int64_t t_lo, t_hi;      // the sweep's lines
  int64_t offset;          // first cell of the slab within a component
  int64_t width, pitch, rows;  // rows of `width` cells, `pitch` apart
};

int HostSlabs(const fvs_solver* s, int dir, SlabCopy* out) {
  const int64_t nx = s->g.n[0], ny = s->g.n[1], nz = s->g.n[2];
  // the line index t of a sweep in `dir` and its slowest transverse extent
  int64_t outer, inner;  // t = a + inner * b, b in [0, outer)
  if (dir == 0) {
    inner = ny;
    outer = nz;
  } else if (dir == 1) {
    inner = nx;
    outer = nz;
  } else {
    inner = nx;
    outer = ny;
  }
  if (s->g.rank == 2 && dir == 0) {  // rows j: slabs of rows
    inner = 1;
    outer = ny;
  }
  if (s->g.rank == 2 && dir == 1) {  // columns i: slabs of columns
    inner = 1;
    outer = nx;
  }
  const int n = static_cast<int>(std::min<int64_t>(fvs::kHostSlabs, std::max<int64_t>(1, outer)));
  if (s->g.rank == 1) {
    out[0] = {0, 1, 0, nx, nx, 1};
    return 1;
  }
  for (int k = 0; k < n; ++k) {
    const int64_t b0 = outer * k / n, b1 = outer * (k + 1) / n;
    SlabCopy& c = out[k];
    c.t_lo = b0 * inner;
    c.t_hi = b1 * inner;
    if (s->g.rank == 3 && dir <= 1) {  // z-planes [b0, b1): contiguous
      c.offset = b0 * nx * ny;
      c.width = (b1 - b0) * nx * ny;
      c.pitch = c.width;
      c.rows = 1;
    } else if (s->g.rank == 3) {  // y-rows [b0, b1) of every z-plane
      c.offset = b0 * nx;
      c.width = (b1 - b0) * nx;
      c.pitch = nx * ny;
      c.rows = nz;
    } else if (dir == 0) {  // 2-D rows [b0, b1): contiguous
      c.offset = b0 * nx;
      c.width = (b1 - b0) * nx;
      c.pitch = c.width;
      c.rows = 1;
    } else {  // 2-D columns [b0, b1) of every row
      c.offset = b0;
      c.width = b1 - b0;
      c.pitch = nx;
      c.rows = ny;
    }
  }
  return n;
}

// Enqueue one device-driven split step starting in buffer `start`.  With
// `host_out`, the step's last sweep runs slab by slab and each slab's cells
// are copied to host_out on the copy stream as soon as the slab is done
// (the stream joins back into the solver's stream at the end).
cudaError_t EnqueueStep(fvs_solver* s, int start, int64_t cycle, int step_in_batch,
                        double* host_out = nullptr, bool stable_enqueued = false) {
  const fvs::StepPlan plan = MakePlan(s, cycle);
  cudaError_t e = cudaSuccess;
  if (s->cc) {
    // KbnCutCellMethod::PreAdvanceHierarchy: reference states of the step
    e = CcReferenceStates(s, s->buf[start]);
    if (e != cudaSuccess) return e;
  }
  if (!stable_enqueued) {
    // the pass's max slots start at zero (its screened speeds need it)
    e = cudaMemsetAsync(s->ctrl->smax_stable, 0, sizeof(s->ctrl->smax_stable), s->stream);
    if (e != cudaSuccess) return e;
    e = LaunchStable(s, s->buf[start], s->ctrl->smax_stable, s->ctrl);
    if (e != cudaSuccess) return e;
  }
  fvs::BeginStepKernel<<<1, 1, 0, s->stream>>>(s->ctrl, plan);
  const int X = (start + 1) % 3, Y = (start + 2) % 3;
  int src = start, dst = X;
  for (int q = 0; q < plan.nsweeps; ++q) {
    const bool skip = q == 0 && plan.skip0;
    if (host_out && q == plan.nsweeps - 1) {
      // the slabs alternate between the solver's stream and `slab` (forked
      // here, joined below) so that one slab's tail overlaps the next slab
      SlabCopy slabs[fvs::kHostSlabs];
      const int n = HostSlabs(s, plan.dir[q], slabs);
      const size_t cs = size_t(s->cells);
      e = cudaEventRecord(s->slab_fork, s->stream);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s->slab, s->slab_fork, 0);
      for (int k = 0; k < n && e == cudaSuccess; ++k) {
        cudaStream_t st = (k % 2) ? s->slab : s->stream;
        e = LaunchSweep(s, s->buf[src], s->buf[dst], plan.dir[q], &s->ctrl->dt, plan.frac, 0.0,
                        skip ? nullptr : &s->ctrl->smax_check[q], s->ctrl,
                        q > 0 ? q - 1 : -1, q > 0 ? plan.dx[q - 1] : 0.0, skip, slabs[k].t_lo,
                        slabs[k].t_hi, st);
        if (e == cudaSuccess) e = cudaEventRecord(s->slab_ev[k], st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s->copy, s->slab_ev[k], 0);
        for (int c = 0; c < s->ncons && e == cudaSuccess; ++c) {
          const SlabCopy& sc = slabs[k];
          double* dsth = host_out + c * cs + sc.offset;
          const double* srcd = s->buf[dst] + c * cs + sc.offset;
          e = sc.rows == 1
                  ? cudaMemcpyAsync(dsth, srcd, size_t(sc.width) * 8, cudaMemcpyDeviceToHost,
                                    s->copy)
                  : cudaMemcpy2DAsync(dsth, size_t(sc.pitch) * 8, srcd, size_t(sc.pitch) * 8,
                                      size_t(sc.width) * 8, size_t(sc.rows),
                                      cudaMemcpyDeviceToHost, s->copy);
        }
      }
      if (e == cudaSuccess) e = cudaEventRecord(s->slab_fork, s->slab);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s->stream, s->slab_fork, 0);
      if (e == cudaSuccess) e = cudaEventRecord(s->slab_ev[fvs::kHostSlabs], s->copy);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s->stream, s->slab_ev[fvs::kHostSlabs], 0);
    } else {
      e = LaunchSweep(s, s->buf[src], s->buf[dst], plan.dir[q], &s->ctrl->dt,
                      plan.frac, 0.0, skip ? nullptr : &s->ctrl->smax_check[q], s->ctrl,
                      q > 0 ? q - 1 : -1, q > 0 ? plan.dx[q - 1] : 0.0, skip);
    }
    if (e != cudaSuccess) return e;
    src = dst;
    dst = (dst == X) ? Y : X;
  }
  fvs::EndStepKernel<<<1, 1, 0, s->stream>>>(s->ctrl, plan, step_in_batch,
                                             s->dt_log_dev, s->dt_log_cap);
  return cudaGetLastError();
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI

extern "C" {

void fvs_method_default(fvs_method* m) {
  if (!m) return;
  std::memset(m, 0, sizeof *m);
  m->flux_method = FVS_MUSCL_HLLE;
  m->limiter = FVS_VAN_LEER;
  m->precision = FVS_FP64_EXACT;
  m->guess = FVS_GUESS_MEAN;
  m->max_iterations = 5000;
  m->tolerance = 1e-7;
  m->gamma = 1.4;
}

const char* fvs_last_error(void) { return g_last_error.c_str(); }

int fvs_abi_version(void) { return 1; }

int fvs_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int fvs_compute_numeric_fluxes(const fvs_method* m, int rank,
                               double* fluxes_dev, fvs_box face_box,
                               const double* states_dev, fvs_box cell_box,
                               double dt, double dx, int dir, void* stream) {
  if (int r = CheckMethod(m, rank)) return r;
  if (dir < 0 || dir >= rank) return Fail(FVS_ERR_INVALID, "direction out of range");
  if (!ValidBox(face_box) || !ValidBox(cell_box))
    return Fail(FVS_ERR_INVALID, "invalid box");
  if (Volume(face_box) == 0) return FVS_OK;
  if (!fluxes_dev || !states_dev) return Fail(FVS_ERR_INVALID, "NULL data pointer");
  // every stencil cell must lie in cell_box
  const int w = StencilWidth(m->flux_method);
  int lo[3], hi[3];
  for (int d = 0; d < 3; ++d) {
    lo[d] = face_box.lo[d];
    hi[d] = face_box.hi[d];
  }
  lo[dir] -= w;
  hi[dir] += w - 1;
  if (!Contains(cell_box, lo, hi))
    return Fail(FVS_ERR_INVALID, "cell box does not cover the faces' stencils");
  if (m->precision != FVS_FP64_EXACT)
    return Fail(FVS_ERR_UNSUPPORTED, "patch-level calls run in exact FP64");
  if (IsGodunov(m->flux_method) && m->guess == FVS_GUESS_MLP && !m->mlp_params)
    return Fail(FVS_ERR_INVALID, "FVS_GUESS_MLP needs mlp_params");
  if (int r = CheckDevice()) return r;
  if (m->flux_method == FVS_GODUNOV || m->flux_method == FVS_MUSCL_GODUNOV) {
    FVS_CUDA(fvs::LaunchPatchGodunovFluxes(
        m->flux_method == FVS_MUSCL_GODUNOV, m->limiter, rank, m->gamma, m->guess,
        m->max_iterations, m->tolerance, m->mlp_params, fluxes_dev, ToDesc(face_box),
        states_dev, ToDesc(cell_box), dt, dx, dir, nullptr, static_cast<cudaStream_t>(stream)));
    return FVS_OK;
  }
  FVS_CUDA(fvs::LaunchPatchFluxesExact(m->flux_method, m->limiter, rank, m->gamma,
                                       fluxes_dev, ToDesc(face_box), states_dev,
                                       ToDesc(cell_box), dt, dx, dir,
                                       static_cast<cudaStream_t>(stream)));
  return FVS_OK;
}

int fvs_compute_stable_dt(const fvs_method* m, int rank, const double* states_dev,
                          fvs_box cell_box, double dx, int dir, int window_rule,
                          double* dt_out, void* stream) {
  if (int r = CheckMethod(m, rank)) return r;
  if (dir < 0 || dir >= rank) return Fail(FVS_ERR_INVALID, "direction out of range");
  if (!ValidBox(cell_box)) return Fail(FVS_ERR_INVALID, "invalid box");
  if (!dt_out) return Fail(FVS_ERR_INVALID, "dt_out is NULL");
  if (window_rule != 0 && window_rule != 1)
    return Fail(FVS_ERR_INVALID, "window_rule must be 0 or 1");
  if (IsGodunov(m->flux_method) && m->guess == FVS_GUESS_MLP && !m->mlp_params)
    return Fail(FVS_ERR_INVALID, "FVS_GUESS_MLP needs mlp_params");
  if (int r = CheckDevice()) return r;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned long long* word = nullptr;
  FVS_CUDA(cudaMallocAsync(&word, sizeof *word, st));
  FVS_CUDA(cudaMemsetAsync(word, 0, sizeof *word, st));
  cudaError_t e;
  if (m->flux_method == FVS_GODUNOV || m->flux_method == FVS_MUSCL_GODUNOV) {
    e = fvs::LaunchPatchGodunovStableDt(m->flux_method == FVS_MUSCL_GODUNOV, rank, m->gamma,
                                        m->guess, m->max_iterations, m->tolerance,
                                        m->mlp_params, states_dev, ToDesc(cell_box),
                                        window_rule, dir, word, st);
  } else {
    e = fvs::LaunchPatchStableDtExact(m->flux_method, rank, m->gamma, states_dev,
                                      ToDesc(cell_box), window_rule, dir, word, st);
  }
  unsigned long long bits = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&bits, word, sizeof bits, cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(word, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return CudaFail(e, "fvs_compute_stable_dt");
  const double smax = BitsToDouble(bits);
  *dt_out = (smax > 0.0) ? dx / smax : INFINITY;
  return FVS_OK;
}

int fvs_compute_max_speed(const fvs_method* m, int rank, const double* states_dev,
                          fvs_box cell_box, int dir, int window_rule,
                          unsigned long long* smax_bits_dev, void* stream) {
  if (int r = CheckMethod(m, rank)) return r;
  if (dir < 0 || dir >= rank) return Fail(FVS_ERR_INVALID, "direction out of range");
  if (!ValidBox(cell_box)) return Fail(FVS_ERR_INVALID, "invalid box");
  if (!smax_bits_dev) return Fail(FVS_ERR_INVALID, "smax_bits_dev is NULL");
  if (window_rule != 0 && window_rule != 1)
    return Fail(FVS_ERR_INVALID, "window_rule must be 0 or 1");
  if (IsGodunov(m->flux_method) && m->guess == FVS_GUESS_MLP && !m->mlp_params)
    return Fail(FVS_ERR_INVALID, "FVS_GUESS_MLP needs mlp_params");
  if (int r = CheckDevice()) return r;
  if (Volume(cell_box) == 0) return FVS_OK;
  if (!states_dev) return Fail(FVS_ERR_INVALID, "NULL data pointer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if (IsGodunov(m->flux_method)) {
    e = fvs::LaunchPatchGodunovStableDt(m->flux_method == FVS_MUSCL_GODUNOV, rank, m->gamma,
                                        m->guess, m->max_iterations, m->tolerance,
                                        m->mlp_params, states_dev, ToDesc(cell_box),
                                        window_rule, dir, smax_bits_dev, st);
  } else {
    e = fvs::LaunchPatchStableDtExact(m->flux_method, rank, m->gamma, states_dev,
                                      ToDesc(cell_box), window_rule, dir, smax_bits_dev, st);
  }
  if (e != cudaSuccess) return CudaFail(e, "fvs_compute_max_speed");
  return FVS_OK;
}

int fvs_update_conservatively_region(double* next_dev, fvs_box next_box, fvs_box region,
                                     const double* prev_dev, fvs_box prev_box,
                                     const double* fluxes_dev, fvs_box face_box, int ncomp,
                                     double dt, double dx, int dir, void* stream) {
  if (dir < 0 || dir > 2) return Fail(FVS_ERR_INVALID, "direction out of range");
  if (ncomp < 1) return Fail(FVS_ERR_INVALID, "ncomp must be positive");
  if (!ValidBox(next_box) || !ValidBox(prev_box) || !ValidBox(face_box) || !ValidBox(region))
    return Fail(FVS_ERR_INVALID, "invalid box");
  if (Volume(region) == 0) return FVS_OK;
  if (!Contains(next_box, region.lo, region.hi))
    return Fail(FVS_ERR_INVALID, "next box does not cover the region");
  if (!Contains(prev_box, region.lo, region.hi))
    return Fail(FVS_ERR_INVALID, "prev box does not cover the region");
  int hi[3] = {region.hi[0], region.hi[1], region.hi[2]};
  hi[dir] += 1;
  if (!Contains(face_box, region.lo, hi))
    return Fail(FVS_ERR_INVALID, "face box does not cover the faces of the region");
  if (int r = CheckDevice()) return r;
  FVS_CUDA(fvs::LaunchPatchUpdate(next_dev, ToDesc(next_box), ToDesc(region), prev_dev,
                                  ToDesc(prev_box), fluxes_dev, ToDesc(face_box), ncomp, dt,
                                  dx, dir, static_cast<cudaStream_t>(stream)));
  return FVS_OK;
}

int fvs_update_conservatively(double* next_dev, fvs_box next_box,
                              const double* prev_dev, fvs_box prev_box,
                              const double* fluxes_dev, fvs_box face_box,
                              int ncomp, double dt, double dx, int dir,
                              void* stream) {
  return fvs_update_conservatively_region(next_dev, next_box, next_box, prev_dev, prev_box,
                                          fluxes_dev, face_box, ncomp, dt, dx, dir, stream);
}

int fvs_complete_from_cons(int rank, double gamma, double* complete_dev,
                           fvs_box complete_box, const double* cons_dev,
                           fvs_box cons_box, fvs_box region, void* stream) {
  if (rank < 1 || rank > 3) return Fail(FVS_ERR_INVALID, "rank must be 1, 2 or 3");
  if (!(gamma > 1.0)) return Fail(FVS_ERR_INVALID, "gamma must exceed 1");
  if (!ValidBox(complete_box) || !ValidBox(cons_box) || !ValidBox(region))
    return Fail(FVS_ERR_INVALID, "invalid box");
  if (Volume(region) == 0) return FVS_OK;
  if (!Contains(complete_box, region.lo, region.hi) ||
      !Contains(cons_box, region.lo, region.hi))
    return Fail(FVS_ERR_INVALID, "region outside the data boxes");
  if (int r = CheckDevice()) return r;
  FVS_CUDA(fvs::LaunchPatchCompleteFromCons(rank, gamma, complete_dev,
                                            ToDesc(complete_box), cons_dev,
                                            ToDesc(cons_box), ToDesc(region),
                                            static_cast<cudaStream_t>(stream)));
  return FVS_OK;
}

int fvs_solver_create(const fvs_grid_desc* grid, const fvs_method* m,
                      fvs_solver** out) {
  if (!grid || !out) return Fail(FVS_ERR_INVALID, "NULL argument");
  if (int r = CheckMethod(m, grid->rank)) return r;
  if ((m->flux_method == FVS_HLLE))
    return Fail(FVS_ERR_UNSUPPORTED, "the solver runs MUSCL-Hancock, HLLEM or Godunov fluxes");
  if (HllemRecon(m->flux_method) >= 0 && m->precision != FVS_FP64_EXACT)
    return Fail(FVS_ERR_UNSUPPORTED, "HLLEM runs in exact FP64");
  if (IsGodunov(m->flux_method) && m->precision != FVS_FP64_EXACT &&
      m->precision != FVS_FP64_FAST)
    return Fail(FVS_ERR_UNSUPPORTED, "the exact Riemann solver runs in FP64");
  if (IsGodunov(m->flux_method) && m->guess == FVS_GUESS_MLP && !m->mlp_params)
    return Fail(FVS_ERR_INVALID, "FVS_GUESS_MLP needs mlp_params");
  for (int d = 0; d < 3; ++d) {
    const bool used = d < grid->rank;
    if (used && grid->n[d] < 1) return Fail(FVS_ERR_INVALID, "extent must be >= 1");
    if (!used && grid->n[d] != 1)
      return Fail(FVS_ERR_INVALID, "unused directions must have extent 1");
    if (used && grid->bc[d] != FVS_BC_PERIODIC && grid->bc[d] != FVS_BC_TRANSMISSIVE &&
        grid->bc[d] != FVS_BC_REFLECTIVE)
      return Fail(FVS_ERR_INVALID, "unknown boundary condition");
    if (used && grid->bc[d] == FVS_BC_REFLECTIVE && grid->n[d] < 2)
      return Fail(FVS_ERR_INVALID, "a reflective direction needs at least 2 cells");
    if (used && !(grid->dx[d] > 0.0)) return Fail(FVS_ERR_INVALID, "dx must be positive");
  }
  if (grid->dt_rule != 0 && grid->dt_rule != 1)
    return Fail(FVS_ERR_INVALID, "dt_rule must be 0 or 1");
  if (int r = CheckDevice()) return r;
  fvs_solver* s = new fvs_solver();
  s->g = *grid;
  s->m = *m;
  s->cells = int64_t(grid->n[0]) * grid->n[1] * grid->n[2];
  s->ncons = grid->rank + 2;
  const size_t bytes = size_t(s->cells) * s->ncons * sizeof(double);
  cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  for (int b = 0; b < 3 && e == cudaSuccess; ++b) e = cudaMalloc(&s->buf[b], bytes);
  if (e == cudaSuccess) e = cudaMalloc(&s->ctrl, sizeof(fvs::Control));
  if (e == cudaSuccess) e = cudaMallocHost(&s->ctrl_host, sizeof(fvs::Control));
  if (e == cudaSuccess) e = cudaMalloc(&s->scratch_words, 8 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&s->newton_words, 3 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(s->newton_words, 0, 3 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(s->ctrl, 0, sizeof(fvs::Control));
  if (e != cudaSuccess) {
    delete s;
    return CudaFail(e, "fvs_solver_create");
  }
  *out = s;
  return FVS_OK;
}

int fvs_solver_destroy(fvs_solver* s) {
  if (!s) return FVS_OK;
  if (s->stream) cudaStreamSynchronize(s->stream);
  delete s;
  return FVS_OK;
}

int fvs_solver_upload(fvs_solver* s, const double* cons_host) {
  if (!s || !cons_host) return Fail(FVS_ERR_INVALID, "NULL argument");
  const size_t bytes = size_t(s->cells) * s->ncons * sizeof(double);
  FVS_CUDA(cudaMemcpyAsync(s->buf[s->cur], cons_host, bytes, cudaMemcpyHostToDevice,
                           s->stream));
  FVS_CUDA(cudaStreamSynchronize(s->stream));
  return FVS_OK;
}

int fvs_solver_download(fvs_solver* s, double* cons_host) {
  if (!s || !cons_host) return Fail(FVS_ERR_INVALID, "NULL argument");
  const size_t bytes = size_t(s->cells) * s->ncons * sizeof(double);
  FVS_CUDA(cudaMemcpyAsync(cons_host, s->buf[s->cur], bytes, cudaMemcpyDeviceToHost,
                           s->stream));
  FVS_CUDA(cudaStreamSynchronize(s->stream));
  return FVS_OK;
}

int fvs_solver_write_plotfile(fvs_solver* s, const char* dir) {
  if (!s || !dir || !*dir) return Fail(FVS_ERR_INVALID, "NULL argument");
  const int rank = s->g.rank;
  fvs::plot::Plotfile pf;
  pf.dir = dir;
  pf.dim = rank;
  pf.time = s->t;
  pf.vars = fvs::plot::CompleteNames(rank);
  if (s->cc) {
    pf.vars.push_back("Boundary_X");
    pf.vars.push_back("Boundary_Y");
    pf.vars.push_back("vfrac");
  }
  const int ncomp = static_cast<int>(pf.vars.size());
  fvs::plot::Level L{};
  for (int d = 0; d < 3; ++d) {
    L.domain.lo[d] = 0;
    L.domain.hi[d] = s->g.n[d] - 1;
    L.dx[d] = d < rank ? s->g.dx[d] : 1.0;
    pf.prob_hi[d] = d < rank ? s->g.n[d] * s->g.dx[d] : 1.0;
  }
  L.step = static_cast<int>(s->cycle);
  L.ratio_to_next = 2;
  // slabs of the slowest direction, at most 2^21 cells each
  const int slow = rank - 1;
  const int64_t plane = s->cells / s->g.n[slow];
  const int per = static_cast<int>(std::max<int64_t>(
      1, std::min<int64_t>(s->g.n[slow], (int64_t(1) << 21) / plane)));
  for (int z0 = 0; z0 < s->g.n[slow]; z0 += per) {
    fvs::plot::Box b = L.domain;
    b.lo[slow] = z0;
    b.hi[slow] = std::min(s->g.n[slow] - 1, z0 + per - 1);
    L.boxes.push_back(b);
  }
  pf.levels.push_back(L);
  if (std::string e = fvs::plot::WriteHeader(pf); !e.empty()) return Fail(FVS_ERR_IO, e);
  if (int r = CheckDevice()) return r;
  const int64_t max_cells = plane * per;
  const size_t bytes = size_t(max_cells) * size_t(ncomp) * sizeof(double);
  double* dbuf = nullptr;
  double* hbuf = nullptr;
  FVS_CUDA(cudaMallocAsync(&dbuf, bytes, s->stream));
  if (cudaMallocHost(&hbuf, bytes) != cudaSuccess) {
    cudaFreeAsync(dbuf, s->stream);
    return Fail(FVS_ERR_CUDA, "cudaMallocHost failed for the plotfile buffer");
  }
  fvs::plot::LevelWriter w(pf, 0);
  std::string err;
  cudaError_t ce = cudaSuccess;
  const double* cons = s->buf[s->cur];
  for (size_t bi = 0; bi < pf.levels[0].boxes.size() && err.empty() && ce == cudaSuccess;
       ++bi) {
    const fvs::plot::Box& b = pf.levels[0].boxes[bi];
    const int64_t n = b.Cells(3);
    if (s->cc) {
      ce = fvs::LaunchCutCellPlotData(s->ccg, cons, s->m.gamma, b.lo[1], b.hi[1] - b.lo[1] + 1,
                                      dbuf, s->stream);
    } else {
      fvs::BoxDesc q{}, u{};
      for (int d = 0; d < 3; ++d) {
        q.lo[d] = b.lo[d];
        q.n[d] = b.hi[d] - b.lo[d] + 1;
        u.lo[d] = 0;
        u.n[d] = s->g.n[d];
      }
      ce = fvs::LaunchPatchCompleteFromCons(rank, s->m.gamma, dbuf, q, cons, u, q, s->stream);
    }
    if (ce == cudaSuccess)
      ce = cudaMemcpyAsync(hbuf, dbuf, size_t(n) * size_t(ncomp) * sizeof(double),
                           cudaMemcpyDeviceToHost, s->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s->stream);
    if (ce == cudaSuccess) err = w.Append(static_cast<int>(bi), hbuf);
  }
  if (err.empty() && ce == cudaSuccess) err = w.Finish();
  cudaFreeAsync(dbuf, s->stream);
  cudaStreamSynchronize(s->stream);
  cudaFreeHost(hbuf);
  if (ce != cudaSuccess) return Fail(FVS_ERR_CUDA, cudaGetErrorString(ce));
  if (!err.empty()) return Fail(FVS_ERR_IO, err);
  return FVS_OK;
}

int fvs_solver_state_device(fvs_solver* s, double** cons_dev) {
  if (!s || !cons_dev) return Fail(FVS_ERR_INVALID, "NULL argument");
  *cons_dev = s->buf[s->cur];
  return FVS_OK;
}

int fvs_solver_set_tiling(fvs_solver* s, int seg_len) {
  if (!s || seg_len < 0) return Fail(FVS_ERR_INVALID, "bad tiling");
  s->seg_len = seg_len;
  return FVS_OK;
}

int fvs_solver_set_launch(fvs_solver* s, int dir, int seg_len, int variant) {
  if (!s) return Fail(FVS_ERR_INVALID, "NULL solver");
  if (dir < 0 || dir >= s->g.rank) return Fail(FVS_ERR_INVALID, "direction out of range");
  if (seg_len < 0) return Fail(FVS_ERR_INVALID, "segment length must be >= 0");
  const bool plain_hlle = s->m.flux_method <= FVS_HLLE && !s->cc;
  bool ok = variant == 0;
  if (s->m.precision == FVS_MIXED && plain_hlle)
    ok = variant == 0 || variant == 4 || variant == 5 ||
         (dir == 0 && (variant == 10 || variant == 14 || variant == 15)) ||
         (dir >= 1 && (variant == 20 || variant == 24 || variant == 25) && TmaMapsReady(s));
  if (s->m.precision == FVS_FP64_DF && plain_hlle) ok = variant == 0 || variant == 3;
  // cut cells: the mixed flavour's y sweeps march (10) instead of tiling (0)
  if (s->cc) ok = variant == 0 || (variant == 10 && dir == 1 && s->m.precision == FVS_MIXED);
  if (!ok) return Fail(FVS_ERR_INVALID, "no such launch variant for this method");
  s->seg_tuned[dir] = seg_len;
  s->occ_tuned[dir] = variant;
  for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
  s->graphs.clear();
  return FVS_OK;
}

int fvs_solver_autotune(fvs_solver* s, int* seg_out) {
  if (!s) return Fail(FVS_ERR_INVALID, "NULL solver");
  // Candidate segment lengths per direction (and, for the mixed flavour,
  // register/occupancy variants of the same kernel), timed on the current
  // state with a small dt (output goes to a spare buffer; the state is not
  // changed).
  const int cands[] = {8, 16, 32, 64, 128, 256, 512};
  const bool plain_hlle = s->m.flux_method <= FVS_HLLE && !s->cc;
  const bool mixed = s->m.precision == FVS_MIXED && plain_hlle;
  const bool df = s->m.precision == FVS_FP64_DF && plain_hlle;
  // mixed x sweeps: lanes-along-x kernel (0, 4, 5) or marching kernel (10, 14, 15);
  // mixed y/z sweeps: marching kernel (0, 4, 5) or TMA-staged kernel (20, 24, 25)
  const int occs_mixed_x[] = {0, 4, 5, 10, 14, 15};
  const int occs_mixed[] = {0, 4, 5, 20, 24, 25};
  const bool tma = mixed && TmaMapsReady(s);
  const int occs_df[] = {0, 3};
  const int occs_plain[] = {0};
  // cut cells: segment lengths of the FP64 flavours' regular-cell sweep (the
  // mixed flavour's cut-cell kernels have no launch parameter to tune)
  const bool cc_cell = s->cc && s->m.precision == FVS_MIXED;
  const int occs_cc_mixed_y[] = {0, 10};
  const int saved = s->seg_len;
  cudaEvent_t e0, e1;
  FVS_CUDA(cudaEventCreate(&e0));
  FVS_CUDA(cudaEventCreate(&e1));
  double dt = 0.0;
  {
    const int r = fvs_solver_stable_dt(s, -1, &dt);
    if (r) return r;
  }
  dt = std::isfinite(dt) ? 0.1 * dt : 1e-6;
  const int out = (s->cur + 1) % 3;
  // cut cells: the sweeps read the wall reference states of the current state
  if (s->cc) FVS_CUDA(CcReferenceStates(s, s->buf[s->cur]));
  for (int d = 0; d < s->g.rank; ++d) {
    const int nd = s->g.n[d];
    const int* occs = mixed                ? (d == 0 ? occs_mixed_x : occs_mixed)
                      : (cc_cell && d == 1) ? occs_cc_mixed_y
                      : df                  ? occs_df
                                            : occs_plain;
    const int nocc = mixed ? (d == 0 || tma ? 6 : 3) : ((cc_cell && d == 1) || df ? 2 : 1);
    float best = 1e30f;
    int best_seg = 0, best_occ = 0;
    for (int oi = 0; oi < nocc; ++oi) {
      s->occ_tuned[d] = occs[oi];
      // the lanes-along-x kernel has no segment length: one candidate
      const bool warp_x = mixed && d == 0 && occs[oi] < 10;
      for (int c : cands) {
        if (c > 2 * nd && c != cands[0]) break;
        // the tile kernels (mixed cut cells, variant 0) have no segment length
        if ((warp_x || (cc_cell && occs[oi] == 0)) && c != cands[0]) break;
        s->seg_len = c;
        float ms_sum = 0.f;
        for (int rep = 0; rep < 3; ++rep) {
          // the sweep's max slot starts at zero, as in a step
          FVS_CUDA(cudaMemsetAsync(s->scratch_words, 0, sizeof(unsigned long long), s->stream));
          FVS_CUDA(cudaEventRecord(e0, s->stream));
          FVS_CUDA(LaunchSweep(s, s->buf[s->cur], s->buf[out], d, nullptr, 1.0, dt,
                               s->scratch_words, nullptr, -1, 0.0));
          FVS_CUDA(cudaEventRecord(e1, s->stream));
          FVS_CUDA(cudaEventSynchronize(e1));
          float ms = 0.f;
          FVS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
          if (rep > 0) ms_sum += ms;
        }
        if (ms_sum < best) {
          best = ms_sum;
          best_seg = c;
          best_occ = occs[oi];
        }
      }
    }
    s->seg_tuned[d] = best_seg;
    s->occ_tuned[d] = best_occ;
    if (seg_out) seg_out[d] = best_seg;
  }
  s->seg_len = saved;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
  s->graphs.clear();
  return FVS_OK;
}

int fvs_solver_tuning(fvs_solver* s, int32_t* seg, int32_t* occupancy) {
  if (!s) return Fail(FVS_ERR_INVALID, "NULL solver");
  for (int d = 0; d < 3; ++d) {
    if (seg) seg[d] = s->seg_tuned[d];
    if (occupancy) occupancy[d] = s->occ_tuned[d];
  }
  return FVS_OK;
}

int fvs_cutcell_ghost_layers(void) { return fvs::kCcGhost; }

}  // extern "C"

namespace {

// Embeds the body given by shape records (fvs_cutcell_geometry.cuh) into a
// rank-2 MUSCL-HLLE solver: geometry, shielded fractions, cut flags, cell
// classes and band lists on the device.
int EmbedShapes(fvs_solver* s, const std::vector<double>& words, double x0, double y0) {
  if (s->g.rank != 2) return Fail(FVS_ERR_UNSUPPORTED, "cut cells need a rank-2 grid");
  if (s->m.flux_method != FVS_MUSCL_HLLE)
    return Fail(FVS_ERR_UNSUPPORTED, "cut cells run MUSCL-Hancock + HLLE");
  if (s->m.precision == FVS_FP64_DF)
    return Fail(FVS_ERR_UNSUPPORTED, "cut cells run in exact FP64, fast FP64 or mixed precision");
  if (s->cc) return Fail(FVS_ERR_INVALID, "embedded boundary already set");
  fvs::CcGeom& g = s->ccg;
  g.nx = s->g.n[0];
  g.ny = s->g.n[1];
  const size_t cells = size_t(g.NX()) * g.NY();
  const size_t fx = size_t(g.NX() + 1) * g.NY(), fy = size_t(g.NX()) * (g.NY() + 1);
  auto alloc = [&](double** p, size_t n) -> cudaError_t {
    cudaError_t e = cudaMalloc(p, n * sizeof(double));
    if (e == cudaSuccess) {
      s->cc_allocs.push_back(*p);
      e = cudaMemset(*p, 0, n * sizeof(double));
    }
    return e;
  };
  FVS_CUDA(alloc(&g.alpha, cells));
  FVS_CUDA(alloc(&g.beta[0], fx));
  FVS_CUDA(alloc(&g.beta[1], fy));
  FVS_CUDA(alloc(&g.normal, 2 * cells));
  FVS_CUDA(alloc(&g.center, 2 * cells));
  for (int d = 0; d < 2; ++d) {
    const size_t nf = d == 0 ? fx : fy;
    FVS_CUDA(alloc(&g.us[d], nf));
    FVS_CUDA(alloc(&g.sL[d], nf));
    FVS_CUDA(alloc(&g.sR[d], nf));
    FVS_CUDA(alloc(&g.us_rel[d], nf));
    FVS_CUDA(alloc(&g.sL_rel[d], nf));
    FVS_CUDA(alloc(&g.sR_rel[d], nf));
  }
  FVS_CUDA(alloc(&s->cc_refs, 6 * cells));
  void* cut = nullptr;
  FVS_CUDA(cudaMalloc(&cut, cells));
  s->cc_allocs.push_back(cut);
  g.cut = static_cast<signed char*>(cut);
  double* dshape = nullptr;
  FVS_CUDA(alloc(&dshape, words.size()));
  FVS_CUDA(cudaMemcpy(dshape, words.data(), sizeof(double) * words.size(),
                      cudaMemcpyHostToDevice));
  fvs::CcGeomArgs ga{};
  ga.nx = g.nx;
  ga.ny = g.ny;
  ga.x0 = x0;
  ga.y0 = y0;
  ga.dx = s->g.dx[0];
  ga.dy = s->g.dx[1];
  ga.nwords = static_cast<int>(words.size());
  ga.shapes = dshape;
  ga.alpha = g.alpha;
  ga.betax = g.beta[0];
  ga.betay = g.beta[1];
  ga.normal = g.normal;
  ga.center = g.center;
  FVS_CUDA(fvs::LaunchCutCellGeometry(ga, g, s->stream));
  // cell classes of both sweep directions, the tiles with regular cells and
  // the lists of band cells
  for (int d = 0; d < 2; ++d) {
    const size_t ncell = size_t(g.nx) * g.ny;
    const size_t ntiles = size_t(g.NGroups(d)) * g.NTiles(d);
    void* cls = nullptr;
    void* treg = nullptr;
    FVS_CUDA(cudaMalloc(&cls, ncell));
    s->cc_allocs.push_back(cls);
    FVS_CUDA(cudaMalloc(&treg, ntiles));
    s->cc_allocs.push_back(treg);
    g.cell_class[d] = static_cast<signed char*>(cls);
    g.tile_regular[d] = static_cast<signed char*>(treg);
    FVS_CUDA(fvs::LaunchCutCellClasses(g, d, s->stream));
    std::vector<signed char> h(ncell);
    FVS_CUDA(cudaMemcpyAsync(h.data(), cls, ncell, cudaMemcpyDeviceToHost, s->stream));
    FVS_CUDA(cudaStreamSynchronize(s->stream));
    std::vector<int> band;
    for (size_t k = 0; k < ncell; ++k)
      if (h[k] == fvs::kCcBand) band.push_back(static_cast<int>(k));
    g.nband[d] = static_cast<int>(band.size());
    g.band[d] = nullptr;
    if (!band.empty()) {
      void* b = nullptr;
      FVS_CUDA(cudaMalloc(&b, band.size() * sizeof(int)));
      s->cc_allocs.push_back(b);
      g.band[d] = static_cast<int*>(b);
      FVS_CUDA(cudaMemcpy(b, band.data(), band.size() * sizeof(int), cudaMemcpyHostToDevice));
    }
  }
  if (!s->side) {
    FVS_CUDA(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking));
    FVS_CUDA(cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming));
    FVS_CUDA(cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming));
  }
  FVS_CUDA(cudaStreamSynchronize(s->stream));
  s->cc = true;
  for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
  s->graphs.clear();
  return FVS_OK;
}

// Crossings of the grid lines x = x0 + i dx and y = y0 + j dy (the grown
// grid's cell edges) with a polygon's edges, at most per line.
int MaxCrossings(const double* xy, int nv, int n, double origin, double h, bool vertical) {
  int worst = 0;
  for (int i = -fvs::kCcGhost; i <= n + fvs::kCcGhost; ++i) {
    const double c = origin + double(i) * h;
    int m = 0;
    for (int e = 0; e + 1 < nv; ++e) {
      const double vf = vertical ? xy[2 * e] : xy[2 * e + 1];
      const double wf = vertical ? xy[2 * e + 2] : xy[2 * e + 3];
      if ((vf < c && c <= wf) || (wf < c && c <= vf)) ++m;
    }
    worst = std::max(worst, m);
  }
  return worst;
}

}  // namespace

extern "C" {

int fvs_solver_set_embedded_circles(fvs_solver* s, const double* circles, int ncircles,
                                    double x0, double y0) {
  if (!s || !circles) return Fail(FVS_ERR_INVALID, "NULL argument");
  if (ncircles < 1 || ncircles > 16) return Fail(FVS_ERR_INVALID, "1 to 16 circles");
  std::vector<double> words;
  for (int k = 0; k < ncircles; ++k) {
    if (!(circles[3 * k + 2] > 0.0)) return Fail(FVS_ERR_INVALID, "circle radius must be > 0");
    const double rec[5] = {0.0, 0.0, circles[3 * k], circles[3 * k + 1], circles[3 * k + 2]};
    words.insert(words.end(), rec, rec + 5);
  }
  return EmbedShapes(s, words, x0, y0);
}

int fvs_solver_set_embedded_geometry(fvs_solver* s, const fvs_shape* shapes, int nshapes,
                                     double x0, double y0) {
  if (!s || !shapes) return Fail(FVS_ERR_INVALID, "NULL argument");
  if (nshapes < 1 || nshapes > 256) return Fail(FVS_ERR_INVALID, "1 to 256 shapes");
  std::vector<double> words;
  for (int k = 0; k < nshapes; ++k) {
    const fvs_shape& sh = shapes[k];
    const double inv = sh.inverted ? 1.0 : 0.0;
    if (sh.kind == FVS_SHAPE_CIRCLE) {
      if (!(sh.p[2] > 0.0)) return Fail(FVS_ERR_INVALID, "circle radius must be > 0");
      const double rec[5] = {0.0, inv, sh.p[0], sh.p[1], sh.p[2]};
      words.insert(words.end(), rec, rec + 5);
    } else if (sh.kind == FVS_SHAPE_HALFSPACE) {
      // the normal made a unit vector (Halfspace's constructor normalises)
      const double nn = std::sqrt(sh.p[0] * sh.p[0] + sh.p[1] * sh.p[1]);
      if (!(nn > 0.0)) return Fail(FVS_ERR_INVALID, "half-space normal must be nonzero");
      const double rec[5] = {1.0, inv, sh.p[0] / nn, sh.p[1] / nn, sh.p[2]};
      words.insert(words.end(), rec, rec + 5);
    } else if (sh.kind == FVS_SHAPE_POLYGON) {
      const int nv = sh.nvertices;
      if (nv < 4 || !sh.xy) return Fail(FVS_ERR_INVALID, "a polygon needs >= 4 vertices");
      if (sh.xy[0] != sh.xy[2 * (nv - 1)] || sh.xy[1] != sh.xy[2 * (nv - 1) + 1])
        return Fail(FVS_ERR_INVALID, "polygon not closed: first and last vertex must agree");
      const int cx = MaxCrossings(sh.xy, nv, s->g.n[0], x0, s->g.dx[0], true);
      const int cy = MaxCrossings(sh.xy, nv, s->g.n[1], y0, s->g.dx[1], false);
      if (std::max(cx, cy) > 64)
        return Fail(FVS_ERR_UNSUPPORTED, "a grid line crosses the polygon more than 64 times");
      words.push_back(2.0);
      words.push_back(inv);
      words.push_back(double(nv));
      words.insert(words.end(), sh.xy, sh.xy + 2 * nv);
    } else {
      return Fail(FVS_ERR_INVALID, "unknown shape kind");
    }
  }
  return EmbedShapes(s, words, x0, y0);
}

int fvs_solver_cutcell_geometry(fvs_solver* s, double* alpha, double* betax, double* betay,
                                double* normal, double* center, int8_t* cut_flags) {
  if (!s || !s->cc) return Fail(FVS_ERR_INVALID, "no embedded boundary");
  const fvs::CcGeom& g = s->ccg;
  const size_t cells = size_t(g.NX()) * g.NY();
  const size_t fx = size_t(g.NX() + 1) * g.NY(), fy = size_t(g.NX()) * (g.NY() + 1);
  if (alpha) FVS_CUDA(cudaMemcpy(alpha, g.alpha, cells * 8, cudaMemcpyDeviceToHost));
  if (betax) FVS_CUDA(cudaMemcpy(betax, g.beta[0], fx * 8, cudaMemcpyDeviceToHost));
  if (betay) FVS_CUDA(cudaMemcpy(betay, g.beta[1], fy * 8, cudaMemcpyDeviceToHost));
  if (normal) FVS_CUDA(cudaMemcpy(normal, g.normal, 2 * cells * 8, cudaMemcpyDeviceToHost));
  if (center) FVS_CUDA(cudaMemcpy(center, g.center, 2 * cells * 8, cudaMemcpyDeviceToHost));
  if (cut_flags) FVS_CUDA(cudaMemcpy(cut_flags, g.cut, cells, cudaMemcpyDeviceToHost));
  return FVS_OK;
}

int fvs_solver_cutcell_shielded(fvs_solver* s, int dir, double* us, double* sL, double* sR,
                                double* us_rel, double* sL_rel, double* sR_rel) {
  if (!s || !s->cc) return Fail(FVS_ERR_INVALID, "no embedded boundary");
  if (dir < 0 || dir > 1) return Fail(FVS_ERR_INVALID, "direction out of range");
  const fvs::CcGeom& g = s->ccg;
  const size_t nf = dir == 0 ? size_t(g.NX() + 1) * g.NY() : size_t(g.NX()) * (g.NY() + 1);
  double* dst[6] = {us, sL, sR, us_rel, sL_rel, sR_rel};
  const double* src[6] = {g.us[dir], g.sL[dir], g.sR[dir], g.us_rel[dir], g.sL_rel[dir],
                          g.sR_rel[dir]};
  for (int k = 0; k < 6; ++k)
    if (dst[k]) FVS_CUDA(cudaMemcpy(dst[k], src[k], nf * 8, cudaMemcpyDeviceToHost));
  return FVS_OK;
}

int fvs_solver_set_cycle(fvs_solver* s, int64_t cycle) {
  if (!s || cycle < 0) return Fail(FVS_ERR_INVALID, "bad cycle");
  s->cycle = cycle;
  return FVS_OK;
}

int fvs_solver_set_time(fvs_solver* s, double t) {
  if (!s) return Fail(FVS_ERR_INVALID, "NULL solver");
  s->t = t;
  return FVS_OK;
}

int fvs_solver_stable_dt(fvs_solver* s, int dir, double* dt_out) {
  if (!s || !dt_out) return Fail(FVS_ERR_INVALID, "NULL argument");
  if (dir < -1 || dir >= s->g.rank) return Fail(FVS_ERR_INVALID, "direction out of range");
  FVS_CUDA(cudaMemsetAsync(s->scratch_words, 0, 3 * sizeof(unsigned long long), s->stream));
  FVS_CUDA(LaunchStable(s, s->buf[s->cur], s->scratch_words, nullptr));
  unsigned long long bits[3];
  FVS_CUDA(cudaMemcpyAsync(bits, s->scratch_words, sizeof bits, cudaMemcpyDeviceToHost,
                           s->stream));
  FVS_CUDA(cudaStreamSynchronize(s->stream));
  double best = INFINITY;
  for (int d = 0; d < s->g.rank; ++d) {
    if (dir >= 0 && d != dir) continue;
    const double smax = BitsToDouble(bits[d]);
    const double dtd = smax > 0.0 ? s->g.dx[d] / smax : INFINITY;
    best = dtd < best ? dtd : best;
  }
  *dt_out = best;
  return FVS_OK;
}

int fvs_solver_sweep(fvs_solver* s, int dir, double dt, double* level_dt_out) {
  if (!s) return Fail(FVS_ERR_INVALID, "NULL solver");
  if (dir < 0 || dir >= s->g.rank) return Fail(FVS_ERR_INVALID, "direction out of range");
  const int out = (s->cur + 1) % 3;
  if (s->cc)
    FVS_CUDA(CcReferenceStates(s, s->buf[s->cur]));
  FVS_CUDA(cudaMemsetAsync(s->scratch_words, 0, sizeof(unsigned long long), s->stream));
  FVS_CUDA(LaunchSweep(s, s->buf[s->cur], s->buf[out], dir, nullptr, 1.0, dt,
                       s->scratch_words, nullptr, -1, 0.0));
  unsigned long long bits = 0;
  FVS_CUDA(cudaMemcpyAsync(&bits, s->scratch_words, sizeof bits, cudaMemcpyDeviceToHost,
                           s->stream));
  FVS_CUDA(cudaStreamSynchronize(s->stream));
  s->cur = out;
  if (level_dt_out) {
    const double smax = BitsToDouble(bits);
    *level_dt_out = smax > 0.0 ? s->g.dx[dir] / smax : INFINITY;
  }
  return FVS_OK;
}

int fvs_solver_step(fvs_solver* s, double dt, int cycle) {
  if (!s) return Fail(FVS_ERR_INVALID, "NULL solver");
  if (!(dt > 0.0)) return Fail(FVS_ERR_INVALID, "dt must be positive");
  const fvs::StepPlan plan = MakePlan(s, cycle);
  const double split_dt = plan.frac * dt;
  FVS_CUDA(cudaMemsetAsync(s->scratch_words, 0, 8 * sizeof(unsigned long long), s->stream));
  const int start = s->cur;
  if (s->cc)
    FVS_CUDA(CcReferenceStates(s, s->buf[start]));
  const int X = (start + 1) % 3, Y = (start + 2) % 3;
  int src = start, dst = X;
  for (int q = 0; q < plan.nsweeps; ++q) {
    FVS_CUDA(LaunchSweep(s, s->buf[src], s->buf[dst], plan.dir[q], nullptr, 1.0,
                         split_dt, s->scratch_words + q, nullptr, -1, 0.0));
    src = dst;
    dst = (dst == X) ? Y : X;
  }
  unsigned long long bits[8];
  FVS_CUDA(cudaMemcpyAsync(bits, s->scratch_words, sizeof bits, cudaMemcpyDeviceToHost,
                           s->stream));
  FVS_CUDA(cudaStreamSynchronize(s->stream));
  for (int q = 0; q < plan.nsweeps; ++q) {
    const double level_dt = plan.dx[q] / BitsToDouble(bits[q]);
    if (level_dt < split_dt) {
      return Fail(FVS_ERR_DT_TOO_LARGE, "per-sweep CFL check failed");
    }
  }
  s->cur = src;
  return FVS_OK;
}

int fvs_solver_newton_stats(fvs_solver* s, uint64_t* iterations, uint64_t* failures,
                            uint64_t* fallbacks, int reset) {
  if (!s) return Fail(FVS_ERR_INVALID, "NULL solver");
  unsigned long long a[3], b[3];
  FVS_CUDA(cudaMemcpyAsync(a, s->newton_words, sizeof a, cudaMemcpyDeviceToHost, s->stream));
  FVS_CUDA(cudaMemcpyAsync(b, s->ctrl->newton, sizeof b, cudaMemcpyDeviceToHost, s->stream));
  FVS_CUDA(cudaStreamSynchronize(s->stream));
  if (iterations) *iterations = a[0] + b[0];
  if (failures) *failures = a[1] + b[1];
  if (fallbacks) *fallbacks = a[2] + b[2];
  if (reset) {
    FVS_CUDA(cudaMemsetAsync(s->newton_words, 0, sizeof a, s->stream));
    FVS_CUDA(cudaMemsetAsync(s->ctrl->newton, 0, sizeof b, s->stream));
    FVS_CUDA(cudaStreamSynchronize(s->stream));
  }
  return FVS_OK;
}

int fvs_exact_riemann_star(const fvs_method* m, int64_t n, const double* rhoL_dev,
                           const double* uL_dev, const double* pL_dev,
                           const double* rhoR_dev, const double* uR_dev,
                           const double* pR_dev, double* pstar_dev, double* ustar_dev,
                           int32_t* iterations_dev, int32_t* status_dev, void* stream) {
  if (int r = CheckMethod(m, 1)) return r;
  if (n < 0) return Fail(FVS_ERR_INVALID, "n must be non-negative");
  if (n > 0 && (!rhoL_dev || !uL_dev || !pL_dev || !rhoR_dev || !uR_dev || !pR_dev))
    return Fail(FVS_ERR_INVALID, "NULL input array");
  if (m->max_iterations < 0) return Fail(FVS_ERR_INVALID, "max_iterations must be >= 0");
  if (m->guess == FVS_GUESS_MLP && !m->mlp_params)
    return Fail(FVS_ERR_INVALID, "FVS_GUESS_MLP needs mlp_params");
  if (int r = CheckDevice()) return r;
  FVS_CUDA(fvs::LaunchExactStar(n, m->gamma, m->guess, m->max_iterations, m->tolerance,
                                m->mlp_params, rhoL_dev, uL_dev, pL_dev, rhoR_dev, uR_dev, pR_dev,
                                pstar_dev, ustar_dev, iterations_dev, status_dev,
                                static_cast<cudaStream_t>(stream)));
  return FVS_OK;
}

int fvs_solver_stream(fvs_solver* s, void** stream) {
  if (!s || !stream) return Fail(FVS_ERR_INVALID, "NULL argument");
  *stream = static_cast<void*>(s->stream);
  return FVS_OK;
}

int fvs_solver_step_host(fvs_solver* s, double* cons_host, double cfl, double t_end,
                         fvs_run_stats* stats) {
  if (!s || !cons_host) return Fail(FVS_ERR_INVALID, "NULL argument");
  if (!(cfl > 0.0)) return Fail(FVS_ERR_INVALID, "cfl must be positive");
  if (s->cc)
    return Fail(FVS_ERR_UNSUPPORTED,
                "host-resident steps of cut-cell grids: use fvs_solver_upload, _run, _download");
  if (!s->copy) {
    FVS_CUDA(cudaStreamCreateWithFlags(&s->copy, cudaStreamNonBlocking));
    FVS_CUDA(cudaStreamCreateWithFlags(&s->slab, cudaStreamNonBlocking));
    FVS_CUDA(cudaEventCreateWithFlags(&s->slab_fork, cudaEventDisableTiming));
    for (cudaEvent_t& e : s->slab_ev)
      FVS_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  const size_t bytes = size_t(s->cells) * s->ncons * sizeof(double);
  fvs::Control c{};
  c.t = s->t;
  c.t_end = t_end;
  c.cfl = cfl;
  FVS_CUDA(cudaMemcpyAsync(s->ctrl, &c, sizeof c, cudaMemcpyHostToDevice, s->stream));
  // The upload, in slabs of z-planes on the copy stream, overlaps the
  // stable-dt pass, which takes each slab's faces once it has landed (the
  // first slab last: its z faces read the last plane on a periodic grid).
  // Methods whose stable-dt pass has no plane ranges upload in one piece.
  const bool reflective = s->g.bc[0] == FVS_BC_REFLECTIVE || s->g.bc[1] == FVS_BC_REFLECTIVE ||
                          s->g.bc[2] == FVS_BC_REFLECTIVE;
  const bool piped = s->g.rank == 3 && s->m.flux_method <= FVS_HLLE && !reflective &&
                     s->t < t_end && s->g.n[2] >= fvs::kHostSlabs;
  double* dev = s->buf[s->cur];
  if (piped) {
    const int nz = s->g.n[2], ns = fvs::kHostSlabs;
    const size_t plane = size_t(s->g.n[0]) * s->g.n[1], cs = size_t(s->cells);
    FVS_CUDA(cudaMemsetAsync(s->ctrl->smax_stable, 0, sizeof(s->ctrl->smax_stable), s->stream));
    FVS_CUDA(cudaEventRecord(s->slab_ev[fvs::kHostSlabs], s->stream));
    FVS_CUDA(cudaStreamWaitEvent(s->copy, s->slab_ev[fvs::kHostSlabs], 0));
    for (int k = 0; k < ns; ++k) {
      const int z0 = nz * k / ns, z1 = nz * (k + 1) / ns;
      for (int comp = 0; comp < s->ncons; ++comp)
        FVS_CUDA(cudaMemcpyAsync(dev + comp * cs + z0 * plane, cons_host + comp * cs + z0 * plane,
                                 size_t(z1 - z0) * plane * sizeof(double),
                                 cudaMemcpyHostToDevice, s->copy));
      FVS_CUDA(cudaEventRecord(s->slab_ev[k], s->copy));
      if (k == 0) continue;
      FVS_CUDA(cudaStreamWaitEvent(s->stream, s->slab_ev[k], 0));
      FVS_CUDA(LaunchStable(s, dev, s->ctrl->smax_stable, s->ctrl, z0, z1));
    }
    FVS_CUDA(cudaStreamWaitEvent(s->stream, s->slab_ev[0], 0));
    FVS_CUDA(LaunchStable(s, dev, s->ctrl->smax_stable, s->ctrl, 0, nz / ns));
  } else {
    FVS_CUDA(cudaMemcpyAsync(dev, cons_host, bytes, cudaMemcpyHostToDevice, s->stream));
  }
  const int nsweeps = s->g.rank == 1 ? 1 : 2 * s->g.rank;
  int restarts = 0, committed = 0;
  bool stable_enqueued = piped;
  while (s->t < t_end) {
    FVS_CUDA(EnqueueStep(s, s->cur, s->cycle, 0, cons_host, stable_enqueued));
    stable_enqueued = false;  // a restart runs the whole step again
    FVS_CUDA(cudaMemcpyAsync(s->ctrl_host, s->ctrl, sizeof(fvs::Control),
                             cudaMemcpyDeviceToHost, s->stream));
    FVS_CUDA(cudaStreamSynchronize(s->stream));
    const fvs::Control& h = *s->ctrl_host;
    if (h.steps_done > 0) {
      s->cur = NextBuffer(s->cur, nsweeps);
      s->cycle += 1;
      s->t = h.t;
      committed = 1;
      break;
    }
    if (!h.abort) break;
    // a failed per-sweep check: the step is redone from its start buffer with
    // the failing sweep's dt (its downloads are overwritten by the redo)
    if (++restarts > 64) return Fail(FVS_ERR_STATE, "step restarted 64 times");
    const int zero = 0;
    FVS_CUDA(cudaMemcpyAsync(&s->ctrl->abort, &zero, sizeof zero, cudaMemcpyHostToDevice,
                             s->stream));
  }
  FVS_CUDA(cudaStreamSynchronize(s->stream));
  const fvs::Control& h = *s->ctrl_host;
  if (stats) {
    stats->time = s->t;
    stats->steps = committed;
    stats->restarts = restarts;
    stats->status = committed ? h.status : 0;
    stats->last_dt = committed ? h.dt : 0.0;
  }
  if (committed && (h.status & fvs::kStatusCopyTimeout))
    return Fail(FVS_ERR_CUDA, "a staged copy of a sweep did not land in time");
  if (committed && h.status) return Fail(FVS_ERR_STATE, "non-positive density encountered");
  return FVS_OK;
}

int fvs_solver_run(fvs_solver* s, double cfl, double t_end, int max_steps,
                   double* dt_log, int dt_log_len, fvs_run_stats* stats) {
  if (!s) return Fail(FVS_ERR_INVALID, "NULL solver");
  if (!(cfl > 0.0)) return Fail(FVS_ERR_INVALID, "cfl must be positive");
  if (dt_log_len < 0 || (dt_log_len > 0 && !dt_log))
    return Fail(FVS_ERR_INVALID, "bad dt log");
  if (dt_log_len > s->dt_log_cap) {
    FVS_CUDA(cudaStreamSynchronize(s->stream));
    if (s->dt_log_dev) cudaFree(s->dt_log_dev);
    s->dt_log_dev = nullptr;
    FVS_CUDA(cudaMalloc(&s->dt_log_dev, size_t(dt_log_len) * sizeof(double)));
    s->dt_log_cap = dt_log_len;
    for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
    s->graphs.clear();
  }
  fvs::Control c{};
  c.t = s->t;
  c.t_end = t_end;
  c.cfl = cfl;
  FVS_CUDA(cudaMemcpyAsync(s->ctrl, &c, sizeof c, cudaMemcpyHostToDevice, s->stream));
  int committed = 0;
  int restarts = 0;
  const int nsweeps = s->g.rank == 1 ? 1 : 2 * s->g.rank;
  const int kBatch = 3;          // steps per graph (buffer rotation period)
  const int kChunk = 10 * kBatch;  // steps enqueued between host checks
  bool done = false;
  while (!done && (max_steps < 0 || committed < max_steps)) {
    int chunk = kChunk;
    if (max_steps >= 0) chunk = std::min(chunk, max_steps - committed);
    // Enqueue `chunk` steps assuming they all commit; a failed check or the
    // end time makes the remaining kernels return without touching state.
    int cur = s->cur;
    int64_t cycle = s->cycle;
    int enq = 0;
    while (enq < chunk) {
      const int batch = std::min(kBatch, chunk - enq);
      const auto key = std::make_tuple(cur, static_cast<int>(cycle % 2), batch);
      auto it = s->graphs.find(key);
      if (it == s->graphs.end()) {
        cudaGraph_t graph;
        FVS_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        int b = cur;
        cudaError_t e = cudaSuccess;
        for (int q = 0; q < batch && e == cudaSuccess; ++q) {
          e = EnqueueStep(s, b, cycle + q, q);
          b = NextBuffer(b, nsweeps);
        }
        cudaError_t e2 = cudaStreamEndCapture(s->stream, &graph);
        if (e != cudaSuccess) return CudaFail(e, "capture split step");
        if (e2 != cudaSuccess) return CudaFail(e2, "cudaStreamEndCapture");
        cudaGraphExec_t exec;
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return CudaFail(e, "cudaGraphInstantiate");
        it = s->graphs.emplace(key, exec).first;
      }
      FVS_CUDA(cudaGraphLaunch(it->second, s->stream));
      for (int q = 0; q < batch; ++q) cur = NextBuffer(cur, nsweeps);
      cycle += batch;
      enq += batch;
    }
    FVS_CUDA(cudaMemcpyAsync(s->ctrl_host, s->ctrl, sizeof(fvs::Control),
                             cudaMemcpyDeviceToHost, s->stream));
    FVS_CUDA(cudaStreamSynchronize(s->stream));
    const fvs::Control& h = *s->ctrl_host;
    const int new_steps = h.steps_done - committed;
    for (int q = 0; q < new_steps; ++q) s->cur = NextBuffer(s->cur, nsweeps);
    s->cycle += new_steps;
    committed = h.steps_done;
    s->t = h.t;
    if (h.abort) {
      ++restarts;
      const int zero = 0;
      FVS_CUDA(cudaMemcpyAsync(&s->ctrl->abort, &zero, sizeof zero,
                               cudaMemcpyHostToDevice, s->stream));
      continue;
    }
    if (h.done) done = true;
  }
  if (dt_log && committed > 0) {
    const int n = std::min(committed, dt_log_len);
    FVS_CUDA(cudaMemcpyAsync(dt_log, s->dt_log_dev, n * sizeof(double),
                             cudaMemcpyDeviceToHost, s->stream));
  }
  FVS_CUDA(cudaStreamSynchronize(s->stream));
  const fvs::Control& h = *s->ctrl_host;
  if (stats) {
    stats->time = h.t;
    stats->steps = committed;
    stats->restarts = restarts;
    stats->status = h.status;
    stats->last_dt = h.dt;
  }
  if (h.status & fvs::kStatusCopyTimeout)
    return Fail(FVS_ERR_CUDA, "a staged copy of a sweep did not land in time");
  if (h.status) return Fail(FVS_ERR_STATE, "non-positive density encountered");
  return FVS_OK;
}

}  // extern "C"
