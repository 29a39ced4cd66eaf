// fvs_amr_kernels.cuh -- kernels of the batched AMR patch update (2-D).
//
// PatchSweepKernel: one persistent launch per level and sweep.  Each thread
// takes segments of the level's rows (grid-stride) and marches along them
// with the same three-cell window, policy arithmetic and update as the
// uniform grid's SweepMarchKernel (fvs_sweep.cuh): for a segment [j0, j1) of
// a row it reads the ghosted cells j0-2..j1+1 of the input buffer, computes
// the faces j0..j1, writes the updated cells j0..j1-1 to the output buffer,
// accumulates dt_split * F into the flux-register entries of the row's
// captured faces (each entry belongs to exactly one face, so no atomics and
// a deterministic sum) and reduces the row's max signal speed for the
// per-sweep CFL check.  The halo cells at the ends of a row are read where
// they live (Seg::halo): the same level's current buffer or the coarser
// level, which is the ghost fill of those strips at sweep time.
//
// For EinfeldtCfl policies (exact and fast FP64) both kernels screen the CFL
// speeds in FP32 as the uniform sweeps do (fvs_sweep.cuh): a face's exact
// speed is evaluated only when its FP32 speed plus error bound reaches the
// thread's threshold.  The rows of a warp can differ in length, so the
// decisions are per thread (no warp votes); the threshold is the thread's own
// maximum and the launch's max slot, read at every segment start, and a
// thread publishes its maximum at a segment end when it exceeds the slot
// value it read.  The maxima are the same numbers, bit for bit; the max slots
// must start at zero (or at an exact speed of the same sweep).
#pragma once

#include <climits>

#include "fvs_amr.h"
#include "fvs_sweep.cuh"

namespace fvs {
namespace amr {

template <int DIR, template <int> class PT>
__global__ void __launch_bounds__(128, PT<2>::kMinBlocks) PatchSweepKernel(PatchSweepArgs a) {
  using P = PT<2>;
  using R = typename P::Real;
  constexpr int K = kComp;
  const double split_dt = a.dt_scale * (*a.dt_ptr);
  const typename P::Gas eq = P::MakeGas(a.gamma);
  const double lambda_half = 0.5 * split_dt / a.dx;
  const double dt_dx = split_dt / a.dx;
  const int64_t N = a.ncells;
  const double* __restrict__ in = a.in;
  double* __restrict__ out = a.out;
  R smax = R(0);
  int status = 0;
  typename P::Stats stats;
  constexpr bool kFilter = EinfeldtCfl<P>::value && HasFluxOnly<P>::value;
  const bool screen = kFilter && a.gamma > 1.0 && a.gamma <= 2.0;
  fast::Gas<float> g32;
  g32.gamma = static_cast<float>(a.gamma);
  g32.gm1 = static_cast<float>(a.gamma - 1.0);
  float thr = 0.0f;
  unsigned long long known = 0;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < a.nsegs;
       r += gridDim.x * blockDim.x) {
    const Seg w = a.segs[r];
    if constexpr (kFilter) {
      known = *reinterpret_cast<volatile unsigned long long*>(a.smax_out);
      thr = fmaxf(thr, CflFloatBelow(__longlong_as_double(static_cast<long long>(known))));
    }
    int cap = w.cap_begin;
    int next_face = cap < w.cap_end ? a.caps[cap].face : INT_MAX;
    const int j0 = w.j0, j1 = w.j1;
    // returns whether the cell is a reflective boundary's image, whose
    // momentum along the row the caller negates after the conversion (so the
    // prefetched load is not waited for early)
    auto load = [&](double* u, int j) -> bool {
      const double* src = in;
      int64_t off, cs = N;
      bool flip = false;
      if (j >= 0 && j < w.n) {
        off = int64_t(w.base) + int64_t(j + kGhost) * w.stride;
      } else {  // halo cell: its source in this level or the coarser one
        const int h = j < 0 ? j + 2 : j - w.n + 2;
        const int32_t g = w.halo[h];
        if (g >= 0) {
          off = g;
        } else {
          off = -int64_t(g) - 1;
          src = a.coarse;
          cs = a.coarse_ncells;
        }
        flip = (w.flip >> h) & 1;
      }
#pragma unroll
      for (int c = 0; c < K; ++c) u[c] = __ldg(src + c * cs + off);
      return flip;
    };
    // the update re-reads the FP64 state of cell j-1 (an L1 hit) instead of
    // carrying a window of FP64 states in registers
    double dn[K];
    R cm[K], cc[K], cp[K];
    const bool flip_cm = load(dn, j0 - 2);
    P::ToCell(cm, dn);
    if (flip_cm) cm[1 + DIR] = -cm[1 + DIR];
    const bool flip_cc = load(dn, j0 - 1);
    P::ToCell(cc, dn);
    if (flip_cc) cc[1 + DIR] = -cc[1 + DIR];
    bool flip_dn = load(dn, j0);
    using FluxT = typename FluxOf<P>::type;
    typename P::Rec recR_prev;
    typename P::Wave w_prev;
    FluxT F_prev[K];
    fast::Wave<float> v_prev{};
    bool ok_prev = false;
    bool have_prev = false;  // w_prev holds the exact wave of cell j-1
    for (int j = j0 - 1; j <= j1; ++j) {
      if constexpr (kFilter) {
        float c32[K];
#pragma unroll
        for (int c = 0; c < K; ++c) c32[c] = CflToF32(cc[c]);
        const fast::Wave<float> v = fast::MakeWave<2, float>(g32, c32, DIR);
        const bool ok = screen && CflInRange<2>(c32) && v.a > 0.0f;
        if (j >= j0) {
          const float s32 = fast::FaceMaxSpeed<float>(g32, v_prev, v);
          const float sh = fast::Math<float>::Sqrt(fmaxf(v_prev.h, v.h));
          const float bound = fmaf(s32, kCflRel, fmaf(kCflScale, sh, kCflAbs));
          if (!(ok && ok_prev && bound < thr)) {
            const typename P::Wave wl = have_prev ? w_prev : P::MakeWave(eq, cm, DIR);
            w_prev = P::MakeWave(eq, cc, DIR);
            const R s = P::FaceMaxSpeed(eq, wl, w_prev);
            smax = s > smax ? s : smax;
            thr = fmaxf(thr, CflFloatBelow(static_cast<double>(smax)));
            have_prev = true;
          } else {
            have_prev = false;
          }
        }
        ok_prev = ok;
        v_prev = v;
      }
      P::ToCell(cp, dn);
      if (flip_dn) cp[1 + DIR] = -cp[1 + DIR];  // a reflective boundary's image
      if (j + 2 <= j1 + 1) flip_dn = load(dn, j + 2);
      typename P::Rec recL, recR;
      P::Predict(eq, recL, recR, cm, cc, cp, a.limiter, lambda_half, DIR);
      typename P::Wave wv{};
      if constexpr (!kFilter) wv = P::MakeWave(eq, cc, DIR);
      if (j >= j0) {
        FluxT F[K];
        if constexpr (kFilter) {
          SweepFluxOnly<P>(eq, F, recR_prev, recL, DIR);
        } else {
          const R s = SweepFace<P>(eq, F, recR_prev, recL, w_prev, wv, DIR, stats);
          smax = s > smax ? s : smax;
        }
        if (j == next_face) {
          double* dst = a.reg + int64_t(a.caps[cap].dst) * K;
#pragma unroll
          for (int c = 0; c < K; ++c) dst[c] = dst[c] + split_dt * FluxWiden(F[c]);
          ++cap;
          next_face = cap < w.cap_end ? a.caps[cap].face : INT_MAX;
        }
        if (j > j0) {
          const int64_t off = int64_t(w.base) + int64_t(j - 1 + kGhost) * w.stride;
#pragma unroll
          for (int c = 0; c < K; ++c) {
            const double v = __ldg(in + c * N + off) + dt_dx * FluxDiff(F_prev[c], F[c]);
            out[c * N + off] = v;
            if (c == 0 && __double_as_longlong(v) <= 0) status |= kStatusNonPositiveDensity;
          }
        }
#pragma unroll
        for (int c = 0; c < K; ++c) F_prev[c] = F[c];
      }
      recR_prev = recR;
      if constexpr (!kFilter) w_prev = wv;
#pragma unroll
      for (int c = 0; c < K; ++c) {
        cm[c] = cc[c];
        cc[c] = cp[c];
      }
    }
    if constexpr (kFilter) {
      const unsigned long long b =
          static_cast<unsigned long long>(__double_as_longlong(static_cast<double>(smax)));
      if (b > known) atomicMax(a.smax_out, b);
    }
  }
  const double smax_d = static_cast<double>(smax);
  BlockMaxAtomic<1>(a.smax_out, &smax_d);
  if (status) atomicOr(&a.ctrl->step_status, status);
}

// PatchRowWarpKernel: the x sweeps of the mixed flavour with the lanes of a
// warp along x.  The level's x rows are laid end to end as slots, n + 2 per
// row (cells -1..n); warp w takes slots 30w .. 30w + 31 (grid-stride).  Lane
// l holds the cell of slot 30w + l in the compute precision and gets its
// neighbours by shuffles, or loads them where the neighbour lies in another
// row (the halo cells -2 and n + 1) or outside the warp; it evaluates that
// cell's MUSCL predictor once, and lanes 1..31 the flux of the face on the
// cell's left.  Lanes 1..30 own their slots: they update interior cells
// (0 <= c < n) with the faces on both sides (the right one from the next
// lane), accumulate captured faces into the flux registers and fold their
// faces' signal speeds into the sweep's maximum.  Every predictor is
// evaluated once per row (plus those of cells -1 and n, which faces 0 and n
// need), where PatchSweepKernel's segments repeat two per segment and load
// four halo cells each, and a warp's loads of a row are consecutive.  The
// arithmetic per cell and face is PatchSweepKernel's: the results are the
// same, bit for bit.  Policies whose CFL speeds are FP32-screened (the FP64
// flavours) keep PatchSweepKernel.
template <template <int> class PT>
__global__ void __launch_bounds__(128, PT<2>::kMinBlocks) PatchRowWarpKernel(PatchSweepArgs a) {
  using P = PT<2>;
  using R = typename P::Real;
  constexpr int K = kComp;
  static_assert(!(EinfeldtCfl<P>::value && HasFluxOnly<P>::value),
                "screened-CFL policies use PatchSweepKernel");
  using Cell = CellArr<R, K>;
  using FluxT = typename FluxOf<P>::type;
  using Flx = CellArr<FluxT, K>;
  const double split_dt = a.dt_scale * (*a.dt_ptr);
  const typename P::Gas eq = P::MakeGas(a.gamma);
  const double lambda_half = 0.5 * split_dt / a.dx;
  const double dt_dx = split_dt / a.dx;
  const int64_t N = a.ncells;
  const double* __restrict__ in = a.in;
  double* __restrict__ out = a.out;
  const int lane = threadIdx.x & 31;
  R smax = R(0);
  int status = 0;
  typename P::Stats stats;
  const int64_t nwarps = a.nslots > 1 ? (a.nslots - 1 + kRowWarpStep - 1) / kRowWarpStep : 0;
  const int64_t wstride = (int64_t(gridDim.x) * blockDim.x) >> 5;
  for (int64_t w = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; w < nwarps;
       w += wstride) {
    const int64_t s = w * kRowWarpStep + lane;
    const bool valid = s < a.nslots;
    Seg row{};
    int c = 0;
    if (valid) {
      const int32_t r = a.slot_row[s];
      row = a.segs[r];
      c = static_cast<int>(s - a.row_slot0[r]) - 1;
    }
    // cell x (-2..n+1) of the slot's row: interior, or a halo cell where it
    // lives (this level or the coarser one, a reflective image flipped)
    auto load = [&](double* u, int x) {
      const double* src = in;
      int64_t off, cs = N;
      bool flip = false;
      if (x >= 0 && x < row.n) {
        off = int64_t(row.base) + x + kGhost;
      } else {
        const int h = x < 0 ? x + 2 : x - row.n + 2;
        const int32_t g = row.halo[h];
        if (g >= 0) {
          off = g;
        } else {
          off = -int64_t(g) - 1;
          src = a.coarse;
          cs = a.coarse_ncells;
        }
        flip = (row.flip >> h) & 1;
      }
#pragma unroll
      for (int k = 0; k < K; ++k) u[k] = __ldg(src + k * cs + off);
      if (flip) u[1] = -u[1];
    };
    Cell C{}, Cm{}, Cp{};
    double u[K];
    if (valid) {
      load(u, c);
      P::ToCell(C.v, u);
    }
    const Cell up = ShflUp(C, 1), down = ShflDown(C, 1);
    if (valid) {
      if (c == -1 || lane == 0) {
        load(u, c - 1);
        P::ToCell(Cm.v, u);
      } else {
        Cm = up;
      }
      if (c == row.n || lane == 31) {
        load(u, c + 1);
        P::ToCell(Cp.v, u);
      } else {
        Cp = down;
      }
    }
    typename P::Rec recL, recR;
    P::Predict(eq, recL, recR, Cm.v, C.v, Cp.v, a.limiter, lambda_half, 0);
    const typename P::Wave W = P::MakeWave(eq, C.v, 0);
    const typename P::Rec recRm = ShflUp(recR, 1);
    const typename P::Wave Wm = ShflUp(W, 1);
    // face c (cells c-1 and c)
    Flx F{};
    R sp = R(0);
    if (valid && lane >= 1 && c >= 0) sp = SweepFace<P>(eq, F.v, recRm, recL, Wm, W, 0, stats);
    const Flx Fr = ShflDown(F, 1);  // face c + 1
    const bool own = valid && lane >= 1 && lane <= kRowWarpStep && c >= 0;
    if (own) {
      smax = sp > smax ? sp : smax;
      for (int q = row.cap_begin; q < row.cap_end; ++q) {
        const Cap cp = a.caps[q];
        if (cp.face != c) continue;
        double* dst = a.reg + int64_t(cp.dst) * K;
#pragma unroll
        for (int k = 0; k < K; ++k) dst[k] = dst[k] + split_dt * FluxWiden(F.v[k]);
      }
      if (c < row.n) {
        const int64_t off = int64_t(row.base) + c + kGhost;
#pragma unroll
        for (int k = 0; k < K; ++k) {
          const double v = __ldg(in + k * N + off) + dt_dx * FluxDiff(F.v[k], Fr.v[k]);
          out[k * N + off] = v;
          if (k == 0 && __double_as_longlong(v) <= 0) status |= kStatusNonPositiveDensity;
        }
      }
    }
  }
  const double smax_d = static_cast<double>(smax);
  BlockMaxAtomic<1>(a.smax_out, &smax_d);
  if (status) atomicOr(&a.ctrl->step_status, status);
}

template <template <int> class PT>
cudaError_t LaunchPatchRowWarpT(const PatchSweepArgs& a, int grid, int block, cudaStream_t s) {
  if (a.nslots == 0) return cudaSuccess;
  PatchRowWarpKernel<PT><<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

// Max signal speed over the faces 0..n of every row (the stable dt of the
// level in that direction is dx / max): a segment [j0, j1) of a row takes
// the faces j0..j1 (neighbouring segments share a face; the max does not
// mind), so short segments give every row several threads.
template <int DIR, template <int> class PT>
__global__ void __launch_bounds__(128) PatchMaxSpeedKernel(MaxSpeedArgs a) {
  using P = PT<2>;
  using R = typename P::Real;
  constexpr int K = kComp;
  const typename P::Gas eq = P::MakeGas(a.gamma);
  const int64_t N = a.ncells;
  constexpr bool kFilter = EinfeldtCfl<P>::value;
  const bool screen = kFilter && a.gamma > 1.0 && a.gamma <= 2.0;
  fast::Gas<float> g32;
  g32.gamma = static_cast<float>(a.gamma);
  g32.gm1 = static_cast<float>(a.gamma - 1.0);
  float thr = 0.0f;
  unsigned long long known = 0;
  R smax = R(0);
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < a.nsegs;
       r += gridDim.x * blockDim.x) {
    const Seg w = a.segs[r];
    // loads cell j of the segment's row; returns whether it is a reflective
    // boundary's image, whose normal momentum `finish` negates after the
    // conversion (a select on the loaded value would wait for the load)
    auto fetch = [&](int j, double* u) {
      const double* src = a.in;
      int64_t off, cs = N;
      bool flip = false;
      if (j >= 0 && j < w.n) {
        off = int64_t(w.base) + int64_t(j + kGhost) * w.stride;
      } else {  // halo cell (j = -1 or n)
        const int h = j < 0 ? j + 2 : j - w.n + 2;
        const int32_t g = w.halo[h];
        if (g >= 0) {
          off = g;
        } else {
          off = -int64_t(g) - 1;
          src = a.coarse;
          cs = a.coarse_ncells;
        }
        flip = (w.flip >> h) & 1;
      }
#pragma unroll
      for (int c = 0; c < K; ++c) u[c] = __ldg(src + c * cs + off);
      return flip;
    };
    auto finish = [&](const double* u, bool flip, R* v) {
      P::ToCell(v, u);
      if (flip) v[1 + DIR] = -v[1 + DIR];
    };
    // the cells j0 - 1 .. j1 of faces j0 .. j1, each loaded one face before
    // its use: shift(f, v) hands out cell f - 1 and fetches cell f
    double un[K];
    bool fn = fetch(w.j0 - 1, un);
    auto shift = [&](int f, R* v) {
      double uc[K];
#pragma unroll
      for (int c = 0; c < K; ++c) uc[c] = un[c];
      const bool fc = fn;
      if (f <= w.j1) fn = fetch(f, un);
      finish(uc, fc, v);
    };
    if constexpr (kFilter) {
      known = *reinterpret_cast<volatile unsigned long long*>(a.smax_out);
      thr = fmaxf(thr, CflFloatBelow(__longlong_as_double(static_cast<long long>(known))));
      // FP32 screen (see the file comment): the exact waves of a face only
      // when its bound reaches the threshold
      auto screen_wave = [&](const R* u, bool& ok) {
        float c32[K];
#pragma unroll
        for (int c = 0; c < K; ++c) c32[c] = CflToF32(u[c]);
        const fast::Wave<float> v = fast::MakeWave<2, float>(g32, c32, DIR);
        ok = screen && CflInRange<2>(c32) && v.a > 0.0f;
        return v;
      };
      R ul[K];
      shift(w.j0, ul);
      bool ok_l;
      fast::Wave<float> vl = screen_wave(ul, ok_l);
      typename P::Wave wl;
      bool have_l = false;
      for (int f = w.j0; f <= w.j1; ++f) {
        R ur[K];
        shift(f + 1, ur);
        bool ok_r;
        const fast::Wave<float> vr = screen_wave(ur, ok_r);
        const float s32 = fast::FaceMaxSpeed<float>(g32, vl, vr);
        const float sh = fast::Math<float>::Sqrt(fmaxf(vl.h, vr.h));
        const float bound = fmaf(s32, kCflRel, fmaf(kCflScale, sh, kCflAbs));
        if (!(ok_l && ok_r && bound < thr)) {
          if (!have_l) wl = P::MakeWave(eq, ul, DIR);
          const typename P::Wave wr = P::MakeWave(eq, ur, DIR);
          const R s = P::FaceMaxSpeed(eq, wl, wr);
          smax = s > smax ? s : smax;
          thr = fmaxf(thr, CflFloatBelow(static_cast<double>(smax)));
          wl = wr;
          have_l = true;
        } else {
          have_l = false;
        }
#pragma unroll
        for (int c = 0; c < K; ++c) ul[c] = ur[c];
        vl = vr;
        ok_l = ok_r;
      }
      const unsigned long long b =
          static_cast<unsigned long long>(__double_as_longlong(static_cast<double>(smax)));
      if (b > known) atomicMax(a.smax_out, b);
    } else {
      auto wave = [&](int f) {
        R v[K];
        shift(f, v);
        return P::MakeWave(eq, v, DIR);
      };
      typename P::Wave wl = wave(w.j0);
      for (int f = w.j0; f <= w.j1; ++f) {
        const typename P::Wave wr = wave(f + 1);
        const R s = P::FaceMaxSpeed(eq, wl, wr);
        smax = s > smax ? s : smax;
        wl = wr;
      }
    }
  }
  const double smax_d = static_cast<double>(smax);
  BlockMaxAtomic<1>(a.smax_out, &smax_d);
}

template <template <int> class PT>
cudaError_t LaunchPatchSweepT(int dir, const PatchSweepArgs& a, int grid, int block,
                              cudaStream_t s) {
  if (a.nsegs == 0) return cudaSuccess;
  if (dir == 0)
    PatchSweepKernel<0, PT><<<grid, block, 0, s>>>(a);
  else
    PatchSweepKernel<1, PT><<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

template <template <int> class PT>
cudaError_t LaunchPatchMaxSpeedT(int dir, const MaxSpeedArgs& a, int grid, int block,
                                 cudaStream_t s) {
  if (a.nsegs == 0) return cudaSuccess;
  if (dir == 0)
    PatchMaxSpeedKernel<0, PT><<<grid, block, 0, s>>>(a);
  else
    PatchMaxSpeedKernel<1, PT><<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace amr
}  // namespace fvs
