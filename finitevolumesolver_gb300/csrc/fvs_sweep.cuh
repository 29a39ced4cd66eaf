// fvs_sweep.cuh -- the fused directional sweep of a uniform grid.
//
// One pass per sweep does what the reference does in four:
//   ComputeStableDt(level, dir)   (the per-sweep CFL check, on the input)
//   ComputeNumericFluxes          (MUSCL-Hancock + HLLE)
//   UpdateConservatively          (U' = U + dt/dx (F_L - F_R))
//   CompleteFromCons              (p and c are recomputed where needed)
// (include/fub/solver/DimensionalSplitLevelIntegrator.hpp:227-263).
//
// Layout: conservative state, component-major, x fastest, no ghost cells.
// Ghost values are the boundary condition's images (periodic wrap or the
// boundary cell for transmissive), read directly from the interior.
//
// Thread mapping: one thread owns one grid line along the sweep direction
// (or a segment of it) and marches along it, keeping the 3-cell window, the
// previous face state, the previous face flux and the previous cell's wave
// data in registers.  Consecutive threads own neighbouring lines: for y/z
// sweeps these are x-neighbours, so every load and store instruction of a
// warp touches 32 consecutive doubles.  Each cell's MUSCL predictor is
// evaluated once (the reference evaluates it for both faces of the cell).
#pragma once

#include "fvs_internal.h"

namespace fvs {

__device__ __forceinline__ int BcIndex(int j, int n, int bc) {
  if (j >= 0 && j < n) return j;
  if (bc == 0) {
    int r = j % n;
    return r < 0 ? r + n : r;
  }
  return j < 0 ? 0 : n - 1;
}

__device__ __forceinline__ void AtomicMaxPositive(unsigned long long* word,
                                                  double v) {
  // Non-negative doubles order like their bit patterns.
  atomicMax(word, static_cast<unsigned long long>(__double_as_longlong(v)));
}

__device__ __forceinline__ double WarpMax(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

__device__ __forceinline__ double BitsToDouble(unsigned long long b) {
  return __longlong_as_double(static_cast<long long>(b));
}

// Returns false when this sweep must not run (run aborted / finished, or the
// previous sweep's CFL check failed).
__device__ __forceinline__ bool SweepGate(const SweepArgs& a, double split_dt) {
  if (a.ctrl) {
    if (a.ctrl->abort || a.ctrl->done) return false;
    if (a.prev_check >= 0) {
      const double smax = BitsToDouble(a.ctrl->smax_check[a.prev_check]);
      const double level_dt = a.prev_dx / smax;
      if (level_dt < split_dt) return false;
    }
  }
  return true;
}

// Counters of the exact Riemann solver (Newton iterations, faces whose
// Newton iteration did not converge); empty for the HLLE policies.
struct NoStats {
  __device__ __forceinline__ void Flush(unsigned long long*) const {}
};

struct NewtonStats {
  unsigned long long iterations = 0;
  unsigned long long failures = 0;
  __device__ __forceinline__ void Flush(unsigned long long* out) const {
    unsigned long long it = iterations, fl = failures;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      it += __shfl_xor_sync(0xffffffffu, it, o);
      fl += __shfl_xor_sync(0xffffffffu, fl, o);
    }
    if (out && (threadIdx.x & 31) == 0) {
      if (it) atomicAdd(out, it);
      if (fl) atomicAdd(out + 1, fl);
    }
  }
};

// Policy P = PT<D> provides: Real (compute precision), Gas, Rec (face
// state), Wave (cell wave data), Stats, MakeGas(), ToCell() (double ->
// Real), Predict(), MakeWave(), and Face(): the numeric flux of the face
// between recR of the left cell and recL of the right cell (as double) and
// the face's max signal speed of the input state (the CFL check).
template <int D, int DIR, template <int> class PT>
__global__ void __launch_bounds__(128) SweepMarchKernel(SweepArgs a) {
  using P = PT<D>;
  constexpr int K = D + 2;
  const int nx = a.n[0], ny = a.n[1], nz = a.n[2];
  const int nd = a.n[DIR];
  const int64_t cs = int64_t(nx) * ny * nz;  // component stride
  int64_t ntrans;
  if (DIR == 0) ntrans = int64_t(ny) * nz;
  else if (DIR == 1) ntrans = int64_t(nx) * nz;
  else ntrans = int64_t(nx) * ny;
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int j0 = blockIdx.y * a.seg_len;
  const int j1 = min(nd, j0 + a.seg_len);

  const double split_dt = a.dt_ptr ? a.dt_scale * (*a.dt_ptr) : a.dt_value;
  if (!SweepGate(a, split_dt)) return;
  const bool active = t < ntrans;

  int64_t base, stride;
  if (DIR == 0) {
    base = t * nx;
    stride = 1;
  } else if (DIR == 1) {
    const int64_t i = t % nx, k = t / nx;
    base = k * int64_t(nx) * ny + i;
    stride = nx;
  } else {
    base = t;
    stride = int64_t(nx) * ny;
  }

  const typename P::Gas eq = P::MakeGasFor(a);
  const double lambda_half = 0.5 * split_dt / a.dx;
  const double dt_dx = split_dt / a.dx;

  using R = typename P::Real;
  R smax = R(0);
  int status = 0;
  typename P::Stats stats;
  if (active) {
    const double* __restrict__ in = a.in;
    double* __restrict__ out = a.out;
    auto load = [&](double* u, int j) {
      const int64_t off = base + int64_t(BcIndex(j, nd, a.bc)) * stride;
#pragma unroll
      for (int c = 0; c < K; ++c) u[c] = __ldg(in + c * cs + off);
    };
    // double window for the update, compute-precision window for the rest
    double dm[K], dc[K], dp[K];
    R cm[K], cc[K], cp[K];
    load(dm, j0 - 2);
    load(dc, j0 - 1);
    P::ToCell(cm, dm);
    P::ToCell(cc, dc);
    typename P::Rec recR_prev;
    typename P::Wave w_prev;
    double F_prev[K];
    for (int j = j0 - 1; j <= j1; ++j) {
      load(dp, j + 1);
      P::ToCell(cp, dp);
      typename P::Rec recL, recR;
      P::Predict(eq, recL, recR, cm, cc, cp, a.limiter, lambda_half, DIR);
      const typename P::Wave w = P::MakeWave(eq, cc, DIR);
      if (j >= j0) {
        double F[K];
        const R s = P::Face(eq, F, recR_prev, recL, w_prev, w, DIR, stats);
        smax = s > smax ? s : smax;
        if (j > j0) {
          // cell j-1: U' = U + dt/dx (F_{j-1} - F_j)
          const int64_t off = base + int64_t(j - 1) * stride;
#pragma unroll
          for (int c = 0; c < K; ++c) {
            const double v = dm[c] + dt_dx * (F_prev[c] - F[c]);
            out[c * cs + off] = v;
            // non-positive density: sign bit set or zero (integer test)
            if (c == 0 && __double_as_longlong(v) <= 0) status |= kStatusNonPositiveDensity;
          }
        }
#pragma unroll
        for (int c = 0; c < K; ++c) F_prev[c] = F[c];
      }
      recR_prev = recR;
      w_prev = w;
#pragma unroll
      for (int c = 0; c < K; ++c) {
        dm[c] = dc[c];
        dc[c] = dp[c];
        cm[c] = cc[c];
        cc[c] = cp[c];
      }
    }
  }
  stats.Flush(a.stats_out);
  const double smax_w = WarpMax(static_cast<double>(smax));
  if ((threadIdx.x & 31) == 0) {
    if (a.smax_out && smax_w > 0.0) AtomicMaxPositive(a.smax_out, smax_w);
  }
  if (status && a.ctrl) atomicOr(&a.ctrl->step_status, status);
}

template <int D, template <int> class P>
cudaError_t LaunchSweepT(const SweepArgs& a, cudaStream_t s) {
  const int nd = a.n[a.dir];
  int64_t ntrans = 1;
  for (int d = 0; d < 3; ++d)
    if (d != a.dir) ntrans *= a.n[d];
  const int block = 128;
  const int seg = a.seg_len > 0 ? a.seg_len : nd;
  SweepArgs b = a;
  b.seg_len = seg;
  dim3 grid(static_cast<unsigned>((ntrans + block - 1) / block),
            static_cast<unsigned>((nd + seg - 1) / seg));
  switch (a.dir) {
  case 0:
    SweepMarchKernel<D, 0, P><<<grid, block, 0, s>>>(b);
    break;
  case 1:
    if constexpr (D >= 2) SweepMarchKernel<D, 1, P><<<grid, block, 0, s>>>(b);
    break;
  default:
    if constexpr (D >= 3) SweepMarchKernel<D, 2, P><<<grid, block, 0, s>>>(b);
    break;
  }
  return cudaGetLastError();
}

}  // namespace fvs
