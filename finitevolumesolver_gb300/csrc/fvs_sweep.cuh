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

#include <type_traits>

#include "fvs_convert.cuh"
#include "fvs_internal.h"
#include "fvs_physics_fast.cuh"
#include "fvs_tma.cuh"

#include <cstring>

namespace fvs {

// The interior cell whose state ghost cell j of a grid line of n cells
// images under boundary condition bc (FVS_BC_*): periodic -- the periodic
// image; transmissive -- the boundary cell (TransmissiveBoundary.cpp:31-42);
// reflective -- the mirror cell (ReflectIndex,
// src/boundary_condition/ReflectiveBoundary.cpp:24-36; needs n >= 2 for the
// two ghost layers), whose momentum along the line is reflected (BcFlip).
__device__ __forceinline__ int BcIndex(int j, int n, int bc) {
  if (j >= 0 && j < n) return j;
  if (bc == 0) {
    int r = j % n;
    return r < 0 ? r + n : r;
  }
  if (bc == 2) return j < 0 ? -1 - j : 2 * n - 1 - j;
  return j < 0 ? 0 : n - 1;
}

// Whether ghost cell j's state is the reflected image of BcIndex(j, n, bc):
// Reflect (src/equations/PerfectGas.cpp:266-300) with the unit normal of the
// line, m - 2 (m . e) e, negates the momentum along the line and keeps the
// other components.
__device__ __forceinline__ bool BcFlip(int j, int n, int bc) {
  return bc == 2 && (j < 0 || j >= n);
}

__device__ __forceinline__ void AtomicMaxPositive(unsigned long long* word,
                                                  double v) {
  // Non-negative doubles order like their bit patterns.
  atomicMax(word, static_cast<unsigned long long>(__double_as_longlong(v)));
}

// Max over a warp of non-negative face speeds.  A NaN speed (a state of
// negative pressure) counts as 0, so it is skipped wherever it sits: without
// the guard a NaN in lane 0 would survive the butterfly there (NaN > x and
// x > NaN are both false) and discard the other 31 lanes' maxima.
__device__ __forceinline__ double WarpMax(double v) {
  v = v > 0.0 ? v : 0.0;
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

// True on every thread of the block iff `pred` holds on every thread of it:
// a kernel that returns on !BlockAll(...) leaves no thread of a block behind
// a later barrier.
__device__ __forceinline__ bool BlockAll(bool pred) { return __syncthreads_and(pred) != 0; }

// Max over the thread block of per-thread values v[0..N) (each >= 0), then
// one atomic max per word and block (words may be NULL).  Every thread of
// the block calls it exactly once per kernel; one atomic per block instead
// of one per warp keeps the same-address atomic traffic small.
template <int N>
__device__ __forceinline__ void BlockMaxAtomic(unsigned long long* words, const double* v) {
  __shared__ double part[N][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int d = 0; d < N; ++d) {
    const double m = WarpMax(v[d]);
    if (lane == 0) part[d][warp] = m;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int d = 0; d < N; ++d) {
      double m = lane < nw ? part[d][lane] : 0.0;
      m = WarpMax(m);
      if (lane == 0 && words && m > 0.0) AtomicMaxPositive(words + d, m);
    }
  }
}

// Blocks of a grid-stride launch over `work` items: enough to fill every SM
// `per_sm` times, no more than the work needs.
inline unsigned GridStrideBlocks(int64_t work, int block, int per_sm) {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && n > 0)
      sms = n;
    else
      sms = 152;
  }
  const int64_t need = (work + block - 1) / block;
  const int64_t cap = int64_t(sms) * per_sm;
  return static_cast<unsigned>(need < cap ? (need > 0 ? need : 1) : cap);
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

// Policies whose face fluxes are computed in FP32 (the mixed flavour) hand
// them to the sweep in FP32 (kFloatFlux); all others in FP64.
template <class P, class = void> struct FluxOf {
  using type = double;
};
template <class P> struct FluxOf<P, std::enable_if_t<P::kFloatFlux>> {
  using type = float;
};

template <class P> using FluxOfArg = typename FluxOf<P>::type;

template <class P, class F>
__device__ __forceinline__ typename P::Real SweepFace(const typename P::Gas& eq, F* flux,
                                                      const typename P::Rec& L,
                                                      const typename P::Rec& R,
                                                      const typename P::Wave& wL,
                                                      const typename P::Wave& wR, int dir,
                                                      typename P::Stats& stats) {
  if constexpr (std::is_same_v<F, float>) {
    return P::FaceR(eq, flux, L, R, wL, wR, dir, stats);
  } else {
    return P::Face(eq, flux, L, R, wL, wR, dir, stats);
  }
}

// Policies that can compute a face flux without its CFL speed (FluxOnly):
// the first sweep of a step then takes its input's face speeds from the
// stable-dt pass over the same state and skips the cell waves.
// (FP64-flux policies only: the mixed flavour's sweeps are bound by memory
// and its FP64 update, and the extra path would cost them registers.)
template <class P, class = void> struct HasFluxOnly : std::false_type {};
template <class P>
struct HasFluxOnly<P, std::void_t<decltype(&P::FluxOnly)>>
    : std::bool_constant<std::is_same_v<typename FluxOf<P>::type, double>> {};

template <class P, class F>
__device__ __forceinline__ void SweepFluxOnly(const typename P::Gas& eq, F* flux,
                                              const typename P::Rec& L,
                                              const typename P::Rec& R, int dir) {
  if constexpr (std::is_same_v<F, float>) {
    P::FluxOnlyR(eq, flux, L, R, dir);
  } else {
    P::FluxOnly(eq, flux, L, R, dir);
  }
}

// Filtered CFL maximum.  For policies whose CFL speed is the Einfeldt speed
// of the two cell states of a face (kEinfeldtCfl), a sweep evaluates that
// speed in the policy's arithmetic only on faces that can hold the sweep's
// maximum.  Every face first gets an FP32 speed s32 from the FP32-rounded
// states and a bound on its error:
//   |s - s32| <= s32 / 1024 + sqrt(max(h_L, h_R)) / 64 + 2^-24,
// h = (E + p) / rho.  The relative term covers the roundings and the
// approximate FP32 reciprocals and square roots; the h term covers the
// cancellations in p = (gamma - 1)(E - e_kin) and in the Roe sound speed,
// whose absolute errors are below sqrt(c eps h) with c eps < 1e-5 for
// 1 < gamma <= 2; the constant covers underflow.  The bound holds for cells
// with 2^-30 <= rho <= 2^30, |m| <= 2^30, |E| <= 2^40 and a positive FP32
// pressure (no FP32 overflow; underflow errors far below 2^-24); any other
// face is evaluated.  A face is skipped when s32 plus its error bound is
// below a threshold that is itself a lower bound of an evaluated face's
// exact speed (the lane's own maximum and the sweep's maximum published so
// far, rounded down to FP32), so every skipped face is strictly slower than
// an evaluated one and the sweep's maximum is the same number, bit for bit.
// Warps publish their maximum to the sweep's max slot every kCflSyncRows
// rows and read it back, so later blocks start with the maximum of earlier
// ones.  The slot must start at zero (or at an evaluated speed of the same
// sweep).
template <class P, class = void> struct EinfeldtCfl : std::false_type {};
template <class P>
struct EinfeldtCfl<P, std::enable_if_t<P::kEinfeldtCfl>> : std::true_type {};
template <class P, class = void> struct HllemCfl : std::false_type {};
template <class P> struct HllemCfl<P, std::enable_if_t<P::kHllemCfl>> : std::true_type {};
template <class P>
struct FilteredCfl : std::integral_constant<bool, EinfeldtCfl<P>::value || HllemCfl<P>::value> {};

// The FP32 estimates: Einfeldt speeds (fast::MakeWave / fast::FaceMaxSpeed)
// and the HLLEM stable-dt speed (Hllem<PerfectGas>: the Roe average over the
// full velocity, max(c_L, c_R) for both outer waves, no zero in the max).
// The HLLEM speed's errors have the same sources and form (roundings, and the
// cancellations in p and in roeH - |roeU|^2 / 2 <= roeH), so the same bound
// covers it.  V carries h and a for the bound and the range check.
template <int D> struct EinfeldtScreen {
  using V = fast::Wave<float>;
  static __device__ __forceinline__ V Wave(const fast::Gas<float>& g, const float* c, int dir) {
    return fast::MakeWave<D, float>(g, c, dir);
  }
  static __device__ __forceinline__ float Speed(const fast::Gas<float>& g, const V& l,
                                                const V& r, int) {
    return fast::FaceMaxSpeed<float>(g, l, r);
  }
};
template <int D> struct HllemScreen {
  struct V {
    float sq, h, a;
    float u[D];
  };
  static __device__ __forceinline__ V Wave(const fast::Gas<float>& g, const float* c, int) {
    using M = fast::Math<float>;
    V v;
    const float rs = M::Rsqrt(c[0]);
    const float ir = rs * rs;
    v.sq = c[0] * rs;
#pragma unroll
    for (int i = 0; i < D; ++i) v.u[i] = c[1 + i] * ir;
    const float ke = 0.5f * fast::SquaredNorm<D, float>(c + 1) * ir;
    const float p = (c[1 + D] - ke) * g.gm1;
    v.h = (c[1 + D] + p) * ir;
    v.a = M::Sqrt(g.gamma * p * ir);
    return v;
  }
  static __device__ __forceinline__ float Speed(const fast::Gas<float>& g, const V& l,
                                                const V& r, int dir) {
    using M = fast::Math<float>;
    const float oo = M::Rcp(l.sq + r.sq);
    const float wL = l.sq * oo, wR = r.sq * oo;
    float roeU[D];
    float sqN = 0.0f;
#pragma unroll
    for (int i = 0; i < D; ++i) {
      roeU[i] = fmaf(wL, l.u[i], wR * r.u[i]);
      sqN = fmaf(roeU[i], roeU[i], sqN);
    }
    const float roeH = fmaf(wL, l.h, wR * r.h);
    const float roeA = M::Sqrt(g.gm1 * fmaf(-0.5f, sqN, roeH));
    const float maxA = fmaxf(l.a, r.a);
    const float sL = fminf(l.u[dir] - maxA, roeU[dir] - roeA);
    const float sR = fmaxf(roeU[dir] + roeA, r.u[dir] + maxA);
    return fmaxf(fabsf(sL), fabsf(sR));
  }
};
template <class P, int D>
using CflScreen = std::conditional_t<HllemCfl<P>::value, HllemScreen<D>, EinfeldtScreen<D>>;

constexpr float kCflRel = 1.0f + 1.0f / 1024.0f;
constexpr float kCflScale = 1.0f / 64.0f;
constexpr float kCflAbs = 0x1p-24f;
constexpr int kCflSyncRows = 8;

template <class R> __device__ __forceinline__ float CflToF32(const R& x) {
  if constexpr (std::is_same_v<R, double>) {
    return DoubleToFloatBits(x);
  } else {
    return x.hi;  // double-float: its leading FP32 word
  }
}

// FP32 cell values inside the range of the error bound above.
template <int D> __device__ __forceinline__ bool CflInRange(const float* u) {
  bool ok = u[0] >= 0x1p-30f && u[0] <= 0x1p30f && fabsf(u[1 + D]) <= 0x1p40f;
#pragma unroll
  for (int d = 0; d < D; ++d) ok = ok && fabsf(u[1 + d]) <= 0x1p30f;
  return ok;
}

// An FP32 number not above x >= 0 (x rounded to nearest, then lowered by
// more than the rounding; capped at 2^100 so that it stays finite).
__device__ __forceinline__ float CflFloatBelow(double x) {
  return fminf(DoubleToFloatBits(x) * (1.0f - 0x1p-22f), 0x1p100f);
}

// The warp's maximum of the lanes' `mine` (non-negative), folded into the
// sweep's max slot `slot` by one atomic of the first active lane; returns
// the slot's new value to every lane of `amask`.
__device__ __forceinline__ double CflSync(unsigned long long* slot, double mine,
                                          unsigned amask) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(mine));
  const unsigned bhi = static_cast<unsigned>(b >> 32);
  const unsigned mhi = __reduce_max_sync(amask, bhi);
  const unsigned mlo = __reduce_max_sync(amask, bhi == mhi ? static_cast<unsigned>(b) : 0u);
  const unsigned long long w = (static_cast<unsigned long long>(mhi) << 32) | mlo;
  const int leader = __ffs(amask) - 1;
  unsigned long long g = 0;
  if ((threadIdx.x & 31) == leader) g = atomicMax(slot, w);
  g = __shfl_sync(amask, g, leader);
  return __longlong_as_double(static_cast<long long>(g > w ? g : w));
}

// F_L - F_R in FP64 for the conservative update.  FP32 fluxes: the FP64
// difference formed on the FP32 and integer pipes (DiffToDouble: exact
// wherever the FP64 subtraction of the widened fluxes is exact), so the
// update costs one FP64 operation per component, the FMA with dt/dx.
__device__ __forceinline__ double FluxDiff(double a, double b) { return a - b; }
__device__ __forceinline__ double FluxDiff(float a, float b) { return DiffToDouble(a, b); }
__device__ __forceinline__ double FluxWiden(double a) { return a; }
__device__ __forceinline__ double FluxWiden(float a) { return FloatToDoubleBits(a); }

// Counters of the exact Riemann solver (Newton iterations, faces whose
// Newton iteration did not converge); empty for the HLLE policies.
struct NoStats {
  __device__ __forceinline__ void Flush(unsigned long long*) const {}
};

struct NewtonStats {
  unsigned long long iterations = 0;
  unsigned long long failures = 0;
  unsigned long long fallbacks = 0;
  __device__ __forceinline__ void Flush(unsigned long long* out) const {
    unsigned long long it = iterations, fl = failures, fb = fallbacks;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      it += __shfl_xor_sync(0xffffffffu, it, o);
      fl += __shfl_xor_sync(0xffffffffu, fl, o);
      fb += __shfl_xor_sync(0xffffffffu, fb, o);
    }
    if (out && (threadIdx.x & 31) == 0) {
      if (it) atomicAdd(out, it);
      if (fl) atomicAdd(out + 1, fl);
      if (fb) atomicAdd(out + 2, fb);
    }
  }
};

// The cells of one grid line of a marching sweep, read from global memory:
// Load gives cell j's conservative state (FP64; a ghost cell is the
// boundary condition's image) and returns whether the image's momentum
// along the line is to be negated (a reflective wall); the caller negates it
// after the conversion to the compute precision, so that the prefetched load
// is not waited for one iteration early.  CellRef gives an interior cell's
// components for the update; Advance is called at the start of every
// iteration (nothing to do here).
template <int K, int DIR> struct GlobalLine {
  const double* __restrict__ in;
  int64_t base, stride, cs;  // stride: cells between neighbours (1 in x)
  int nd, bc;
  __device__ __forceinline__ int64_t Stride() const { return DIR == 0 ? 1 : stride; }
  __device__ __forceinline__ bool Load(double* u, int j) const {
    const int64_t off = base + int64_t(BcIndex(j, nd, bc)) * Stride();
#pragma unroll
    for (int c = 0; c < K; ++c) u[c] = __ldg(in + c * cs + off);
    return BcFlip(j, nd, bc);
  }
  // interior cell j's components for the update (an L1 hit: loaded two
  // iterations earlier)
  struct Ref {
    const double* p;
    int64_t cs;
    __device__ __forceinline__ double operator[](int c) const { return __ldg(p + c * cs); }
  };
  __device__ __forceinline__ Ref CellRef(int j) const {
    return Ref{in + base + int64_t(j) * Stride(), cs};
  }
  __device__ __forceinline__ void Advance(int) {}
};

// Policy P = PT<D> provides: Real (compute precision), Gas, Rec (face
// state), Wave (cell wave data), Stats, MakeGas(), ToCell() (double ->
// Real), Predict(), MakeWave(), and Face(): the numeric flux of the face
// between recR of the left cell and recL of the right cell (as double) and
// the face's max signal speed of the input state (the CFL check).
//
// MarchSegment: one thread's segment [j0, j1) of its grid line `line`:
// computes the faces j0..j1, writes the updated cells j0..j1-1 and folds the
// input's face speeds into smax.  Lanes of `amask` march together (the CFL
// screen's votes).
template <int D, int DIR, class P, class Line>
__device__ __forceinline__ void MarchSegment(const SweepArgs& a, Line& line, int j0, int j1,
                                             unsigned amask, double split_dt,
                                             typename P::Real& smax, int& status,
                                             typename P::Stats& stats) {
  constexpr int K = D + 2;
  const bool skip_cfl = HasFluxOnly<P>::value && a.skip_cfl != 0;
  constexpr bool kFilter = FilteredCfl<P>::value && HasFluxOnly<P>::value;
  // the FP32 screen's error bound is stated for 1 < gamma <= 2
  const bool screen = kFilter && !skip_cfl && a.gamma > 1.0 && a.gamma <= 2.0;
  const typename P::Gas eq = P::MakeGasFor(a);
  const double lambda_half = 0.5 * split_dt / a.dx;
  const double dt_dx = split_dt / a.dx;
  using R = typename P::Real;
  double* __restrict__ out = a.out;
  const int64_t cs = line.cs;
  // compute-precision window of three cells; the FP64 loads run one cell
  // ahead of the arithmetic (dn is the next "up").  The update of cell j-1
  // re-reads its FP64 state (Line::Cell) instead of carrying a window of
  // FP64 states in registers.
  double dn[K];
  R cm[K], cc[K], cp[K];
  const bool flip_cm = line.Load(dn, j0 - 2);
  P::ToCell(cm, dn);
  if (flip_cm) cm[1 + DIR] = -cm[1 + DIR];
  const bool flip_cc = line.Load(dn, j0 - 1);
  P::ToCell(cc, dn);
  if (flip_cc) cc[1 + DIR] = -cc[1 + DIR];
  bool flip_dn = line.Load(dn, j0);
  using FluxT = typename FluxOf<P>::type;
  typename P::Rec recR_prev;
  typename P::Wave w_prev;
  FluxT F_prev[K];
  fast::Gas<float> g32;
  g32.gamma = static_cast<float>(a.gamma);
  g32.gm1 = static_cast<float>(a.gamma - 1.0);
  using S = CflScreen<P, D>;
  typename S::V v_prev{};
  bool ok_prev = false;
  bool have_prev = false;  // w_prev holds the exact wave of cell j-1
  // skip threshold: a lower bound of an evaluated face's exact speed
  float thr = 0.0f;
  if (kFilter && !skip_cfl && a.smax_out) thr = CflFloatBelow(CflSync(a.smax_out, 0.0, amask));
  for (int j = j0 - 1; j <= j1; ++j) {
    line.Advance(j);
    if constexpr (kFilter) {
      // the CFL speed of face j (cells j-1, j), before the reconstruction
      // so that its registers are free
      if (!skip_cfl) {
        float c32[K];
#pragma unroll
        for (int c = 0; c < K; ++c) c32[c] = CflToF32(cc[c]);
        const typename S::V v = S::Wave(g32, c32, DIR);
        const bool ok = screen && CflInRange<D>(c32) && v.a > 0.0f;
        if (j >= j0) {
          const float s32 = S::Speed(g32, v_prev, v, DIR);
          const float sh = fast::Math<float>::Sqrt(fmaxf(v_prev.h, v.h));
          const float bound = fmaf(s32, kCflRel, fmaf(kCflScale, sh, kCflAbs));
          const bool need = !(ok && ok_prev && bound < thr);
          if (__any_sync(amask, need)) {
            // the whole warp evaluates (the same instructions as some lanes)
            const typename P::Wave wl = have_prev ? w_prev : P::MakeWave(eq, cm, DIR);
            w_prev = P::MakeWave(eq, cc, DIR);
            const R s = P::FaceMaxSpeed(eq, wl, w_prev);
            smax = s > smax ? s : smax;
            thr = fmaxf(thr, CflFloatBelow(static_cast<double>(smax)));
            have_prev = true;
          } else {
            have_prev = false;
          }
          if (a.smax_out && ((j - j0) % kCflSyncRows) == kCflSyncRows - 1)
            thr = fmaxf(thr, CflFloatBelow(CflSync(a.smax_out, static_cast<double>(smax), amask)));
        }
        ok_prev = ok;
        v_prev = v;
      }
    }
    P::ToCell(cp, dn);
    if (flip_dn) cp[1 + DIR] = -cp[1 + DIR];  // a reflective wall's image
    if (j + 2 <= j1 + 1) flip_dn = line.Load(dn, j + 2);
    typename P::Rec recL, recR;
    P::Predict(eq, recL, recR, cm, cc, cp, a.limiter, lambda_half, DIR);
    typename P::Wave w{};
    if (!kFilter && !skip_cfl) w = P::MakeWave(eq, cc, DIR);
    if (j >= j0) {
      FluxT F[K];
      if constexpr (kFilter) {
        SweepFluxOnly<P>(eq, F, recR_prev, recL, DIR);
      } else if constexpr (HasFluxOnly<P>::value) {
        if (skip_cfl) {
          SweepFluxOnly<P>(eq, F, recR_prev, recL, DIR);
        } else {
          const R s = SweepFace<P>(eq, F, recR_prev, recL, w_prev, w, DIR, stats);
          smax = s > smax ? s : smax;
        }
      } else {
        const R s = SweepFace<P>(eq, F, recR_prev, recL, w_prev, w, DIR, stats);
        smax = s > smax ? s : smax;
      }
      if (j > j0) {
        // cell j-1 (inside [0, nd)): U' = U + dt/dx (F_{j-1} - F_j)
        const int64_t off = line.base + int64_t(j - 1) * line.Stride();
        const auto cell = line.CellRef(j - 1);
#pragma unroll
        for (int c = 0; c < K; ++c) {
          const double v = cell[c] + dt_dx * FluxDiff(F_prev[c], F[c]);
          out[c * cs + off] = v;
          // non-positive density: sign bit set or zero (integer test)
          if (c == 0 && __double_as_longlong(v) <= 0) status |= kStatusNonPositiveDensity;
        }
      }
#pragma unroll
      for (int c = 0; c < K; ++c) F_prev[c] = F[c];
    }
    recR_prev = recR;
    if constexpr (!kFilter) w_prev = w;
#pragma unroll
    for (int c = 0; c < K; ++c) {
      cm[c] = cc[c];
      cc[c] = cp[c];
    }
  }
}

template <int D, int DIR, template <int> class PT>
__global__ void __launch_bounds__(128, PT<D>::kMinBlocks) SweepMarchKernel(SweepArgs a) {
  using P = PT<D>;
  constexpr int K = D + 2;
  const int nx = a.n[0], ny = a.n[1], nz = a.n[2];
  int64_t ntrans;
  if (DIR == 0) ntrans = int64_t(ny) * nz;
  else if (DIR == 1) ntrans = int64_t(nx) * nz;
  else ntrans = int64_t(nx) * ny;
  const int64_t t_end = a.t_hi > 0 ? a.t_hi : ntrans;
  const int64_t t = a.t_lo + int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int j0 = blockIdx.y * a.seg_len;
  const int j1 = min(a.n[DIR], j0 + a.seg_len);

  const double split_dt = a.dt_ptr ? a.dt_scale * (*a.dt_ptr) : a.dt_value;
  if (!BlockAll(SweepGate(a, split_dt))) return;
  const bool active = t < t_end;
  const unsigned amask = __ballot_sync(0xffffffffu, active);

  GlobalLine<K, DIR> line;
  line.in = a.in;
  line.cs = int64_t(nx) * ny * nz;
  line.nd = a.n[DIR];
  line.bc = a.bc;
  if (DIR == 0) {
    line.base = t * nx;
    line.stride = 1;
  } else if (DIR == 1) {
    const int64_t i = t % nx, k = t / nx;
    line.base = k * int64_t(nx) * ny + i;
    line.stride = nx;
  } else {
    line.base = t;
    line.stride = int64_t(nx) * ny;
  }
  using R = typename P::Real;
  R smax = R(0);
  int status = 0;
  typename P::Stats stats;
  if (active) MarchSegment<D, DIR, P>(a, line, j0, j1, amask, split_dt, smax, status, stats);
  stats.Flush(a.stats_out);
  const double smax_d = static_cast<double>(smax);
  BlockMaxAtomic<1>(a.smax_out, &smax_d);
  if (status && a.ctrl) atomicOr(&a.ctrl->step_status, status);
}

// The cells of a warp's 32 x-neighbouring grid lines of a y or z sweep,
// staged into shared memory by TMA.  The warp owns a ring of kStages
// buffers, each holding kRows cells of its 32 lines with all K components
// ([K][kRows][32] doubles, one cp.async.bulk.tensor box of this GPU's own
// state buffer: 32 x-cells by kRows cells along the sweep by K components);
// lane 0 issues a buffer's copy, which completes on the buffer's mbarrier,
// and every lane waits for it before its first read.  A buffer is refilled
// with the rows kStages buffers further on once the march has left its last
// row behind (the update's re-read of cell j-1 is its last use): the lanes
// meet at __syncwarp, and lane 0 orders their reads before the copy
// (fence.proxy.async).  Ghost cells outside the grid come from global memory
// as in GlobalLine (the box's rows there are zero-filled and unused).  Every
// wait is bounded: a timeout clears `ok`, the march goes on without waiting
// and the sweep reports kStatusCopyTimeout; Finish waits (bounded) for the
// copies the march did not consume before the warp leaves.
constexpr uint32_t kTmaPolls = 1u << 22;

template <int K, int DIR, int kRows, int kStages> struct TmaLine : GlobalLine<K, DIR> {
  static constexpr int kBox = K * kRows * 32;  // doubles per buffer
  double* ring;     // [kStages][kBox]
  uint64_t* bars;   // [kStages]
  const void* map;  // CUtensorMap (kernel parameter space)
  int lane, x0, tr;     // box origin: x, the other transverse coordinate
  int first, nstages;   // row of buffer 0's first cell; buffers of the segment
  int ready, released;  // buffers waited for; buffers released
  unsigned amask;
  bool ok;

  __device__ __forceinline__ void Issue(int q) {  // lane 0
    const int slot = q % kStages;
    tma::MbarArriveExpectTx(&bars[slot], kBox * 8);
    double* dst = ring + slot * kBox;
    const int row = first + q * kRows;
    if constexpr (K == 5) {
      if (DIR == 1)
        tma::TmaLoad4D(dst, map, x0, row, tr, 0, &bars[slot]);
      else
        tma::TmaLoad4D(dst, map, x0, tr, row, 0, &bars[slot]);
    } else {
      tma::TmaLoad3D(dst, map, x0, row, 0, &bars[slot]);
    }
  }
  __device__ __forceinline__ void Start(int j0, int j1) {
    first = j0 - 2;
    nstages = (j1 - j0 + 4 + kRows - 1) / kRows;
    ready = 0;
    released = 0;
    ok = true;
    if (lane == 0)
      for (int q = 0; q < kStages && q < nstages; ++q) Issue(q);
  }
  __device__ __forceinline__ void WaitUpTo(int q) {
    for (; ready <= q; ++ready)
      if (ok && !tma::MbarWait(&bars[ready % kStages], (ready / kStages) & 1, kTmaPolls))
        ok = false;
  }
  __device__ __forceinline__ const double* At(int j) {  // interior cell j
    const unsigned rel = static_cast<unsigned>(j - first);
    const int q = static_cast<int>(rel / kRows);
    WaitUpTo(q);
    return ring + (q % kStages) * kBox + (rel % kRows) * 32 + lane;
  }
  __device__ __forceinline__ bool Load(double* u, int j) {
    if (j < 0 || j >= this->nd) return GlobalLine<K, DIR>::Load(u, j);
    const double* p = At(j);
#pragma unroll
    for (int c = 0; c < K; ++c) u[c] = p[c * kRows * 32];
    return false;
  }
  struct Ref {
    const double* p;
    __device__ __forceinline__ double operator[](int c) const { return p[c * kRows * 32]; }
  };
  __device__ __forceinline__ Ref CellRef(int j) { return Ref{At(j)}; }
  __device__ __forceinline__ void Advance(int j) {
    while (released < nstages && first + (released + 1) * kRows <= j - 1) {
      WaitUpTo(released);  // the buffer's copy has landed before it is refilled
      __syncwarp(amask);
      if (lane == 0 && ok && released + kStages < nstages) {
        tma::FenceProxyAsync();
        Issue(released + kStages);
      }
      ++released;
    }
  }
  // Lane 0: waits for the issued copies nobody waited for.
  __device__ __forceinline__ void Finish() {
    if (lane != 0) return;
    const int issued = min(nstages, released + kStages);
    for (; ready < issued; ++ready)
      if (!tma::MbarWait(&bars[ready % kStages], (ready / kStages) & 1, kTmaPolls)) ok = false;
  }
};

template <int K> constexpr size_t TmaSweepSmemBytes() {
  return size_t(kTmaWarps) * kTmaStages * (K * kTmaRows * 32 * 8 + 8);
}

// A y or z sweep with the cells staged by TMA (TmaLine): warp w of the grid
// owns x-chunk w % ceil(nx / 32) of the lines at transverse index w / that
// (z for y sweeps, y for z sweeps), segment blockIdx.y.  `map` describes this
// GPU's own input state buffer as [K][nz][ny][nx] doubles (3-D) or
// [K][ny][nx] (2-D) with boxes of 32 x kTmaRows cells along DIR.
template <int D, int DIR, template <int> class PT>
__global__ void __launch_bounds__(128, PT<D>::kMinBlocks)
    SweepTmaKernel(SweepArgs a, const __grid_constant__ CUtensorMap map) {
  static_assert(DIR >= 1 && DIR < D, "y or z sweeps");
  using P = PT<D>;
  constexpr int K = D + 2;
  extern __shared__ __align__(128) unsigned char tma_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nx = a.n[0], ny = a.n[1], nz = a.n[2];
  const int nchunks = (nx + 31) / 32;
  const int ntr = DIR == 1 ? nz : ny;
  const int64_t gw = int64_t(blockIdx.x) * kTmaWarps + warp;
  const bool has_work = gw < int64_t(nchunks) * ntr;  // warp-uniform
  const int xc = has_work ? static_cast<int>(gw % nchunks) : 0;
  const int tr = has_work ? static_cast<int>(gw / nchunks) : 0;
  const int i = xc * 32 + lane;
  const int j0 = blockIdx.y * a.seg_len;
  const int j1 = min(a.n[DIR], j0 + a.seg_len);

  const double split_dt = a.dt_ptr ? a.dt_scale * (*a.dt_ptr) : a.dt_value;
  if (!BlockAll(SweepGate(a, split_dt))) return;
  const bool active = has_work && i < nx;
  const unsigned amask = __ballot_sync(0xffffffffu, active);

  using Line = TmaLine<K, DIR, kTmaRows, kTmaStages>;
  Line line;
  line.in = a.in;
  line.cs = int64_t(nx) * ny * nz;
  line.nd = a.n[DIR];
  line.bc = a.bc;
  if (DIR == 1) {
    line.base = int64_t(tr) * nx * ny + i;
    line.stride = nx;
  } else {
    line.base = int64_t(tr) * nx + i;
    line.stride = int64_t(nx) * ny;
  }
  line.ring = reinterpret_cast<double*>(tma_smem) + size_t(warp) * kTmaStages * Line::kBox;
  line.bars = reinterpret_cast<uint64_t*>(tma_smem + size_t(kTmaWarps) * kTmaStages *
                                                        Line::kBox * 8) +
              warp * kTmaStages;
  line.map = &map;
  line.lane = lane;
  line.x0 = xc * 32;
  line.tr = tr;
  line.amask = amask;

  using R = typename P::Real;
  R smax = R(0);
  int status = 0;
  typename P::Stats stats;
  if (has_work) {
    if (lane == 0) {
      for (int q = 0; q < kTmaStages; ++q) tma::MbarInit(&line.bars[q], 1);
      tma::FenceMbarInit();
    }
    __syncwarp();
    line.Start(j0, j1);
    if (active) MarchSegment<D, DIR, P>(a, line, j0, j1, amask, split_dt, smax, status, stats);
    line.Finish();
    if (!line.ok) status |= kStatusCopyTimeout;
  }
  stats.Flush(a.stats_out);
  const double smax_d = static_cast<double>(smax);
  BlockMaxAtomic<1>(a.smax_out, &smax_d);
  if (status && a.ctrl) atomicOr(&a.ctrl->step_status, status);
}

// Warp shuffles of whole structs (32-bit words).
template <class T> __device__ __forceinline__ T ShflUp(const T& v, unsigned delta) {
  static_assert(sizeof(T) % 4 == 0, "shuffle of 32-bit words");
  constexpr int N = sizeof(T) / 4;
  unsigned w[N];
  memcpy(w, &v, sizeof(T));
#pragma unroll
  for (int i = 0; i < N; ++i) w[i] = __shfl_up_sync(0xffffffffu, w[i], delta);
  T r;
  memcpy(&r, w, sizeof(T));
  return r;
}

template <class T> __device__ __forceinline__ T ShflDown(const T& v, unsigned delta) {
  constexpr int N = sizeof(T) / 4;
  unsigned w[N];
  memcpy(w, &v, sizeof(T));
#pragma unroll
  for (int i = 0; i < N; ++i) w[i] = __shfl_down_sync(0xffffffffu, w[i], delta);
  T r;
  memcpy(&r, w, sizeof(T));
  return r;
}

template <class T> __device__ __forceinline__ T ShflIdx(const T& v, int src) {
  constexpr int N = sizeof(T) / 4;
  unsigned w[N];
  memcpy(w, &v, sizeof(T));
#pragma unroll
  for (int i = 0; i < N; ++i) w[i] = __shfl_sync(0xffffffffu, w[i], src);
  T r;
  memcpy(&r, w, sizeof(T));
  return r;
}

template <class R, int K> struct CellArr {
  R v[K];
};

// x sweep with the lanes of a warp along x: every load and store of a warp
// touches 32 consecutive doubles of one row, and the neighbours a cell needs
// come from the adjacent lanes by shuffles.  One warp owns one row and walks
// it in chunks of 32 cells; lane l of a chunk reconstructs cell x, computes
// the flux of face x (between x-1 and x) and updates cell x-1.  A warm-up
// step reconstructs cells -2 and -1; on a periodic row lane 0 of the first
// chunk then updates cell -1 = nx-1, which closes the ring without a partial
// last step.  A transmissive row finishes with a one-lane step for cell
// nx-1.  The arithmetic per face and cell is the policy's, exactly as in
// SweepMarchKernel.
template <int D, template <int> class PT>
__device__ __forceinline__ void XWarpRow(const SweepArgs& a, int64_t row, double split_dt,
                                         typename PT<D>::Real& smax, int& status,
                                         typename PT<D>::Stats& stats) {
  using P = PT<D>;
  using R = typename P::Real;
  constexpr int K = D + 2;
  using Cell = CellArr<R, K>;
  using Dbl = CellArr<double, K>;
  const int nx = a.n[0];
  const int64_t cs = int64_t(nx) * a.n[1] * a.n[2];
  const int lane = threadIdx.x & 31;
  const int64_t base = row * nx;
  const bool periodic = (a.bc == 0);
  const typename P::Gas eq = P::MakeGasFor(a);
  const double lambda_half = 0.5 * split_dt / a.dx;
  const double dt_dx = split_dt / a.dx;
  const double* __restrict__ in = a.in;
  double* __restrict__ out = a.out;
  auto load = [&](Dbl& u, int x) {
    const int64_t off = base + BcIndex(x, nx, a.bc);
#pragma unroll
    for (int c = 0; c < K; ++c) u.v[c] = __ldg(in + c * cs + off);
  };
  auto to_cell = [&](const Dbl& u) {
    Cell c;
    P::ToCell(c.v, u.v);
    return c;
  };

  // ---- warm-up: cells -3..-1 in lanes 29..31, cell 0 from the first chunk
  Dbl U0;
  load(U0, lane);                      // chunk 0
  Dbl Uw;
  load(Uw, lane >= 29 ? lane - 32 : -3);  // lanes 0..28 hold a copy of cell -3
  Cell Cw = to_cell(Uw);
  const Cell C0 = to_cell(U0);
  Cell Cwm = ShflUp(Cw, 1);
  Cell Cwp = ShflDown(Cw, 1);
  const Cell C0first = ShflIdx(C0, 0);
  if (lane == 31) Cwp = C0first;
  if (lane == 0) Cwm = Cw;
  typename P::Rec wrecL, wrecR;
  P::Predict(eq, wrecL, wrecR, Cwm.v, Cw.v, Cwp.v, a.limiter, lambda_half, 0);
  const bool skip_cfl = HasFluxOnly<P>::value && a.skip_cfl != 0;  // warp-uniform
  // faces with or without their CFL speed (see HasFluxOnly)
  auto face = [&](FluxOfArg<P>* F, const typename P::Rec& L, const typename P::Rec& Rr,
                  const typename P::Wave& wl, const typename P::Wave& wr,
                  typename P::Stats& st) -> R {
    if constexpr (HasFluxOnly<P>::value) {
      if (skip_cfl) {
        SweepFluxOnly<P>(eq, F, L, Rr, 0);
        return R(0);
      }
    }
    return SweepFace<P>(eq, F, L, Rr, wl, wr, 0, st);
  };
  typename P::Wave wW{};
  if (!skip_cfl) wW = P::MakeWave(eq, Cw.v, 0);
  // face -1 (between cells -2 and -1), used to update cell -1 on a periodic row
  const typename P::Rec wrecRm = ShflUp(wrecR, 1);
  typename P::Wave wWm{};
  if (!skip_cfl) wWm = ShflUp(wW, 1);
  using FluxT = typename FluxOf<P>::type;
  using Flx = CellArr<FluxT, K>;
  FluxT Fw[K];
  typename P::Stats wstats;
  face(Fw, wrecRm, wrecL, wWm, wW, wstats);
  // carries into chunk 0 (from lane 31 = cell -1)
  typename P::Rec carry_rec = ShflIdx(wrecR, 31);
  typename P::Wave carry_w{};
  if (!skip_cfl) carry_w = ShflIdx(wW, 31);
  Cell carry_c = ShflIdx(Cw, 31);
  Flx carry_f;
#pragma unroll
  for (int c = 0; c < K; ++c) carry_f.v[c] = Fw[c];
  carry_f = ShflIdx(carry_f, 31);

  Cell C = C0;
  const int nchunks = (nx + 31) / 32;
  Dbl Unext;  // the chunk after the next one is loaded one iteration early
  load(Unext, lane + 32);
  for (int ch = 0; ch < nchunks; ++ch) {
    const int x0 = ch * 32;
    const int x = x0 + lane;
    const bool valid = x < nx;
    const Dbl Un = Unext;
    if (ch + 1 < nchunks) load(Unext, x + 64);
    const Cell Cn = to_cell(Un);
    Cell Cp = ShflDown(C, 1);
    const Cell Cn0 = ShflIdx(Cn, 0);
    if (lane == 31) Cp = Cn0;
    if (x + 1 >= nx && !periodic) Cp = C;  // transmissive: cells >= nx copy nx-1
    Cell Cm = ShflUp(C, 1);
    if (lane == 0) Cm = carry_c;
    typename P::Rec recL, recR;
    P::Predict(eq, recL, recR, Cm.v, C.v, Cp.v, a.limiter, lambda_half, 0);
    typename P::Wave W{};
    if (!skip_cfl) W = P::MakeWave(eq, C.v, 0);
    typename P::Rec recRm = ShflUp(recR, 1);
    typename P::Wave Wm{};
    if (!skip_cfl) Wm = ShflUp(W, 1);
    if (lane == 0) {
      recRm = carry_rec;
      Wm = carry_w;
    }
    Flx Fd;
    const R sp = face(Fd.v, recRm, recL, Wm, W, stats);
    if (valid) smax = sp > smax ? sp : smax;
    Flx Fm = ShflUp(Fd, 1);
    if (lane == 0) Fm = carry_f;
    // update cell x-1 (lane 0 of chunk 0: cell -1, i.e. nx-1 on a periodic row);
    // its FP64 state is re-read (a coalesced L1 hit) rather than shuffled
    const bool upd = valid && (x >= 1 || periodic);
    if (upd) {
      const int64_t off = base + BcIndex(x - 1, nx, a.bc);
#pragma unroll
      for (int c = 0; c < K; ++c) {
        const double v = __ldg(in + c * cs + off) + dt_dx * FluxDiff(Fm.v[c], Fd.v[c]);
        out[c * cs + off] = v;
        if (c == 0 && __double_as_longlong(v) <= 0) status |= kStatusNonPositiveDensity;
      }
    }
    // carries: the chunk's last cell
    const int last = min(31, nx - 1 - x0);
    carry_rec = ShflIdx(recR, last);
    if (!skip_cfl) carry_w = ShflIdx(W, last);
    carry_c = ShflIdx(C, last);
    carry_f = ShflIdx(Fd, last);
    C = Cn;
  }
  if (!periodic) {
    // face nx and cell nx-1 of a transmissive row (cells >= nx copy nx-1)
    typename P::Rec recL, recR;
    P::Predict(eq, recL, recR, carry_c.v, carry_c.v, carry_c.v, a.limiter, lambda_half, 0);
    typename P::Wave W{};
    if (!skip_cfl) W = P::MakeWave(eq, carry_c.v, 0);
    FluxT F[K];
    const R sp = face(F, carry_rec, recL, carry_w, W, stats);
    if (lane == 0) {
      smax = sp > smax ? sp : smax;
      const int64_t off = base + (nx - 1);
#pragma unroll
      for (int c = 0; c < K; ++c) {
        const double v = __ldg(in + c * cs + off) + dt_dx * FluxDiff(carry_f.v[c], F[c]);
        out[c * cs + off] = v;
        if (c == 0 && __double_as_longlong(v) <= 0) status |= kStatusNonPositiveDensity;
      }
    }
  }
}

// The kernel: one row per warp.  A block whose warps all have a row reduces
// their max signal speed before one atomic; the last block of a grid whose
// row count is not a multiple of the warps per block returns its idle warps
// early and reduces per warp (no barrier after the return).
template <int D, template <int> class PT>
__global__ void __launch_bounds__(128, PT<D>::kMinBlocks) SweepXWarpKernel(SweepArgs a) {
  using P = PT<D>;
  using R = typename P::Real;
  const int64_t rows = a.t_hi > 0 ? a.t_hi - a.t_lo : int64_t(a.n[1]) * a.n[2];
  const double split_dt = a.dt_ptr ? a.dt_scale * (*a.dt_ptr) : a.dt_value;
  if (!BlockAll(SweepGate(a, split_dt))) return;
  R smax = R(0);
  int status = 0;
  typename P::Stats stats;
  const int64_t rel = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int64_t row = a.t_lo + rel;
  const bool full_block = int64_t(blockIdx.x + 1) * (blockDim.x >> 5) <= rows;  // block-uniform
  if (rel >= rows) return;  // only in a block that is not full
  XWarpRow<D, PT>(a, row, split_dt, smax, status, stats);
  stats.Flush(a.stats_out);
  const double smax_d = static_cast<double>(smax);
  if (full_block) {
    BlockMaxAtomic<1>(a.smax_out, &smax_d);
  } else {
    const double m = WarpMax(smax_d);
    if ((threadIdx.x & 31) == 0 && a.smax_out && m > 0.0) AtomicMaxPositive(a.smax_out, m);
  }
  if (status && a.ctrl) atomicOr(&a.ctrl->step_status, status);
}

// The TMA-staged y/z sweep (a.tmap: the host's tensor map of a.in), built
// for the mixed flavour's policies with lanes-along-x x sweeps.
template <class P, class = void> struct TmaStaged : std::false_type {};
template <class P>
struct TmaStaged<P, std::enable_if_t<P::kFloatFlux && P::kWarpX>> : std::true_type {};
template <class P> constexpr bool kTmaStaged = TmaStaged<P>::value;

// The TMA-staged y/z sweep (a.tmap: the host's tensor map of a.in).
template <int D, int DIR, template <int> class P>
cudaError_t LaunchSweepTma(const SweepArgs& a, cudaStream_t s) {
  constexpr size_t smem = TmaSweepSmemBytes<D + 2>();
  static bool attr_set = false;
  if (!attr_set) {
    const cudaError_t e = cudaFuncSetAttribute(
        SweepTmaKernel<D, DIR, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  const int64_t warps = int64_t((a.n[0] + 31) / 32) * (DIR == 1 ? a.n[2] : a.n[1]);
  const int seg = a.seg_len > 0 ? a.seg_len : a.n[DIR];
  dim3 grid(static_cast<unsigned>((warps + kTmaWarps - 1) / kTmaWarps),
            static_cast<unsigned>((a.n[DIR] + seg - 1) / seg));
  SweepTmaKernel<D, DIR, P><<<grid, 32 * kTmaWarps, smem, s>>>(
      a, *static_cast<const CUtensorMap*>(a.tmap));
  return cudaGetLastError();
}

template <int D, template <int> class P>
cudaError_t LaunchSweepT(const SweepArgs& a, cudaStream_t s) {
  const int nd = a.n[a.dir];
  int64_t ntrans = 1;
  for (int d = 0; d < 3; ++d)
    if (d != a.dir) ntrans *= a.n[d];
  if (a.t_hi > 0) ntrans = a.t_hi - a.t_lo;  // a range of the lines
  const int block = 128;
  const int seg = a.seg_len > 0 ? a.seg_len : nd;
  SweepArgs b = a;
  b.seg_len = seg;
  dim3 grid(static_cast<unsigned>((ntrans + block - 1) / block),
            static_cast<unsigned>((nd + seg - 1) / seg));
  switch (a.dir) {
  case 0:
    if constexpr (P<D>::kWarpX) {
      // (x sweeps of reflective rows take the marching kernel: the caller
      // routes them to a policy without kWarpX)
      const int64_t rows = ntrans;
      const unsigned xgrid = static_cast<unsigned>((rows * 32 + block - 1) / block);
      SweepXWarpKernel<D, P><<<xgrid, block, 0, s>>>(b);
    } else {
      SweepMarchKernel<D, 0, P><<<grid, block, 0, s>>>(b);
    }
    break;
  case 1:
    if constexpr (D >= 2) {
      if constexpr (kTmaStaged<P<D>>)
        if (a.occupancy >= 20 && a.tmap && a.t_hi == 0) return LaunchSweepTma<D, 1, P>(b, s);
      SweepMarchKernel<D, 1, P><<<grid, block, 0, s>>>(b);
    }
    break;
  default:
    if constexpr (D >= 3) {
      if constexpr (kTmaStaged<P<D>>)
        if (a.occupancy >= 20 && a.tmap && a.t_hi == 0) return LaunchSweepTma<D, 2, P>(b, s);
      SweepMarchKernel<D, 2, P><<<grid, block, 0, s>>>(b);
    }
    break;
  }
  return cudaGetLastError();
}

}  // namespace fvs
