// fvs_internal.h -- declarations shared between the translation units of
// libfvs_gb300 (not part of the C ABI).
#pragma once

#include <cstdint>
#include <string>

#include <cuda_runtime.h>

struct fvs_method;  // include/fvs_gpu.h

namespace fvs {

// A box of an FArrayBox-layout array: lower corner and extents.
struct BoxDesc {
  int lo[3];
  int n[3];
};

// Per-run control block resident in device memory.  The time step lives on
// the device so that a whole split step (stable dt, sweeps, checks) runs
// without a host round trip and can be captured in a CUDA graph.
struct Control {
  double t;          // current time point
  double dt;         // time step of the step in flight
  double t_end;      // final time
  double cfl;        // CFL number
  double fail_dt;    // level dt of the first failed per-sweep check
  double dt_override;  // > 0: use this dt for the next step instead of cfl*stable
  unsigned long long smax_stable[3];  // bits of max face speed, per direction
  unsigned long long smax_check[6];   // bits of max face speed, per sweep
  unsigned long long newton[3];       // Newton iterations, non-converged faces,
                                      // faces whose learned start was rejected
  int abort;         // a per-sweep check failed; later kernels do nothing
  int done;          // t reached t_end; later kernels do nothing
  int failed_step;   // index of the failed step within the batch
  int steps_done;    // committed steps since the counter was reset
  int status;        // FVS_STATUS_* bits of committed steps
  int step_status;   // status bits of the step in flight
  int have_failure;  // next step uses fail_dt instead of the stable dt pass
  int pad;
};

enum StatusBits : int {
  kStatusNonPositiveDensity = 1,
  kStatusNonFinite = 2,
  kStatusNewtonNotConverged = 4,
  kStatusCopyTimeout = 8,  // a staged (TMA) copy did not land in time
};

// Slabs of a host-resident step's last sweep (fvs_solver_step_host): each
// slab's download starts when the slab's cells are final.
constexpr int kHostSlabs = 8;

// The TMA-staged y/z sweep (mixed flavour): each warp stages its 32 lines
// in a ring of kTmaStages buffers of kTmaRows cells; blocks of kTmaWarps.
constexpr int kTmaRows = 2;
constexpr int kTmaStages = 4;
constexpr int kTmaWarps = 4;

// One directional sweep of a uniform grid: fluxes, conservative update and
// the CFL reduction of the input state, in one pass.
struct SweepArgs {
  const double* in;     // conservative state, component-major [D+2][nz][ny][nx]
  double* out;          // updated state, same layout (must not alias `in`)
  int n[3];
  int rank;
  int dir;
  int bc;               // 0 periodic, 1 transmissive (in `dir`)
  int limiter;
  int seg_len;          // cells per thread segment along `dir`
  int block;            // threads per block
  double gamma;
  double dx;
  // split dt = dt_scale * (*dt_ptr) when dt_ptr is set, else dt_value
  const double* dt_ptr;
  double dt_scale;
  double dt_value;
  unsigned long long* smax_out;  // atomicMax of the input state's face speeds
  Control* ctrl;        // optional: abort/done gating and status bits
  // previous sweep's check (skip this sweep when it failed); -1 for none
  int prev_check;
  double prev_dx;
  // exact Riemann solver (Godunov policies)
  int guess;            // fvs_guess
  int max_iterations;
  double tolerance;
  const float* mlp;     // learned-guess weights (guess == FVS_GUESS_MLP)
  unsigned long long* stats_out;  // [3]: Newton iterations, non-converged, fallbacks
  // the first sweep of a step: its input's face speeds are the stable-dt
  // pass's, so the sweep computes no cell waves and no CFL speeds
  int skip_cfl;
  int occupancy;        // 0 (registers as needed) or the resident blocks per SM a
                        // variant is compiled for (mixed: 4, 5; double-float: 3);
                        // mixed x sweeps: + 10 for the marching kernel in x;
                        // mixed y/z sweeps: + 20 for the TMA-staged kernel
  const void* tmap;     // host: CUtensorMap of `in` for the TMA-staged kernel, or NULL
  // grid lines [t_lo, t_hi) only (t: the line index of the marching and
  // lanes-along-x kernels); t_hi == 0: every line
  int64_t t_lo, t_hi;
};

// Stable-dt pass over all directions (max face speed per direction).
struct StableDtArgs {
  const double* in;
  int n[3];
  int rank;
  int bc[3];
  int rule;             // 0 all faces, 1 reference MFIter tiles of 8 in y/z
  int width;            // stencil width of the method (windows of 2 width cells)
  double gamma;
  unsigned long long* smax_out;  // [rank]
  Control* ctrl;
  // 3-D: the faces of the planes [k_lo, k_hi) only (their z faces read plane
  // k_lo - 1); k_hi == 0: every plane
  int k_lo, k_hi;
};

// Sets the message returned by fvs_last_error() (fvs_capi.cu).
void SetLastError(const std::string& msg);
// Argument checks shared by the C ABI's entry points (fvs_capi.cu): the
// method's fields and rank (FVS_ERR_INVALID / FVS_ERR_UNSUPPORTED), and that
// a CUDA device is present (FVS_ERR_NO_DEVICE, clearing the runtime's sticky
// "no device" error).  Return FVS_OK or the status, with fvs_last_error() set.
int CheckMethod(const ::fvs_method* m, int rank);
int CheckDevice();

// Exact FP64 kernels (fvs_kernels_exact.cu, compiled with -fmad=false).
cudaError_t LaunchSweepExact(const SweepArgs& a, cudaStream_t s);
cudaError_t LaunchStableDtExact(const StableDtArgs& a, cudaStream_t s);
// recon: 0 none (HLLEM), 1 conservative MUSCL-Hancock, 2 characteristic,
// 3 primitive reconstruction
cudaError_t LaunchSweepHllem(const SweepArgs& a, int recon, cudaStream_t s);
cudaError_t LaunchSweepDf64(const SweepArgs& a, cudaStream_t s);
cudaError_t LaunchStableDtDf64(const StableDtArgs& a, cudaStream_t s);
cudaError_t LaunchStableDtHllem(const StableDtArgs& a, cudaStream_t s);

// Fast FP64 and mixed FP32/FP64 kernels (fvs_kernels_fast.cu).
cudaError_t LaunchSweepFast(const SweepArgs& a, cudaStream_t s);
cudaError_t LaunchSweepMixed(const SweepArgs& a, cudaStream_t s);
cudaError_t LaunchStableDtFast(const StableDtArgs& a, cudaStream_t s);
cudaError_t LaunchStableDtMixed(const StableDtArgs& a, cudaStream_t s);

// Godunov / exact Riemann solver kernels (fvs_kernels_godunov.cu).
cudaError_t LaunchSweepGodunov(const SweepArgs& a, bool muscl, cudaStream_t s);
cudaError_t LaunchStableDtGodunov(const StableDtArgs& a, int guess, int max_it, double tol,
                                  const float* mlp, cudaStream_t s);
cudaError_t LaunchPatchGodunovFluxes(bool muscl, int limiter, int rank, double gamma, int guess,
                                     int max_it, double tol, const float* mlp, double* fluxes,
                                     BoxDesc fbox, const double* states, BoxDesc cbox, double dt,
                                     double dx, int dir, unsigned long long* stats,
                                     cudaStream_t s);
cudaError_t LaunchPatchGodunovStableDt(bool muscl, int rank, double gamma, int guess, int max_it,
                                       double tol, const float* mlp, const double* states,
                                       BoxDesc cbox, int window_rule, int dir,
                                       unsigned long long* smax, cudaStream_t s);
cudaError_t LaunchExactStar(int64_t n, double gamma, int guess, int max_it, double tol,
                            const float* mlp, const double* rhoL, const double* uL,
                            const double* pL, const double* rhoR, const double* uR,
                            const double* pR, double* pstar, double* ustar, int* iters,
                            int* converged, cudaStream_t s);

// Patch-level kernels over FArrayBox-layout views (fvs_kernels_exact.cu).
cudaError_t LaunchPatchFluxesExact(int method, int limiter, int rank, double gamma,
                                   double* fluxes, BoxDesc fbox,
                                   const double* states, BoxDesc cbox,
                                   double dt, double dx, int dir,
                                   cudaStream_t s);
cudaError_t LaunchPatchStableDtExact(int method, int rank, double gamma,
                                     const double* states, BoxDesc cbox,
                                     int window_rule, int dir,
                                     unsigned long long* smax, cudaStream_t s);
cudaError_t LaunchPatchUpdate(double* next, BoxDesc nbox, BoxDesc region, const double* prev,
                              BoxDesc pbox, const double* fluxes, BoxDesc fbox,
                              int ncomp, double dt, double dx, int dir,
                              cudaStream_t s);
cudaError_t LaunchPatchCompleteFromCons(int rank, double gamma, double* complete,
                                        BoxDesc qbox, const double* cons,
                                        BoxDesc ubox, BoxDesc region,
                                        cudaStream_t s);

}  // namespace fvs
