/* fvs_gpu.h -- C ABI of libfvs_gb300: the GB300 (sm_103a) split
 * finite-volume patch update for the perfect-gas Euler equations.
 *
 * This library is a drop-in for the patch-level calls of
 * maikel/FiniteVolumeSolver's FluxMethod / HyperbolicPatchIntegrator API:
 * ComputeNumericFluxes, ComputeStableDt and UpdateConservatively on a ghosted
 * patch, one direction at a time, plus CompleteFromCons.  A solver context
 * runs whole split steps on a device-resident uniform grid.
 *
 * Conventions
 *  - Patch data uses the reference's FArrayBox layout: component-major,
 *    x fastest; element (c, i, j, k) of a box [lo, hi) is at
 *    ((c*n2 + k-lo2)*n1 + j-lo1)*n0 + i-lo0 with n = hi - lo
 *    (include/fub/AMReX/ViewFArrayBox.hpp:73-82).  Unused dimensions have
 *    lo = 0, hi = 1.
 *  - Complete states have rank+4 components (rho, m[rank], E, p, c);
 *    conservative states rank+2 (rho, m[rank], E)
 *    (include/fub/equations/PerfectGas.hpp:132-161).
 *  - Face boxes follow AMReX: face i in direction d lies between cells i-1
 *    and i.
 *  - Pointers named *_dev are device pointers; `stream` is a cudaStream_t
 *    (NULL = legacy default stream).
 *  - Every call returns an fvs_status.  The library never falls back to a
 *    CPU path: without a usable GPU the calls return FVS_ERR_NO_DEVICE.
 */
#ifndef FVS_GPU_H
#define FVS_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum fvs_status {
  FVS_OK = 0,
  FVS_ERR_INVALID = 1,        /* bad argument (box, rank, direction, ...) */
  FVS_ERR_CUDA = 2,           /* a CUDA call failed; see fvs_last_error() */
  FVS_ERR_DT_TOO_LARGE = 3,   /* a per-sweep CFL check failed */
  FVS_ERR_UNSUPPORTED = 4,    /* method / precision not available here */
  FVS_ERR_NO_DEVICE = 5,      /* no CUDA device */
  FVS_ERR_STATE = 6,          /* non-positive density / non-finite state */
  FVS_ERR_IO = 7              /* a file or directory could not be written */
} fvs_status;

typedef enum fvs_flux_method {
  FVS_MUSCL_HLLE = 0,   /* MusclHancock<PerfectGas, Hll<Einfeldt>, Limiter> */
  FVS_HLLE = 1,         /* Hll<PerfectGas, EinfeldtSignalVelocities> */
  FVS_GODUNOV = 2,      /* Godunov<PerfectGas, ExactRiemannSolver> */
  FVS_MUSCL_GODUNOV = 3, /* MusclHancock<PerfectGas, Godunov<Exact>, Limiter> */
  FVS_HLLEM = 4,        /* perfect_gas::Hllem<PerfectGas, Larrouturou = true> */
  FVS_MUSCL_HLLEM = 5,  /* MusclHancock<PerfectGas, Hllem, Limiter> (exact FP64) */
  FVS_MUSCL_CHAR = 6,   /* perfect_gas::MusclHancockCharacteristic<Rank>: characteristic
                           reconstruction + Hllem (exact FP64, van Leer only);
                           src/equations/perfect_gas/MusclHancockCharacteristicMethod.hpp */
  FVS_MUSCL_PRIM = 7    /* perfect_gas::MusclHancockPrim<Dim>: primitive reconstruction
                           with its own limiter + Hllem (exact FP64; limiter must be
                           FVS_VAN_LEER, the default);
                           src/equations/perfect_gas/MusclHancockPrimMethod.hpp */
} fvs_flux_method;

/* Slope limiters of MusclHancock (include/fub/flux_method/
 * MusclHancockMethod.hpp:31-187). */
typedef enum fvs_limiter {
  FVS_VAN_LEER = 0,
  FVS_MINMOD = 1,
  FVS_NO_LIMITER = 2,   /* NoLimiter: the central slope 0.5 (sL + sR), unlimited */
  FVS_NO_GRADIENT = 3   /* NoGradient: slope 0 (first order in space) */
} fvs_limiter;

typedef enum fvs_precision {
  FVS_FP64_EXACT = 0, /* reference operation order, no FMA: bit-identical */
  FVS_FP64_FAST = 1,  /* FP64 with FMA and shared reciprocals (<= 1e-12 rel) */
  FVS_MIXED = 2,      /* FP32 reconstruction/flux, FP64 state and update */
  FVS_FP64_DF = 3     /* MUSCL-HLLE in double-float (FP32 pairs, ~48 bits) on the
                         FP32 pipes, FP64 state and update (uniform grids); FP32's
                         exponent range: states and products such as rho u^2 within
                         about 1e-30 .. 1e30 */
} fvs_precision;

typedef enum fvs_guess {
  FVS_GUESS_MEAN = 0,    /* reference: 0.5 (pL + pR) */
  FVS_GUESS_PVRS_TR = 1, /* PVRS, two-rarefaction below min(pL, pR) */
  FVS_GUESS_MLP = 2      /* learned guess, PVRS/TR fallback */
} fvs_guess;

/* Boundary conditions, per direction (both sides):
 *  periodic;
 *  transmissive: ghost cells copy the boundary cell
 *    (src/AMReX/boundary_condition/TransmissiveBoundary.cpp:31-93);
 *  reflective: ghost cells are the mirror cells' states reflected at the wall,
 *    the momentum normal to it negated (include/fub/AMReX/boundary_condition/
 *    ReflectiveBoundary.hpp:34-64, src/boundary_condition/
 *    ReflectiveBoundary.cpp:24-36, Reflect src/equations/PerfectGas.cpp:266-300);
 *    needs at least 2 cells in that direction. */
typedef enum fvs_bc {
  FVS_BC_PERIODIC = 0,
  FVS_BC_TRANSMISSIVE = 1,
  FVS_BC_REFLECTIVE = 2
} fvs_bc;

typedef struct fvs_box {
  int32_t lo[3];
  int32_t hi[3]; /* half-open */
} fvs_box;

typedef struct fvs_method {
  int32_t flux_method;   /* fvs_flux_method */
  int32_t limiter;       /* fvs_limiter */
  int32_t precision;     /* fvs_precision */
  int32_t guess;         /* fvs_guess (exact Riemann solver only) */
  int32_t max_iterations;/* Newton iteration bound (exact solver) */
  int32_t reserved;
  double tolerance;      /* Newton tolerance on |f(p)| (reference: 1e-7) */
  double gamma;          /* ratio of specific heats (reference: 1.4) */
  const float* mlp_params; /* device pointer to the learned-guess parameters
                              (FVS_GUESS_MLP); see fvs_mlp_param_count() */
} fvs_method;

/* Fills `m` with the reference's defaults: MUSCL-Hancock + HLLE, van Leer,
 * exact FP64, mean guess, 5000 iterations, tolerance 1e-7, gamma 1.4. */
void fvs_method_default(fvs_method* m);

const char* fvs_last_error(void);
int fvs_abi_version(void);
/* Number of CUDA devices visible (0 without a GPU); never fails. */
int fvs_device_count(void);

/* ---- Patch level: drop-in for the reference's per-patch calls ---------- */

/* FluxMethod<Base>::ComputeNumericFluxes(View<Conservative> fluxes,
 *   View<const Complete> states, Duration dt, double dx, Direction dir)
 * include/fub/flux_method/FluxMethod.hpp:115-134, 200-293.
 * `states_dev` holds rank+4 components over `cell_box`, which must contain
 * every stencil cell of every face of `face_box` (w = 2 for MUSCL, 1 for
 * HLLE/Godunov); `fluxes_dev` receives rank+2 components over `face_box`. */
int fvs_compute_numeric_fluxes(const fvs_method* m, int rank,
                               double* fluxes_dev, fvs_box face_box,
                               const double* states_dev, fvs_box cell_box,
                               double dt, double dx, int dir, void* stream);

/* FluxMethod<Base>::ComputeStableDt(View<const Complete> states, double dx,
 * Direction dir)  include/fub/flux_method/FluxMethod.hpp:154-170, 295-382.
 * window_rule 0 = sequential tag windows, 1 = simd tag windows (the
 * reference's default OpenMpSimdTag).  Synchronises `stream`; writes the
 * minimum stable dt of the patch to *dt_out (host). */
int fvs_compute_stable_dt(const fvs_method* m, int rank,
                          const double* states_dev, fvs_box cell_box,
                          double dx, int dir, int window_rule, double* dt_out,
                          void* stream);

/* The reduction of fvs_compute_stable_dt without its synchronisation: folds
 * the patch's maximum face speed max(0, |sL|, |sR|) into *smax_bits_dev
 * (device, 8 bytes) by an atomic maximum on the bit pattern of the double
 * (non-negative doubles order like their bits; the caller zeroes the word
 * first).  Enqueued on `stream`; allocates nothing.  After the launches of
 * every patch of a level, dx / (the word as a double) is the level's stable
 * dt in `dir` -- the same number as the minimum of the patches'
 * fvs_compute_stable_dt -- with one synchronisation instead of one per patch
 * (FluxMethodAdapter.hpp:69-114 reduces the patches' dts). */
int fvs_compute_max_speed(const fvs_method* m, int rank, const double* states_dev,
                          fvs_box cell_box, int dir, int window_rule,
                          unsigned long long* smax_bits_dev, void* stream);

/* Allocation-free variant of fvs_compute_stable_dt, for callers that cannot
 * let a library allocate device memory -- for example an integrator that
 * hands out every byte of device memory through its own arena, where a
 * cudaMalloc/cudaFree behind its back would synchronise the device, escape
 * the arena's budget, and can fail once the arena holds the memory.  This
 * entry point has no counterpart in the reference (whose CPU code allocates
 * nothing on a device); it returns the same dt as fvs_compute_stable_dt, bit
 * for bit, for the HLLE methods (FVS_MUSCL_HLLE, FVS_HLLE).
 *  - Scratch: a fixed 65,544-byte array inside the library (8192 partial
 *    maxima + 1 result), held by every GPU that loads the library until the
 *    process exits.  It calls no cudaMalloc, cudaFree or other allocating
 *    routine.
 *  - Limit: at most 2,097,152 stencil windows per call (8192 blocks x 256
 *    threads); larger patches return FVS_ERR_INVALID with a message naming
 *    the limit -- split the patch or use fvs_compute_stable_dt.
 *  - The first call on each device looks up the array's device address
 *    (cudaGetSymbolAddress, with that device current); make that first call
 *    before any stream capture.  The address is kept for the life of the
 *    process: after cudaDeviceReset on a device, do not call this entry
 *    point on that device again (the kept address belongs to the context the
 *    reset destroyed).
 *  - Argument checks and status codes are those of fvs_compute_stable_dt
 *    (FVS_ERR_NO_DEVICE without a GPU); other flux methods return
 *    FVS_ERR_UNSUPPORTED.
 *  - All calls share the one array, and each call overwrites what the
 *    previous one left there (every slot it reads it has written first, so
 *    nothing needs clearing).  Calls that overlap on the GPU -- from several
 *    streams or host threads at once -- race on the array and may return a
 *    wrong dt; serialise them.
 *  - Synchronises `stream`; writes the patch's minimum stable dt to *dt_out. */
int fvs_compute_stable_dt_noalloc(const fvs_method* m, int rank,
                                  const double* states_dev, fvs_box cell_box,
                                  double dx, int dir, int window_rule,
                                  double* dt_out, void* stream);

/* HyperbolicPatchIntegrator<Tag>::UpdateConservatively(next, prev, fluxes,
 * dt, dx, dir)  include/fub/HyperbolicPatchIntegrator.hpp:34-54,
 * src/HyperbolicPatchIntegrator.cpp:35-105:
 *   next = prev + dt/dx (F[face i] - F[face i+1]), `ncomp` components.
 * next_box is the updated region; prev_box / face_box are the boxes the
 * prev / fluxes arrays are laid out over. */
int fvs_update_conservatively(double* next_dev, fvs_box next_box,
                              const double* prev_dev, fvs_box prev_box,
                              const double* fluxes_dev, fvs_box face_box,
                              int ncomp, double dt, double dx, int dir,
                              void* stream);
/* The same update on `region`, a sub-box of next_box, with next laid out over
 * next_box -- the reference's update through views of a larger FArrayBox
 * (src/AMReX/TimeIntegrator.cpp:29-56 updates the cells enclosed by the flux
 * box in place on the scratch).  next_dev may equal prev_dev (in place) when
 * next_box == prev_box. */
int fvs_update_conservatively_region(double* next_dev, fvs_box next_box, fvs_box region,
                                     const double* prev_dev, fvs_box prev_box,
                                     const double* fluxes_dev, fvs_box face_box, int ncomp,
                                     double dt, double dx, int dir, void* stream);

/* PerfectGas<D>::CompleteFromCons over `region` (src/equations/
 * PerfectGas.cpp:96-124; the scratch update of include/fub/AMReX/
 * Reconstruction.hpp:44-60).  cons: rank+2 components over cons_box,
 * complete: rank+4 components over complete_box. */
int fvs_complete_from_cons(int rank, double gamma, double* complete_dev,
                           fvs_box complete_box, const double* cons_dev,
                           fvs_box cons_box, fvs_box region, void* stream);

/* ---- Patch level with host-resident patches ---------------------------- */
/* The four patch calls above for patch arrays in host memory, the way a CPU
 * build of the reference hands FluxMethodAdapter its FArrayBoxes
 * (include/fub/AMReX/FluxMethodAdapter.hpp:120-150; HyperbolicMethod's
 * time integrator and reconstruction likewise).  A patch context owns a
 * CUDA stream and device staging buffers that grow to the largest patch it
 * has seen (the only allocations; a context reused for same-sized patches
 * allocates nothing more).  Each call copies its input boxes to the device
 * (one cudaMemcpyAsync per array), runs the device entry point on them,
 * copies its output box back and synchronises the context's stream, so the
 * host arrays are complete on return.  Results equal the device-pointer
 * calls' bit for bit.  Arguments, layouts and status codes as above; pinned
 * host memory copies fastest.  A context serves one host thread at a time. */
typedef struct fvs_patch_ctx fvs_patch_ctx;
int fvs_patch_ctx_create(fvs_patch_ctx** out);
int fvs_patch_ctx_destroy(fvs_patch_ctx* c);
int fvs_compute_numeric_fluxes_host(fvs_patch_ctx* c, const fvs_method* m, int rank,
                                    double* fluxes_host, fvs_box face_box,
                                    const double* states_host, fvs_box cell_box, double dt,
                                    double dx, int dir);
int fvs_compute_stable_dt_host(fvs_patch_ctx* c, const fvs_method* m, int rank,
                               const double* states_host, fvs_box cell_box, double dx, int dir,
                               int window_rule, double* dt_out);
int fvs_update_conservatively_host(fvs_patch_ctx* c, double* next_host, fvs_box next_box,
                                   const double* prev_host, fvs_box prev_box,
                                   const double* fluxes_host, fvs_box face_box, int ncomp,
                                   double dt, double dx, int dir);
/* Cells of complete_box outside `region` keep the values complete_host holds. */
int fvs_complete_from_cons_host(fvs_patch_ctx* c, int rank, double gamma, double* complete_host,
                                fvs_box complete_box, const double* cons_host, fvs_box cons_box,
                                fvs_box region);

/* ExactRiemannSolver<PerfectGas<1>>::ComputeMiddleState for n independent
 * problems given by primitive states (device arrays of length n)
 * (src/equations/perfect_gas/ExactRiemannSolver.hpp:34-97,
 * include/fub/NewtonIteration.hpp:28-52), with the start value of
 * m->guess, tolerance m->tolerance and at most m->max_iterations Newton
 * steps.  Outputs (device, may be NULL): p*, u*, iteration counts and a
 * status per problem (1 converged, 2 converged after the learned start was
 * rejected, 0 not converged). */
int fvs_exact_riemann_star(const fvs_method* m, int64_t n, const double* rhoL_dev,
                           const double* uL_dev, const double* pL_dev,
                           const double* rhoR_dev, const double* uR_dev,
                           const double* pR_dev, double* pstar_dev, double* ustar_dev,
                           int32_t* iterations_dev, int32_t* status_dev, void* stream);

/* ---- Solver context: a uniform single-level grid ----------------------- */

typedef struct fvs_grid_desc {
  int32_t rank;
  int32_t n[3];   /* cells per direction (1 for unused directions) */
  int32_t bc[3];  /* fvs_bc per direction */
  int32_t dt_rule;/* 0: every face; 1: the reference's MFIter tile rule */
  double dx[3];
} fvs_grid_desc;

typedef struct fvs_solver fvs_solver;

typedef struct fvs_run_stats {
  double time;          /* time point reached */
  int32_t steps;        /* committed steps */
  int32_t restarts;     /* steps redone after a failed CFL check */
  int32_t status;       /* state status bits of committed steps */
  int32_t reserved;
  double last_dt;
} fvs_run_stats;

int fvs_solver_create(const fvs_grid_desc* grid, const fvs_method* m,
                      fvs_solver** out);
int fvs_solver_destroy(fvs_solver* s);
/* Conservative state, rank+2 components, [c][nz][ny][nx], host memory. */
int fvs_solver_upload(fvs_solver* s, const double* cons_host);
/* One split step of a state that lives in host memory, in place: uploads
 * cons_host (rank+2 components, [c][nz][ny][nx]), advances it by one step as
 * fvs_solver_run does (stable dt, dt = min(cfl * stable dt, t_end - t), the
 * sweeps and their checks, a restart on a failed check) and writes the new
 * state back to cons_host.  The write-back overlaps the step's last sweep:
 * that sweep runs in slabs of its slowest transverse direction and each
 * slab is copied to the host as soon as it is final (one cudaMemcpyAsync or
 * cudaMemcpy2DAsync per component and slab), so only the last slab's copy
 * adds to the step.  Page-locked cons_host (cudaHostAlloc, cudaHostRegister)
 * lets the copies run asynchronously.  With t >= t_end nothing is advanced
 * (stats->steps 0).  Afterwards the solver's device state equals cons_host.
 * Uniform grids (no embedded boundary). */
int fvs_solver_step_host(fvs_solver* s, double* cons_host, double cfl, double t_end,
                         fvs_run_stats* stats);
int fvs_solver_download(fvs_solver* s, double* cons_host);
/* Device pointer of the current state (valid until the next call). */
int fvs_solver_state_device(fvs_solver* s, double** cons_dev);
/* Writes the current state as an AMReX plotfile directory `dir` (created if
 * missing; its files are overwritten): the Complete state (Density,
 * Momentum_d (Momentum in 1-D), Energy, Pressure, SpeedOfSound) computed on
 * the device, one level whose boxes are slabs of the slowest direction of at
 * most 2^21 cells, the solver's time and step count.  With cut cells the
 * state is masked by alpha > 0 and Boundary_X, Boundary_Y and vfrac follow.
 * Replaces fub::amrex::PlotfileOutput / WritePlotFile
 * (include/fub/AMReX/output/WritePlotfiles.hpp:33-56,
 * include/fub/AMReX/PatchHierarchy.hpp:278-315,
 * include/fub/AMReX/cutcell/PatchHierarchy.hpp:265-314). */
int fvs_solver_write_plotfile(fvs_solver* s, const char* dir);
/* Threads per block / cells per thread segment of the sweep kernels
 * (0 = automatic). */
int fvs_solver_set_tiling(fvs_solver* s, int seg_len);
/* Autotuner: times the sweep kernel on the current state for candidate
 * segment lengths (cells per thread along the sweep direction) and keeps
 * the fastest per direction (used unless fvs_solver_set_tiling forces one).
 * seg_out (may be NULL) receives rank values.  Does not change the state. */
int fvs_solver_autotune(fvs_solver* s, int* seg_out);
/* The tuned segment lengths and occupancy variants per direction: 0 =
 * registers as needed, 3 (double-float), 4 or 5 (mixed) = compiled for that
 * many resident 128-thread blocks per SM; for mixed x sweeps 10 + v = variant
 * v with the marching kernel instead of the lanes-along-x kernel.  Grids with
 * cut cells have variant 0 only.  Either pointer may be NULL. */
int fvs_solver_tuning(fvs_solver* s, int32_t* seg, int32_t* occupancy);
/* Forces the launch shape of direction dir, as fvs_solver_autotune would set
 * it: segment length (0 = automatic) and variant (the occupancy codes above;
 * 0 for the flavours without variants). */
int fvs_solver_set_launch(fvs_solver* s, int dir, int seg_len, int variant);
/* Stable dt of the current state: dir = -1 for the minimum over all
 * directions (DimensionalSplitLevelIntegrator::ComputeStableDt). */
int fvs_solver_stable_dt(fvs_solver* s, int dir, double* dt_out);
/* One fused sweep in `dir` with time step `dt`: fluxes + update + the CFL
 * reduction of the input state; *level_dt_out (may be NULL) receives the
 * input state's stable dt in `dir`. */
int fvs_solver_sweep(fvs_solver* s, int dir, double dt, double* level_dt_out);
/* One split step of size dt (Strang for rank >= 2; direction order reversed
 * on odd cycles).  Returns FVS_ERR_DT_TOO_LARGE (state unchanged) when a
 * per-sweep check fails. */
int fvs_solver_step(fvs_solver* s, double dt, int cycle);
/* RunSimulation without outputs: steps with dt = min(t_end - t,
 * cfl * stable_dt) until t_end or max_steps (< 0: unbounded), redoing a
 * step with the failed check's dt like the reference's backup/restart.
 * The time step stays on the device; steps run as CUDA graphs.
 * dt_log (host, may be NULL) receives up to `dt_log_len` committed dts. */
int fvs_solver_run(fvs_solver* s, double cfl, double t_end, int max_steps,
                   double* dt_log, int dt_log_len, fvs_run_stats* stats);
/* Newton iterations, non-converged faces and faces whose learned start
 * value was rejected (FVS_GUESS_MLP falls back to the PVRS start) of the
 * exact Riemann solver, accumulated by the solver's Godunov sweeps
 * (fvs_solver_sweep/step since the last reset, plus the last
 * fvs_solver_run, which restarts its count).  Any pointer may be NULL. */
int fvs_solver_newton_stats(fvs_solver* s, uint64_t* iterations, uint64_t* failures,
                            uint64_t* fallbacks, int reset);
/* The solver's CUDA stream (cudaStream_t): every solver call runs on it. */
int fvs_solver_stream(fvs_solver* s, void** stream);
/* ---- Embedded boundary: KBN h-box cut cells (rank 2) ------------------ */

/* Ghost layers of the cut-cell geometry arrays. */
int fvs_cutcell_ghost_layers(void);
/* Embeds the union of `ncircles` (1..16) circles, host array of (cx, cy, r)
 * triples, the body being their inside, into a rank-2 MUSCL-HLLE solver
 * (exact FP64, fast FP64, or mixed: FP32 reconstruction, fluxes, wall states
 * and CFL speeds with FP64 state, fractions and update) whose cell (0, 0)
 * has its lower-left corner at (x0, y0).  The FP64
 * geometry (volume / face fractions, normals, centroids, shielded fractions)
 * is computed on the device; from then on every sweep is the
 * KbnCutCellMethod update (include/fub/cutcell_method/KbnStabilisation.hpp:
 * 188-450, src/AMReX/cutcell/TimeIntegrator.cpp:65-221) with HLL boundary
 * states, and each step starts by computing the cut cells' reference
 * states (PreAdvanceHierarchy). */
int fvs_solver_set_embedded_circles(fvs_solver* s, const double* circles, int ncircles,
                                    double x0, double y0);
/* Shapes of an embedded body, the forms of the reference's geometry
 * (include/fub/geometry/Ball.hpp, Halfspace.hpp, Polygon.hpp, Invert.hpp;
 * a list of shapes is their PolymorphicUnion):
 *  circle:    p = (cx, cy, r), inside |x - c| < r;
 *  halfspace: p = (nx, ny, offset), inside n . x - offset > 0 with n
 *             normalised (src/geometry/Halfspace.cpp);
 *  polygon:   nvertices (x, y) pairs in xy (host), closed (the last vertex
 *             equals the first, as the reference requires), inside by the
 *             even-odd rule (src/geometry/Polygon.cpp); a grid line may cross
 *             it at most 64 times;
 *  inverted != 0: the body is the shape's outside (Invert). */
typedef enum fvs_shape_kind {
  FVS_SHAPE_CIRCLE = 0,
  FVS_SHAPE_HALFSPACE = 1,
  FVS_SHAPE_POLYGON = 2
} fvs_shape_kind;

typedef struct fvs_shape {
  int32_t kind;      /* fvs_shape_kind */
  int32_t inverted;
  double p[3];
  int32_t nvertices; /* polygon */
  int32_t reserved;
  const double* xy;  /* polygon: host array [nvertices][2] */
} fvs_shape;

/* Embeds the union of `nshapes` (1..256) shapes as the body of a rank-2
 * MUSCL-HLLE solver, exactly as fvs_solver_set_embedded_circles does for
 * circles (which is this call with circle shapes): the library's FP64
 * cut-cell geometry of the shapes (the reference hands them to AMReX's EB2,
 * src/AMReX/cutcell/PatchHierarchy.cpp:507-547), computed on the device. */
int fvs_solver_set_embedded_geometry(fvs_solver* s, const fvs_shape* shapes, int nshapes,
                                     double x0, double y0);
/* Copies the geometry to host arrays over the grid grown by
 * fvs_cutcell_ghost_layers() = G layers (NX = nx + 2G, NY = ny + 2G):
 * alpha [NY][NX], betax [NY][NX+1], betay [NY+1][NX], normal and center
 * [2][NY][NX], cut flags [NY][NX].  Any pointer may be NULL. */
int fvs_solver_cutcell_geometry(fvs_solver* s, double* alpha, double* betax, double* betay,
                                double* normal, double* center, int8_t* cut_flags);
/* The shielded face fractions of direction dir (FillCutCellData,
 * src/AMReX/cutcell/FillCutCellData.cpp:28-118): unshielded, left- and
 * right-shielded fractions and the same divided by the face fraction, over
 * the face array of the grown grid (betax's shape for dir 0, betay's for
 * dir 1).  Any pointer may be NULL. */
int fvs_solver_cutcell_shielded(fvs_solver* s, int dir, double* us, double* sL, double* sR,
                                double* us_rel, double* sL_rel, double* sR_rel);
/* Cycle counter used for the direction order of the next step. */
int fvs_solver_set_cycle(fvs_solver* s, int64_t cycle);
int fvs_solver_set_time(fvs_solver* s, double t);

/* ---- Batched AMR patch set (rank 2, refinement ratio 2) ---------------- */
/* The subcycled, refluxed block-structured update that the reference runs
 * with SubcycleFineFirstSolver over DimensionalSplitLevelIntegrator
 * (include/fub/solver/SubcycleFineFirstSolver.hpp:100-191,
 * include/fub/solver/DimensionalSplitLevelIntegrator.hpp:204-276) on an
 * AMReX patch hierarchy with FluxRegister refluxing and average_down
 * (src/AMReX/IntegratorContext.cpp:380-533), for a static hierarchy:
 *  - level l has (n0 << l) cells per direction of size dx0 / 2^l; level-0
 *    patches tile the domain, finer patches have even corners, do not
 *    overlap within a level, and are nested (their footprint grown by the 2
 *    ghost cells lies inside the next coarser level);
 *  - every patch of a level is advanced by one persistent kernel launch per
 *    sweep over a device-resident table of patch rows; a whole coarse step
 *    (ghost fills, stable dt, dt selection, fine-first subcycles with Strang
 *    sweeps, refluxing, average-down, per-sweep CFL checks) is one CUDA
 *    graph;
 *  - ghost cells are refilled before every sweep: same-level copies, the
 *    boundary condition (periodic wrap / transmissive clamp), and otherwise
 *    piecewise-constant injection from the coarser level's state at the
 *    start of the coarse step.
 * Methods: MUSCL-Hancock + HLLE (any limiter) in exact FP64, fast FP64 or
 * mixed precision. */
typedef struct fvs_amr fvs_amr;

typedef struct fvs_amr_desc {
  int32_t rank;           /* 2 */
  int32_t nlevels;        /* 1..4 */
  int32_t n0[3];          /* level-0 cells per direction */
  int32_t bc[3];          /* fvs_bc per direction */
  double dx0;             /* level-0 cell size */
  int32_t npatches;
  int32_t reserved;
  const int32_t* patch_level; /* [npatches] */
  const fvs_box* patch_box;   /* [npatches], in the patch level's index space */
} fvs_amr_desc;

int fvs_amr_create(const fvs_amr_desc* d, const fvs_method* m, fvs_amr** out);
int fvs_amr_destroy(fvs_amr* a);
/* Host data: the patches' interiors concatenated in patch order, each
 * [4][ny][nx] (FArrayBox layout of the patch box). */
int fvs_amr_upload(fvs_amr* a, const double* host);
int fvs_amr_download(fvs_amr* a, double* host);
/* AMReX plotfile of every level (one box per patch, in patch order; level l
 * has step count 2^l times the coarse steps), as fvs_solver_write_plotfile. */
int fvs_amr_write_plotfile(fvs_amr* a, const char* dir);
/* Interior cells and storage cells (with ghosts) per level, and the number
 * of coarse-fine register faces.  Any pointer may be NULL. */
int fvs_amr_info(fvs_amr* a, int64_t* cells_per_level, int64_t* storage_per_level,
                 int32_t* nslots);
int fvs_amr_stream(fvs_amr* a, void** stream);
/* Coarse-step stable dt: min over levels of 2^l times the level's stable dt
 * (SubcycleFineFirstSolver.hpp:100-112), without the CFL factor. */
int fvs_amr_stable_dt(fvs_amr* a, double* dt);
/* RunSimulation's loop over coarse steps: dt = min(t_end - t,
 * cfl * stable dt); a failed per-sweep check restarts the coarse step from
 * its start with cfl times 2^l times the failing level's dt. */
int fvs_amr_run(fvs_amr* a, double cfl, double t_end, int max_steps, double* dt_log,
                int log_len, fvs_run_stats* stats);
/* Persistent launch shape of a level's sweeps in direction dir: threads per
 * block, blocks, and threads per patch row (1, 2, 4 or 8: each row split into
 * that many segments; 32, mixed flavour x sweeps only: the rows laid end to
 * end with the lanes of a warp along x). */
int fvs_amr_set_launch(fvs_amr* a, int level, int dir, int block, int grid, int threads_per_row);
/* Times the sweeps of every level and direction for a set of launch shapes
 * (threads per row, threads per block, blocks, and for the mixed flavour a
 * register/occupancy variant) and keeps the fastest; results are cached per
 * process under the key (precision, direction, the level's patch-size
 * histogram), so hierarchies with the same histogram reuse them.  configs
 * (may be NULL) receives [nlevels][2 directions][block, grid, threads per
 * row]. */
int fvs_amr_autotune(fvs_amr* a, int32_t* configs);

/* ---- Learned start value of the exact Riemann solver ------------------- */
/* No counterpart in the reference: its ExactRiemannSolver starts Newton's
 * iteration from the mean pressure (src/equations/perfect_gas/
 * ExactRiemannSolver.hpp:34-97).  A 5 -> 64 -> 64 -> 1 GELU perceptron
 * predicts y = log(p* / max(pL, pR)); it is trained and evaluated with BF16
 * operands on the tcgen05 tensor cores (FP32 accumulation), and
 * fvs_mlp_params() gives the blob that fvs_method.mlp_params points to. */
typedef struct fvs_mlp fvs_mlp;

/* Number of floats in the parameter blob: mean[5], inv_std[5], W1[64][5],
 * b1[64], W2[64][64], b2[64], w3[64], b3. */
int fvs_mlp_param_count(void);
/* Deterministic uniform (He) initialisation from `seed`. */
int fvs_mlp_create(uint64_t seed, fvs_mlp** out);
int fvs_mlp_destroy(fvs_mlp* m);
/* Features (float [n][5]) of n Riemann problems given by primitive states
 * and, when pstar_dev and labels_dev are given, the labels
 * log(p* / max(pL, pR)) (float [n]).  Device arrays. */
int fvs_riemann_features(int64_t n, double gamma, const double* rhoL_dev, const double* uL_dev,
                         const double* pL_dev, const double* rhoR_dev, const double* uR_dev,
                         const double* pR_dev, const double* pstar_dev, float* features_dev,
                         float* labels_dev, void* stream);
/* Sets the standardisation (mean, 1/std) from n feature rows. */
int fvs_mlp_set_normalization(fvs_mlp* m, const float* features_dev, int64_t n);
/* `steps` Adam steps (beta 0.9 / 0.999, eps 1e-8, learning rate lr) on
 * batches of `batch` rows (a multiple of 256) drawn from the n training rows
 * by a hash of (seed, step, row); *mean_loss receives the mean squared
 * error over all rows of all steps. */
int fvs_mlp_train(fvs_mlp* m, const float* features_dev, const float* labels_dev, int64_t n,
                  int steps, int batch, float lr, uint64_t seed, float* mean_loss);
/* Gradients (host, fvs_mlp_param_count() floats in the blob layout; the
 * normalisation entries are 0) and loss of the mean squared error over the
 * first `batch` rows, without an update. */
int fvs_mlp_gradients(fvs_mlp* m, const float* features_dev, const float* labels_dev, int batch,
                      float* grads_host, float* loss_host);
/* y (device float [n]) for n feature rows, through the tensor-core path. */
int fvs_mlp_predict(fvs_mlp* m, const float* features_dev, int64_t n, float* y_dev);
/* Device pointer to the inference blob (BF16-rounded weights as floats). */
int fvs_mlp_params(fvs_mlp* m, const float** params_dev);
/* FP32 master parameters in the blob layout (host copies). */
int fvs_mlp_get_master(fvs_mlp* m, float* host);
int fvs_mlp_set_master(fvs_mlp* m, const float* host);
/* C[M x N] (+)= A[M x K] . B[N x K]^T with A, B bf16 (K contiguous, 16-byte
 * aligned rows) and C fp32, on the tcgen05 tensor cores; N in {16, 32, 64},
 * K a multiple of 16; splits > 1 splits K and needs accumulate = 1. */
int fvs_tc_gemm_bf16(const void* A_dev, int lda, const void* B_dev, int ldb, float* C_dev, int ldc,
                     int M, int N, int K, int splits, int accumulate, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FVS_GPU_H */
