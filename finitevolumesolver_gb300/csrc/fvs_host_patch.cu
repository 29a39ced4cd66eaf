// fvs_host_patch.cu -- the patch-level calls for patches that live in host
// memory.
//
// A CPU build of the reference hands FluxMethodAdapter host FArrayBoxes
// (include/fub/AMReX/FluxMethodAdapter.hpp:120-150): the patch arrays of
// ComputeNumericFluxes, ComputeStableDt, UpdateConservatively and
// CompleteFromCons are host memory.  A patch context owns a stream and
// device staging buffers that grow to the largest patch seen; each call
// copies its input boxes to the device (one cudaMemcpyAsync per array),
// runs the device entry point of fvs_gpu.h on the staged copies and copies
// the output box back, then synchronises the context's stream.  Results are
// those of the device-pointer calls, bit for bit.  Pinned host memory gives
// the fastest copies; pageable memory works too.
#include "../../include/fvs_gpu.h"
#include "fvs_internal.h"

#include <cstring>
#include <string>

struct fvs_patch_ctx {
  cudaStream_t stream = nullptr;
  double* buf[4] = {nullptr, nullptr, nullptr, nullptr};
  size_t cap[4] = {0, 0, 0, 0};  // doubles
  ~fvs_patch_ctx() {
    for (double* b : buf)
      if (b) cudaFree(b);
    if (stream) cudaStreamDestroy(stream);
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

bool ValidBox(const fvs_box& b) {
  for (int i = 0; i < 3; ++i)
    if (b.hi[i] < b.lo[i]) return false;
  return true;
}

size_t Cells(const fvs_box& b) {
  return size_t(b.hi[0] - b.lo[0]) * size_t(b.hi[1] - b.lo[1]) * size_t(b.hi[2] - b.lo[2]);
}

// Staging buffer k with room for n doubles (grown, never shrunk).
int Stage(fvs_patch_ctx* c, int k, size_t n, double** out) {
  if (n > c->cap[k]) {
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return CudaFail(e, "cudaStreamSynchronize");
    if (c->buf[k]) cudaFree(c->buf[k]);
    c->buf[k] = nullptr;
    c->cap[k] = 0;
    e = cudaMalloc(&c->buf[k], n * sizeof(double));
    if (e != cudaSuccess) return CudaFail(e, "cudaMalloc (patch staging)");
    c->cap[k] = n;
  }
  *out = c->buf[k];
  return FVS_OK;
}

int Upload(fvs_patch_ctx* c, double* dev, const double* host, size_t n) {
  if (n == 0) return FVS_OK;
  cudaError_t e = cudaMemcpyAsync(dev, host, n * sizeof(double), cudaMemcpyHostToDevice,
                                  c->stream);
  return e == cudaSuccess ? FVS_OK : CudaFail(e, "cudaMemcpyAsync (to device)");
}

int DownloadAndSync(fvs_patch_ctx* c, double* host, const double* dev, size_t n) {
  cudaError_t e = cudaSuccess;
  if (n > 0)
    e = cudaMemcpyAsync(host, dev, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return e == cudaSuccess ? FVS_OK : CudaFail(e, "patch copy to host");
}

}  // namespace

extern "C" {

int fvs_patch_ctx_create(fvs_patch_ctx** out) {
  if (!out) return Fail(FVS_ERR_INVALID, "NULL argument");
  *out = nullptr;
  if (int r = fvs::CheckDevice()) return r;
  fvs_patch_ctx* c = new fvs_patch_ctx();
  const cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return CudaFail(e, "cudaStreamCreate");
  }
  *out = c;
  return FVS_OK;
}

int fvs_patch_ctx_destroy(fvs_patch_ctx* c) {
  if (c) {
    cudaStreamSynchronize(c->stream);
    delete c;
  }
  return FVS_OK;
}

int fvs_compute_numeric_fluxes_host(fvs_patch_ctx* c, const fvs_method* m, int rank,
                                    double* fluxes_host, fvs_box face_box,
                                    const double* states_host, fvs_box cell_box, double dt,
                                    double dx, int dir) {
  if (!c) return Fail(FVS_ERR_INVALID, "NULL patch context");
  if (int r = fvs::CheckMethod(m, rank)) return r;
  if (!ValidBox(face_box) || !ValidBox(cell_box)) return Fail(FVS_ERR_INVALID, "invalid box");
  if (Cells(face_box) == 0) return FVS_OK;
  if (!fluxes_host || !states_host) return Fail(FVS_ERR_INVALID, "NULL data pointer");
  const size_t nf = Cells(face_box) * size_t(rank + 2), ns = Cells(cell_box) * size_t(rank + 4);
  double *df = nullptr, *ds = nullptr;
  if (int r = Stage(c, 0, ns, &ds)) return r;
  if (int r = Stage(c, 1, nf, &df)) return r;
  if (int r = Upload(c, ds, states_host, ns)) return r;
  if (int r = fvs_compute_numeric_fluxes(m, rank, df, face_box, ds, cell_box, dt, dx, dir,
                                         c->stream))
    return r;
  return DownloadAndSync(c, fluxes_host, df, nf);
}

int fvs_compute_stable_dt_host(fvs_patch_ctx* c, const fvs_method* m, int rank,
                               const double* states_host, fvs_box cell_box, double dx, int dir,
                               int window_rule, double* dt_out) {
  if (!c) return Fail(FVS_ERR_INVALID, "NULL patch context");
  if (int r = fvs::CheckMethod(m, rank)) return r;
  if (!ValidBox(cell_box)) return Fail(FVS_ERR_INVALID, "invalid box");
  if (!states_host || !dt_out) return Fail(FVS_ERR_INVALID, "NULL data pointer");
  const size_t ns = Cells(cell_box) * size_t(rank + 4);
  double* ds = nullptr;
  if (int r = Stage(c, 0, ns > 0 ? ns : 1, &ds)) return r;
  if (int r = Upload(c, ds, states_host, ns)) return r;
  // synchronises the stream and writes *dt_out
  return fvs_compute_stable_dt(m, rank, ds, cell_box, dx, dir, window_rule, dt_out, c->stream);
}

int fvs_update_conservatively_host(fvs_patch_ctx* c, double* next_host, fvs_box next_box,
                                   const double* prev_host, fvs_box prev_box,
                                   const double* fluxes_host, fvs_box face_box, int ncomp,
                                   double dt, double dx, int dir) {
  if (!c) return Fail(FVS_ERR_INVALID, "NULL patch context");
  if (ncomp < 1) return Fail(FVS_ERR_INVALID, "ncomp must be positive");
  if (!ValidBox(next_box) || !ValidBox(prev_box) || !ValidBox(face_box))
    return Fail(FVS_ERR_INVALID, "invalid box");
  if (Cells(next_box) == 0) return FVS_OK;
  if (!next_host || !prev_host || !fluxes_host) return Fail(FVS_ERR_INVALID, "NULL data pointer");
  const size_t nn = Cells(next_box) * size_t(ncomp), np = Cells(prev_box) * size_t(ncomp),
               nf = Cells(face_box) * size_t(ncomp);
  double *dn = nullptr, *dp = nullptr, *df = nullptr;
  if (int r = Stage(c, 0, np, &dp)) return r;
  if (int r = Stage(c, 1, nf, &df)) return r;
  if (int r = Stage(c, 2, nn, &dn)) return r;
  if (int r = Upload(c, dp, prev_host, np)) return r;
  if (int r = Upload(c, df, fluxes_host, nf)) return r;
  if (int r = fvs_update_conservatively(dn, next_box, dp, prev_box, df, face_box, ncomp, dt, dx,
                                        dir, c->stream))
    return r;
  return DownloadAndSync(c, next_host, dn, nn);
}

int fvs_complete_from_cons_host(fvs_patch_ctx* c, int rank, double gamma, double* complete_host,
                                fvs_box complete_box, const double* cons_host, fvs_box cons_box,
                                fvs_box region) {
  if (!c) return Fail(FVS_ERR_INVALID, "NULL patch context");
  if (rank < 1 || rank > 3) return Fail(FVS_ERR_INVALID, "rank must be 1, 2 or 3");
  if (!ValidBox(complete_box) || !ValidBox(cons_box) || !ValidBox(region))
    return Fail(FVS_ERR_INVALID, "invalid box");
  if (Cells(region) == 0) return FVS_OK;
  if (!complete_host || !cons_host) return Fail(FVS_ERR_INVALID, "NULL data pointer");
  const size_t nq = Cells(complete_box) * size_t(rank + 4), nu = Cells(cons_box) * size_t(rank + 2);
  double *dq = nullptr, *du = nullptr;
  if (int r = Stage(c, 0, nu, &du)) return r;
  if (int r = Stage(c, 3, nq, &dq)) return r;
  if (int r = Upload(c, du, cons_host, nu)) return r;
  // cells of complete_box outside `region` keep the caller's values
  if (int r = Upload(c, dq, complete_host, nq)) return r;
  if (int r = fvs_complete_from_cons(rank, gamma, dq, complete_box, du, cons_box, region,
                                     c->stream))
    return r;
  return DownloadAndSync(c, complete_host, dq, nq);
}

}  // extern "C"
