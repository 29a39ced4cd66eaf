// Compile-and-run check of include/fvs_gpu.hpp: a one-patch fake integrator
// context drives the shim's context-level members through the C ABI.
//   no argument: no GPU expected -- every call must raise fvs_gpu::Error
//                with FVS_ERR_NO_DEVICE;
//   "gpu":       a uniform 2-D state on one 16x8 patch: the stable dt is
//                dx / (|u| + c), the fluxes are the physical flux, and the
//                update and CompleteFromCons leave the state unchanged;
//   "patches IN OUT": a level of several patches read from file IN (doubles:
//                nx, ny, ghosts, npatch, dx, then each patch's Complete
//                scratch, 6 x (ny + 2g) x (nx + 2g)), each on its own CUDA
//                stream: the level's stable dt in x, the x fluxes with half
//                of it, the update and CompleteFromCons; writes to OUT the dt,
//                then each patch's fluxes and its scratch.
#include <cuda_runtime_api.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "fvs_gpu.hpp"

namespace {

enum class Direction { X = 0, Y = 1 };

struct FakeContext {
  fvs_gpu::Patch patch;
  double dx = 1.0 / 16;
};

struct OnePatchAdapter {
  int Rank() const { return 2; }
  double Gamma() const { return 1.4; }
  double CellSize(FakeContext& c, int, int) { return c.dx; }
  template <class F> void ForEachPatch(FakeContext& c, int, int, F&& f) { f(c.patch); }
};

struct LevelContext {
  std::vector<fvs_gpu::Patch> patches;
  double dx = 0.0;
};

struct LevelAdapter {
  int Rank() const { return 2; }
  double Gamma() const { return 1.4; }
  double CellSize(LevelContext& c, int, int) { return c.dx; }
  template <class F> void ForEachPatch(LevelContext& c, int, int, F&& f) {
    for (const fvs_gpu::Patch& p : c.patches) f(p);
  }
};

int Patches(const char* in_path, const char* out_path) {
  std::FILE* in = std::fopen(in_path, "rb");
  if (!in) return 3;
  double head[5];
  if (std::fread(head, sizeof(double), 5, in) != 5) return 3;
  const int nx = int(head[0]), ny = int(head[1]), g = int(head[2]), np = int(head[3]);
  const int NX = nx + 2 * g, NY = ny + 2 * g;
  const size_t nscr = size_t(6) * NX * NY, nflux = size_t(4) * (nx + 1) * ny;
  LevelContext ctx;
  ctx.dx = head[4];
  std::vector<double*> dev_s(np), dev_f(np);
  std::vector<cudaStream_t> streams(np);
  std::vector<double> h(nscr);
  for (int p = 0; p < np; ++p) {
    if (std::fread(h.data(), sizeof(double), nscr, in) != nscr) return 3;
    if (cudaStreamCreate(&streams[p]) != cudaSuccess ||
        cudaMalloc(reinterpret_cast<void**>(&dev_s[p]), nscr * sizeof(double)) != cudaSuccess ||
        cudaMalloc(reinterpret_cast<void**>(&dev_f[p]), nflux * sizeof(double)) != cudaSuccess)
      return 2;
    cudaMemcpy(dev_s[p], h.data(), nscr * sizeof(double), cudaMemcpyHostToDevice);
    fvs_gpu::Patch pt{};
    pt.scratch = dev_s[p];
    pt.scratch_box = {{-g, -g, 0}, {nx + g, ny + g, 1}};
    pt.valid_box = {{0, 0, 0}, {nx, ny, 1}};
    pt.fluxes = dev_f[p];
    pt.flux_box = {{0, 0, 0}, {nx + 1, ny, 1}};
    pt.stream = streams[p];
    ctx.patches.push_back(pt);
  }
  std::fclose(in);
  fvs_gpu::FluxMethod<LevelAdapter> fm;
  fvs_gpu::TimeIntegrator<LevelAdapter> ti;
  fvs_gpu::Reconstruction<LevelAdapter> rc;
  const double dt = fm.ComputeStableDt(ctx, 0, Direction::X).count();
  fm.ComputeNumericFluxes(ctx, 0, fvs_gpu::Duration(0.5 * dt), Direction::X);
  ti.UpdateConservatively(ctx, 0, fvs_gpu::Duration(0.5 * dt), Direction::X);
  rc.CompleteFromCons(ctx, 0, fvs_gpu::Duration(0.5 * dt));
  if (cudaDeviceSynchronize() != cudaSuccess) return 2;
  std::FILE* out = std::fopen(out_path, "wb");
  if (!out) return 3;
  std::fwrite(&dt, sizeof(double), 1, out);
  std::vector<double> f(nflux);
  for (int p = 0; p < np; ++p) {
    cudaMemcpy(f.data(), dev_f[p], nflux * sizeof(double), cudaMemcpyDeviceToHost);
    cudaMemcpy(h.data(), dev_s[p], nscr * sizeof(double), cudaMemcpyDeviceToHost);
    std::fwrite(f.data(), sizeof(double), nflux, out);
    std::fwrite(h.data(), sizeof(double), nscr, out);
    cudaFree(dev_s[p]);
    cudaFree(dev_f[p]);
    cudaStreamDestroy(streams[p]);
  }
  std::fclose(out);
  std::printf("patches %d dt %.17g\n", np, dt);
  return 0;
}

int NoDevice() {
  FakeContext ctx{};
  std::vector<double> dummy(4096, 1.0);
  ctx.patch.scratch = dummy.data();
  ctx.patch.scratch_box = {{-2, -2, 0}, {18, 10, 1}};
  ctx.patch.valid_box = {{0, 0, 0}, {16, 8, 1}};
  ctx.patch.fluxes = dummy.data();
  ctx.patch.flux_box = {{0, 0, 0}, {17, 8, 1}};
  fvs_gpu::FluxMethod<OnePatchAdapter> fm;
  int raised = 0;
  try {
    fm.ComputeStableDt(ctx, 0, Direction::X);
  } catch (const fvs_gpu::Error& e) {
    raised += e.code() == FVS_ERR_NO_DEVICE;
  }
  try {
    fm.ComputeNumericFluxes(ctx, 0, fvs_gpu::Duration(1e-3), Direction::X);
  } catch (const fvs_gpu::Error& e) {
    raised += e.code() == FVS_ERR_NO_DEVICE;
  }
  std::printf("stencil %d raised %d\n", fm.GetStencilWidth(), raised);
  return (raised == 2 && fm.GetStencilWidth() == 2) ? 0 : 1;
}

int WithGpu() {
  const int nx = 16, ny = 8, g = 2;
  const int NX = nx + 2 * g, NY = ny + 2 * g;
  const double rho = 1.2, u = 0.3, v = -0.2, p = 0.9, gamma = 1.4;
  const double E = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v);
  const double c = std::sqrt(gamma * p / rho);
  std::vector<double> h(size_t(6) * NX * NY);
  const double vals[6] = {rho, rho * u, rho * v, E, p, c};
  for (int k = 0; k < 6; ++k)
    for (int i = 0; i < NX * NY; ++i) h[size_t(k) * NX * NY + i] = vals[k];
  double *d_state = nullptr, *d_flux = nullptr;
  const size_t nflux = size_t(4) * (nx + 1) * ny;
  if (cudaMalloc(reinterpret_cast<void**>(&d_state), h.size() * sizeof(double)) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void**>(&d_flux), nflux * sizeof(double)) != cudaSuccess)
    return 2;
  cudaMemcpy(d_state, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice);
  FakeContext ctx{};
  ctx.patch.scratch = d_state;
  ctx.patch.scratch_box = {{-g, -g, 0}, {nx + g, ny + g, 1}};
  ctx.patch.valid_box = {{0, 0, 0}, {nx, ny, 1}};
  ctx.patch.fluxes = d_flux;
  ctx.patch.flux_box = {{0, 0, 0}, {nx + 1, ny, 1}};
  ctx.patch.stream = nullptr;
  fvs_gpu::FluxMethod<OnePatchAdapter> fm;
  fvs_gpu::TimeIntegrator<OnePatchAdapter> ti;
  fvs_gpu::Reconstruction<OnePatchAdapter> rc;
  const double dt = fm.ComputeStableDt(ctx, 0, Direction::X).count();
  fm.ComputeNumericFluxes(ctx, 0, fvs_gpu::Duration(0.5 * dt), Direction::X);
  ti.UpdateConservatively(ctx, 0, fvs_gpu::Duration(0.5 * dt), Direction::X);
  rc.CompleteFromCons(ctx, 0, fvs_gpu::Duration(0.5 * dt));
  std::vector<double> f(nflux), out(h.size());
  cudaMemcpy(f.data(), d_flux, nflux * sizeof(double), cudaMemcpyDeviceToHost);
  cudaMemcpy(out.data(), d_state, out.size() * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(d_state);
  cudaFree(d_flux);
  // Einfeldt speeds of two equal states: u -+ a_roe with the Roe sound speed
  // of the total enthalpy, a_roe^2 = c^2 + (gamma - 1) v^2 / 2
  // (src/equations/perfect_gas/EinfeldtSignalVelocities.hpp:25-62)
  const double a_roe = std::sqrt(c * c + 0.5 * (gamma - 1.0) * v * v);
  const double dt_expected = ctx.dx / (std::fabs(u) + a_roe);
  const double flux[4] = {rho * u, rho * u * u + p, rho * u * v, u * (E + p)};
  double err = std::fabs(dt - dt_expected) / dt_expected;
  for (int k = 0; k < 4; ++k)
    for (int i = 0; i < (nx + 1) * ny; ++i)
      err = std::max(err, std::fabs(f[size_t(k) * (nx + 1) * ny + i] - flux[k]) /
                              (std::fabs(flux[k]) + 1.0));
  for (size_t i = 0; i < out.size(); ++i)
    err = std::max(err, std::fabs(out[i] - h[i]) / (std::fabs(h[i]) + 1.0));
  std::printf("dt %.17g expected %.17g max rel err %.3g\n", dt, dt_expected, err);
  return err < 1e-13 ? 0 : 1;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc > 1 && std::strcmp(argv[1], "gpu") == 0) return WithGpu();
  if (argc > 3 && std::strcmp(argv[1], "patches") == 0) return Patches(argv[2], argv[3]);
  return NoDevice();
}
