// Compile-and-run check of include/fvs_gpu.hpp: a one-patch fake integrator
// context drives the shim's context-level members through the C ABI.
//   no argument: no GPU expected -- every call must raise fvs_gpu::Error
//                with FVS_ERR_NO_DEVICE;
//   "gpu":       a uniform 2-D state on one 16x8 patch: the stable dt is
//                dx / (|u| + c), the fluxes are the physical flux, and the
//                update and CompleteFromCons leave the state unchanged.
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
  return NoDevice();
}
