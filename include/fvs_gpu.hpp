// fvs_gpu.hpp -- header-only C++17 shim over the C ABI of libfvs_gb300.
//
// It gives the reference's context-level strategy members, so that the GPU
// update drops into fub's type-erased HyperbolicMethod
// {flux_method, time_integrator, reconstruction}
// (include/fub/HyperbolicMethod.hpp:40-64, 155-159, 333-380):
//
//   FluxMethod<Adapter>::GetStencilWidth()
//   FluxMethod<Adapter>::ComputeStableDt(Context&, int level, Direction)
//   FluxMethod<Adapter>::ComputeNumericFluxes(Context&, int level, Duration, Direction)
//       -- the context-level members FluxMethodAdapter forwards to when present
//          (include/fub/AMReX/FluxMethodAdapter.hpp:72-75, 123-126);
//   TimeIntegrator<Adapter>::UpdateConservatively(Context&, int level, Duration, Direction)
//       -- TimeIntegratorBase (HyperbolicMethod.hpp:47-52), in place on the
//          scratch like src/AMReX/TimeIntegrator.cpp:29-67;
//   Reconstruction<Adapter>::CompleteFromCons(Context&, int level, Duration)
//       -- ReconstructionBase (HyperbolicMethod.hpp:40-45),
//          include/fub/AMReX/Reconstruction.hpp:44-60.
//
// The Adapter is the one piece that knows the integrator context: it visits
// the patches (MFIter tiles) of a level and hands out device pointers and
// boxes of the scratch (Complete states, rank+4 components) and of the face
// fluxes of a direction (rank+2 components), in the FArrayBox layout
// (component-major, x fastest), plus the cell size and a CUDA stream:
//
//   struct Adapter {
//     int Rank() const;
//     double Gamma() const;
//     template <class Context> double CellSize(Context&, int level, int dir);
//     template <class Context, class F>
//     void ForEachPatch(Context&, int level, int dir, F&& f);  // f(const fvs_gpu::Patch&)
//   };
//
// Errors come back as fvs_gpu::Error (a std::runtime_error), the reference's
// way of reporting failures (NewtonIteration.hpp:44-50).
#pragma once

#include <algorithm>
#include <chrono>
#include <limits>
#include <stdexcept>
#include <string>

#include "fvs_gpu.h"

namespace fvs_gpu {

using Duration = std::chrono::duration<double>;

class Error : public std::runtime_error {
 public:
  Error(int code, const char* what)
      : std::runtime_error(std::string("libfvs_gb300: ") + (what ? what : "")), code_(code) {}
  int code() const noexcept { return code_; }

 private:
  int code_;
};

inline void Check(int code) {
  if (code != FVS_OK) throw Error(code, fvs_last_error());
}

// One patch (tile) of a level, device pointers.
struct Patch {
  double* scratch;      // Complete states over scratch_box (rank+4 components)
  fvs_box scratch_box;  // the ghosted box the scratch array is laid out over
  fvs_box valid_box;    // the cells this patch updates
  double* fluxes;       // face fluxes of the visited direction (rank+2 components)
  fvs_box flux_box;     // the face box the flux array is laid out over
  void* stream;         // cudaStream_t
};

// Faces of the cells `cells` in direction dir (AMReX surroundingNodes).
inline fvs_box FacesOf(const fvs_box& cells, int dir) {
  fvs_box f = cells;
  f.hi[dir] += 1;
  return f;
}

// Cells between the faces `faces` in direction dir (AMReX enclosedCells).
inline fvs_box CellsOf(const fvs_box& faces, int dir) {
  fvs_box c = faces;
  c.hi[dir] -= 1;
  return c;
}

template <class Adapter> class FluxMethod {
 public:
  explicit FluxMethod(const fvs_method& m, Adapter adapter = Adapter{})
      : m_(m), adapter_(std::move(adapter)) {}
  explicit FluxMethod(Adapter adapter = Adapter{}) : adapter_(std::move(adapter)) {
    fvs_method_default(&m_);
    m_.gamma = adapter_.Gamma();
  }

  int GetStencilWidth() const {
    return (m_.flux_method == FVS_HLLE || m_.flux_method == FVS_GODUNOV ||
            m_.flux_method == FVS_HLLEM)
               ? 1
               : 2;
  }

  // min over the level's patches of FluxMethod::ComputeStableDt (simd window
  // rule, the reference's default OpenMpSimdTag).
  template <class Context, class Direction>
  Duration ComputeStableDt(Context& ctx, int level, Direction dir) {
    const int d = static_cast<int>(dir);
    const double dx = adapter_.CellSize(ctx, level, d);
    double dt = std::numeric_limits<double>::max();
    adapter_.ForEachPatch(ctx, level, d, [&](const Patch& p) {
      double local = 0.0;
      Check(fvs_compute_stable_dt(&m_, adapter_.Rank(), p.scratch, p.scratch_box, dx, d, 1,
                                  &local, p.stream));
      dt = std::min(dt, local);
    });
    return Duration(dt);
  }

  // Fluxes on every face of the patch's flux array (its box must leave the
  // stencil inside the scratch box).
  template <class Context, class Direction>
  void ComputeNumericFluxes(Context& ctx, int level, Duration dt, Direction dir) {
    const int d = static_cast<int>(dir);
    const double dx = adapter_.CellSize(ctx, level, d);
    adapter_.ForEachPatch(ctx, level, d, [&](const Patch& p) {
      Check(fvs_compute_numeric_fluxes(&m_, adapter_.Rank(), p.fluxes, p.flux_box, p.scratch,
                                       p.scratch_box, dt.count(), dx, d, p.stream));
    });
  }

  const fvs_method& method() const { return m_; }
  fvs_method& method() { return m_; }

 private:
  fvs_method m_{};
  Adapter adapter_;
};

template <class Adapter> class TimeIntegrator {
 public:
  explicit TimeIntegrator(Adapter adapter = Adapter{}) : adapter_(std::move(adapter)) {}

  // U' = U + dt/dx (F_i - F_{i+1}) on the cells enclosed by the patch's
  // flux box (src/AMReX/TimeIntegrator.cpp:29-56), in place on the scratch's
  // conservative components.
  template <class Context, class Direction>
  void UpdateConservatively(Context& ctx, int level, Duration dt, Direction dir) {
    const int d = static_cast<int>(dir);
    const double dx = adapter_.CellSize(ctx, level, d);
    adapter_.ForEachPatch(ctx, level, d, [&](const Patch& p) {
      Check(fvs_update_conservatively_region(p.scratch, p.scratch_box, CellsOf(p.flux_box, d),
                                             p.scratch, p.scratch_box, p.fluxes, p.flux_box,
                                             adapter_.Rank() + 2, dt.count(), dx, d,
                                             p.stream));
    });
  }

 private:
  Adapter adapter_;
};

template <class Adapter> class Reconstruction {
 public:
  explicit Reconstruction(Adapter adapter = Adapter{}) : adapter_(std::move(adapter)) {}

  // p and c of every scratch cell from its conservative components, in place.
  template <class Context> void CompleteFromCons(Context& ctx, int level, Duration) {
    adapter_.ForEachPatch(ctx, level, 0, [&](const Patch& p) {
      Check(fvs_complete_from_cons(adapter_.Rank(), adapter_.Gamma(), p.scratch, p.scratch_box,
                                   p.scratch, p.scratch_box, p.scratch_box, p.stream));
    });
  }

 private:
  Adapter adapter_;
};

}  // namespace fvs_gpu
