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

#include <cuda_runtime_api.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

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

inline void CheckCuda(cudaError_t e) {
  if (e != cudaSuccess) throw Error(FVS_ERR_CUDA, cudaGetErrorString(e));
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
  // rule, the reference's default OpenMpSimdTag): every patch folds its
  // maximum face speed into one device word (fvs_compute_max_speed), the
  // level synchronises once, dt = dx / max speed (the minimum of the
  // patches' dts: division by a positive number is monotonic).  Patches on
  // other streams wait for the word's reset and are waited for.
  template <class Context, class Direction>
  Duration ComputeStableDt(Context& ctx, int level, Direction dir) {
    const int d = static_cast<int>(dir);
    const double dx = adapter_.CellSize(ctx, level, d);
    if (fvs_device_count() == 0) throw Error(FVS_ERR_NO_DEVICE, "no CUDA device available");
    std::vector<cudaStream_t> streams;
    adapter_.ForEachPatch(ctx, level, d, [&](const Patch& p) {
      const cudaStream_t s = static_cast<cudaStream_t>(p.stream);
      if (std::find(streams.begin(), streams.end(), s) == streams.end()) streams.push_back(s);
    });
    if (streams.empty()) return Duration(std::numeric_limits<double>::max());
    Reduction& r = reduction();
    const cudaStream_t s0 = streams.front();
    CheckCuda(cudaMemsetAsync(r.word, 0, sizeof(unsigned long long), s0));
    CheckCuda(cudaEventRecord(r.ready, s0));
    for (size_t k = 1; k < streams.size(); ++k) CheckCuda(cudaStreamWaitEvent(streams[k], r.ready, 0));
    adapter_.ForEachPatch(ctx, level, d, [&](const Patch& p) {
      Check(fvs_compute_max_speed(&m_, adapter_.Rank(), p.scratch, p.scratch_box, d, 1, r.word,
                                  p.stream));
    });
    for (size_t k = 1; k < streams.size(); ++k) {
      CheckCuda(cudaEventRecord(r.done, streams[k]));
      CheckCuda(cudaStreamWaitEvent(s0, r.done, 0));
    }
    unsigned long long bits = 0;
    CheckCuda(cudaMemcpyAsync(&bits, r.word, sizeof bits, cudaMemcpyDeviceToHost, s0));
    CheckCuda(cudaStreamSynchronize(s0));
    double smax;
    std::memcpy(&smax, &bits, sizeof smax);
    return Duration(smax > 0.0 ? dx / smax : std::numeric_limits<double>::infinity());
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
  // the level reduction's device word and events, made on first use and
  // shared by copies of the flux method (the reference copies methods)
  struct Reduction {
    unsigned long long* word = nullptr;
    cudaEvent_t ready = nullptr, done = nullptr;
    ~Reduction() {
      if (word) cudaFree(word);
      if (ready) cudaEventDestroy(ready);
      if (done) cudaEventDestroy(done);
    }
  };
  Reduction& reduction() {
    if (!reduction_) {
      auto r = std::make_shared<Reduction>();
      CheckCuda(cudaMalloc(reinterpret_cast<void**>(&r->word), sizeof(unsigned long long)));
      CheckCuda(cudaEventCreateWithFlags(&r->ready, cudaEventDisableTiming));
      CheckCuda(cudaEventCreateWithFlags(&r->done, cudaEventDisableTiming));
      reduction_ = std::move(r);
    }
    return *reduction_;
  }

  fvs_method m_{};
  Adapter adapter_;
  std::shared_ptr<Reduction> reduction_;
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
