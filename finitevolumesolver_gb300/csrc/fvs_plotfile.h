// fvs_plotfile.h -- writer of AMReX plotfile directories (the layout of
// amrex::WriteMultiLevelPlotfile, which fub::amrex::WritePlotFile calls,
// include/fub/AMReX/PatchHierarchy.hpp:278-315 and
// include/fub/AMReX/cutcell/PatchHierarchy.hpp:265-314):
//
//   <dir>/Header                 "HyperCLaw-V1.1" plot header: variable
//                                names, dimension, time, levels, problem
//                                domain, refinement ratios, index domains,
//                                level steps, cell sizes, and per level the
//                                boxes in physical coordinates
//   <dir>/Level_<l>/Cell_H       VisMF (version 1) header of the level's
//                                data: component count, box array, the file
//                                and byte offset of every box, and per box
//                                the minimum and maximum of each component
//   <dir>/Level_<l>/Cell_D_00000 every box as a FAB: an ASCII line naming the
//                                number format (IEEE double, little endian),
//                                the box and the component count, then the
//                                values component by component, x fastest
//
// Host code: the caller computes the cell data on the device and hands each
// box's values over as it copies them back.
#pragma once

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace fvs {
namespace plot {

// A box of cells, inclusive corners (AMReX's smallEnd / bigEnd).
struct Box {
  int lo[3];
  int hi[3];
  int64_t Cells(int dim) const {
    int64_t n = 1;
    for (int d = 0; d < dim; ++d) n *= int64_t(hi[d] - lo[d] + 1);
    return n;
  }
};

struct Level {
  Box domain;            // index domain of the level
  double dx[3];          // cell sizes
  int step;              // level step count
  int ratio_to_next;     // refinement ratio to the next finer level
  std::vector<Box> boxes;
};

struct Plotfile {
  std::string dir;
  int dim = 3;
  double time = 0.0;
  double prob_lo[3] = {0, 0, 0};
  double prob_hi[3] = {1, 1, 1};
  std::vector<std::string> vars;
  std::vector<Level> levels;
};

// Creates the directories and writes <dir>/Header.  Returns an empty string
// on success, else a message.
std::string WriteHeader(const Plotfile& pf);

// Streams the boxes of one level into Level_<l>/Cell_D_00000 and writes
// Level_<l>/Cell_H on Finish().  Boxes are appended in the level's order.
class LevelWriter {
 public:
  LevelWriter(const Plotfile& pf, int level);
  ~LevelWriter();
  // data: [ncomp][cells of box b], x fastest
  std::string Append(int b, const double* data);
  std::string Finish();

 private:
  const Plotfile& pf_;
  int level_;
  std::FILE* f_ = nullptr;
  std::string error_;
  std::vector<int64_t> offsets_;
  std::vector<std::vector<double>> min_, max_;
};

// "Density", "Momentum_0".. (or "Momentum" in 1-D), "Energy", "Pressure",
// "SpeedOfSound": the Complete state's names with their depths
// (include/fub/equations/PerfectGas.hpp:152-161).
std::vector<std::string> CompleteNames(int rank);

}  // namespace plot
}  // namespace fvs
