// Writes a small two-level 2-D plotfile with the library's plotfile writer
// (finitevolumesolver_gb300/csrc/fvs_plotfile.cpp) for the format test:
// value of component c at cell (i, j) of box b on level l =
// 1000 c + 100 l + 10 b + (i - lo_x) + 0.5 (j - lo_y).
#include <cstdio>
#include <vector>

#include "fvs_plotfile.h"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  using namespace fvs::plot;
  Plotfile pf;
  pf.dir = argv[1];
  pf.dim = 2;
  pf.time = 0.125;
  pf.prob_hi[0] = 1.0;
  pf.prob_hi[1] = 0.75;
  pf.vars = CompleteNames(2);
  Level l0{};
  l0.domain = Box{{0, 0, 0}, {7, 5, 0}};
  l0.dx[0] = l0.dx[1] = 0.125;
  l0.step = 3;
  l0.ratio_to_next = 2;
  l0.boxes = {Box{{0, 0, 0}, {3, 5, 0}}, Box{{4, 0, 0}, {7, 5, 0}}};
  Level l1{};
  l1.domain = Box{{0, 0, 0}, {15, 11, 0}};
  l1.dx[0] = l1.dx[1] = 0.0625;
  l1.step = 6;
  l1.ratio_to_next = 2;
  l1.boxes = {Box{{4, 2, 0}, {9, 5, 0}}};
  pf.levels = {l0, l1};
  if (!WriteHeader(pf).empty()) return 1;
  for (int l = 0; l < 2; ++l) {
    LevelWriter w(pf, l);
    int b = 0;
    for (const Box& box : pf.levels[l].boxes) {
      const int nx = box.hi[0] - box.lo[0] + 1, ny = box.hi[1] - box.lo[1] + 1;
      std::vector<double> v;
      for (size_t c = 0; c < pf.vars.size(); ++c)
        for (int j = 0; j < ny; ++j)
          for (int i = 0; i < nx; ++i) v.push_back(1000.0 * c + 100 * l + 10 * b + i + 0.5 * j);
      if (!w.Append(b++, v.data()).empty()) return 1;
    }
    if (!w.Finish().empty()) return 1;
  }
  std::printf("plotfile written\n");
  return 0;
}
