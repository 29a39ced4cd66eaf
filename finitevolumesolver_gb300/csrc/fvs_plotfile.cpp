// fvs_plotfile.cpp -- AMReX plotfile directories (see fvs_plotfile.h); plain
// host C++.
#include "fvs_plotfile.h"

#include <sys/stat.h>
#include <sys/types.h>

#include <cerrno>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <limits>
#include <sstream>

namespace fvs {
namespace plot {
namespace {

std::string MakeDirs(const std::string& path) {
  std::string cur;
  size_t pos = 0;
  while (pos != std::string::npos) {
    pos = path.find('/', pos + 1);
    cur = path.substr(0, pos);
    if (cur.empty()) continue;
    if (mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST)
      return "cannot create directory " + cur + ": " + std::strerror(errno);
  }
  struct stat st;
  if (stat(path.c_str(), &st) != 0 || !S_ISDIR(st.st_mode)) return path + " is not a directory";
  return {};
}

// IntVect "(a,b,c)" and Box "((lo) (hi) (0,0,0))" in AMReX's text form.
void PutIntVect(std::ostream& os, const int* v, int dim) {
  os << '(';
  for (int d = 0; d < dim; ++d) os << (d ? "," : "") << v[d];
  os << ')';
}

void PutBox(std::ostream& os, const Box& b, int dim) {
  const int zero[3] = {0, 0, 0};
  os << '(';
  PutIntVect(os, b.lo, dim);
  os << ' ';
  PutIntVect(os, b.hi, dim);
  os << ' ';
  PutIntVect(os, zero, dim);  // cell-centred index type
  os << ')';
}

std::string LevelDir(const Plotfile& pf, int l) { return pf.dir + "/Level_" + std::to_string(l); }

}  // namespace

std::vector<std::string> CompleteNames(int rank) {
  std::vector<std::string> v{"Density"};
  if (rank == 1) {
    v.push_back("Momentum");
  } else {
    for (int d = 0; d < rank; ++d) v.push_back("Momentum_" + std::to_string(d));
  }
  v.push_back("Energy");
  v.push_back("Pressure");
  v.push_back("SpeedOfSound");
  return v;
}

std::string WriteHeader(const Plotfile& pf) {
  if (std::string e = MakeDirs(pf.dir); !e.empty()) return e;
  const int nl = static_cast<int>(pf.levels.size());
  for (int l = 0; l < nl; ++l)
    if (std::string e = MakeDirs(LevelDir(pf, l)); !e.empty()) return e;
  std::ostringstream h;
  h.precision(17);
  h << "HyperCLaw-V1.1\n" << pf.vars.size() << '\n';
  for (const std::string& v : pf.vars) h << v << '\n';
  h << pf.dim << '\n' << pf.time << '\n' << nl - 1 << '\n';
  for (int d = 0; d < pf.dim; ++d) h << pf.prob_lo[d] << ' ';
  h << '\n';
  for (int d = 0; d < pf.dim; ++d) h << pf.prob_hi[d] << ' ';
  h << '\n';
  for (int l = 0; l + 1 < nl; ++l) h << pf.levels[size_t(l)].ratio_to_next << ' ';
  h << '\n';
  for (int l = 0; l < nl; ++l) {
    PutBox(h, pf.levels[size_t(l)].domain, pf.dim);
    h << ' ';
  }
  h << '\n';
  for (int l = 0; l < nl; ++l) h << pf.levels[size_t(l)].step << ' ';
  h << '\n';
  for (int l = 0; l < nl; ++l) {
    for (int d = 0; d < pf.dim; ++d) h << pf.levels[size_t(l)].dx[d] << ' ';
    h << '\n';
  }
  h << 0 << '\n';  // Cartesian coordinates
  h << "0\n";      // boundary width
  for (int l = 0; l < nl; ++l) {
    const Level& L = pf.levels[size_t(l)];
    h << l << ' ' << L.boxes.size() << ' ' << pf.time << '\n' << L.step << '\n';
    for (const Box& b : L.boxes)
      for (int d = 0; d < pf.dim; ++d)
        h << pf.prob_lo[d] + L.dx[d] * (b.lo[d] - L.domain.lo[d]) << ' '
          << pf.prob_lo[d] + L.dx[d] * (b.hi[d] + 1 - L.domain.lo[d]) << '\n';
    h << "Level_" << l << "/Cell\n";
  }
  std::ofstream f(pf.dir + "/Header", std::ios::binary | std::ios::trunc);
  if (!f) return "cannot write " + pf.dir + "/Header";
  f << h.str();
  return f.good() ? std::string() : "write error on " + pf.dir + "/Header";
}

LevelWriter::LevelWriter(const Plotfile& pf, int level) : pf_(pf), level_(level) {
  const std::string path = LevelDir(pf, level) + "/Cell_D_00000";
  f_ = std::fopen(path.c_str(), "wb");
  if (!f_) error_ = "cannot write " + path;
  const size_t nb = pf.levels[size_t(level)].boxes.size();
  min_.assign(nb, std::vector<double>(pf.vars.size(), 0.0));
  max_.assign(nb, std::vector<double>(pf.vars.size(), 0.0));
}

LevelWriter::~LevelWriter() {
  if (f_) std::fclose(f_);
}

std::string LevelWriter::Append(int b, const double* data) {
  if (!error_.empty()) return error_;
  const Level& L = pf_.levels[size_t(level_)];
  if (b != static_cast<int>(offsets_.size()) || b >= static_cast<int>(L.boxes.size()))
    return error_ = "plotfile boxes must be appended in order";
  const Box& box = L.boxes[size_t(b)];
  const int64_t n = box.Cells(pf_.dim);
  const int ncomp = static_cast<int>(pf_.vars.size());
  const long pos = std::ftell(f_);
  if (pos < 0) return error_ = "cannot tell the position in the level data file";
  offsets_.push_back(static_cast<int64_t>(pos));
  std::ostringstream h;
  // IEEE double, little-endian byte order (the native order of both hosts)
  h << "FAB ((8, (64 11 52 0 1 12 0 1023)),(8, (8 7 6 5 4 3 2 1)))";
  PutBox(h, box, pf_.dim);
  h << ' ' << ncomp << '\n';
  const std::string s = h.str();
  if (std::fwrite(s.data(), 1, s.size(), f_) != s.size() ||
      std::fwrite(data, sizeof(double), size_t(n * ncomp), f_) != size_t(n * ncomp))
    return error_ = "write error on the level data file";
  for (int c = 0; c < ncomp; ++c) {
    double lo = std::numeric_limits<double>::infinity(), hi = -lo;
    for (int64_t i = 0; i < n; ++i) {
      const double v = data[c * n + i];
      lo = v < lo ? v : lo;
      hi = v > hi ? v : hi;
    }
    min_[size_t(b)][size_t(c)] = lo;
    max_[size_t(b)][size_t(c)] = hi;
  }
  return {};
}

std::string LevelWriter::Finish() {
  if (!error_.empty()) return error_;
  const Level& L = pf_.levels[size_t(level_)];
  if (offsets_.size() != L.boxes.size()) return error_ = "plotfile level is incomplete";
  if (std::fclose(f_) != 0) {
    f_ = nullptr;
    return error_ = "write error on the level data file";
  }
  f_ = nullptr;
  std::ostringstream h;
  h << "1\n1\n" << pf_.vars.size() << "\n0\n";
  h << '(' << L.boxes.size() << " 0\n";
  for (const Box& b : L.boxes) {
    PutBox(h, b, pf_.dim);
    h << '\n';
  }
  h << ")\n";
  h << L.boxes.size() << '\n';
  for (int64_t off : offsets_) h << "FabOnDisk: Cell_D_00000 " << off << '\n';
  h << '\n';
  h << std::scientific << std::setprecision(15);
  for (const auto* mm : {&min_, &max_}) {
    h << mm->size() << ',' << pf_.vars.size() << '\n';
    for (const auto& row : *mm) {
      for (double v : row) h << v << ',';
      h << '\n';
    }
    h << '\n';
  }
  const std::string path = LevelDir(pf_, level_) + "/Cell_H";
  std::ofstream f(path, std::ios::binary | std::ios::trunc);
  if (!f) return error_ = "cannot write " + path;
  f << h.str();
  return f.good() ? std::string() : (error_ = "write error on " + path);
}

}  // namespace plot
}  // namespace fvs
