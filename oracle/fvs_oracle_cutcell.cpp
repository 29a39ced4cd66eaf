// fvs_oracle_cutcell.cpp -- CPU oracle of the KBN h-box cut-cell update
// (2-D perfect gas, MUSCL-Hancock + HLLE base method, HLL boundary solver).
//
// TEST INFRASTRUCTURE ONLY (see fvs_oracle.hpp).  Restates:
//   KbnCutCellMethod::PreAdvanceHierarchy     include/fub/cutcell_method/KbnStabilisation.hpp:188-210
//   KbnCutCellMethod::ComputeBoundaryFlux(es) KbnStabilisation.hpp:212-273
//   KbnCutCellMethod::ComputeStableDt         KbnStabilisation.hpp:275-345
//   KbnCutCellMethod::ComputeRegularFluxes    KbnStabilisation.hpp:347-429
//   ComputeStableFluxComponents               src/cutcell_method/KbnStabilisation.cpp:55-159
//   MusclHancock masked ComputeNumericFlux    include/fub/flux_method/MusclHancockMethod.hpp:487-571
//   Hll masked ComputeNumericFlux / StableDt  include/fub/flux_method/HllMethod.hpp:295-365
//   cutcell UpdateConservatively_Row           src/AMReX/cutcell/TimeIntegrator.cpp:65-221
//   FillCutCellData__ (shielded fractions)     src/AMReX/cutcell/FillCutCellData.cpp:28-118
//   IsCutCell_                                 src/CutCellData.cpp:227-246
//   MakeRotation (2-D), Rotate, Reflect        include/fub/ext/Eigen.hpp:104-115,
//                                              src/equations/PerfectGas.cpp:230-300
//   masked CompleteFromCons                    include/fub/AMReX/cutcell/Reconstruction.hpp:124-157
// The boundary Riemann solver is HllMethod<PerfectGas, Einfeldt> (CTAD of
// KbnCutCellMethod(MusclHancock, HllMethod) in examples/AMReX/EB/2D/Schardin.cpp:58-61).
//
// Geometry: AMReX EB2 is not part of the reference, so this oracle computes
// its own FP64 cut-cell geometry for a union of shapes -- circles,
// half-spaces and polygons, each possibly inverted (the body is the union of
// their insides): face fractions from the exact covered intervals of
// each cell face, volume fractions as the area of the polygon formed by the
// fluid parts of the cell boundary joined by straight chords, boundary normal
// (into the fluid) and centroid (cell units, relative to the cell centre)
// from those chords; a face next to a cell without volume is closed.  The
// GPU library computes the same quantities with its own kernels; the two must
// agree bit for bit.
#include "fvs_oracle.hpp"

#include <cmath>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

using namespace fvs_oracle;

namespace {

// ---------------------------------------------------------------------------
// Geometry

struct Interval {
  double lo, hi;
};

// Shape records of the embedded body, the union of the shapes, as a flat
// array of doubles (the forms of include/fub/geometry/*: Ball, Halfspace,
// Polygon, Invert, PolymorphicUnion):
//   circle     [0, inverted, cx, cy, r]     inside: |x - c| < r
//   halfspace  [1, inverted, nx, ny, o]     inside: n . x - o > 0, n a unit vector
//                                           (Halfspace::operator(), src/geometry/Halfspace.cpp)
//   polygon    [2, inverted, nv, x_0, y_0, ..., x_{nv-1}, y_{nv-1}]
//              closed (last vertex = first), inside by the even-odd rule
//              (Polygon::ComputeDistanceTo, src/geometry/Polygon.cpp)
// `inverted` != 0: the shape's outside (Invert).
constexpr int kMaxIntervals = 64;

int ShapeWords(const double* s) { return s[0] == 2.0 ? 3 + 2 * int(s[2]) : 5; }

// Intervals of [a, b] (sorted, disjoint) inside one shape on the segment
// {fixed coordinate = c, free coordinate in [a, b]}; `vertical`: x = c.
int ShapeIntervals(const double* s, double c, double a, double b, bool vertical, Interval* out) {
  int n = 0;
  const int kind = int(s[0]);
  if (kind == 0) {
    const double cx = s[2], cy = s[3], r = s[4];
    const double d = vertical ? (c - cx) : (c - cy);
    if (std::fabs(d) < r) {
      const double h = std::sqrt(r * r - d * d);
      const double m = vertical ? cy : cx;
      double lo = m - h, hi = m + h;
      lo = lo > a ? lo : a;
      hi = hi < b ? hi : b;
      if (lo < hi) out[n++] = Interval{lo, hi};
    }
  } else if (kind == 1) {
    // phi(free) = k1 * free + k0 > 0 inside
    const double nx = s[2], ny = s[3], o = s[4];
    const double k1 = vertical ? ny : nx;
    const double k0 = (vertical ? nx : ny) * c - o;
    if (k1 == 0.0) {
      if (k0 > 0.0) out[n++] = Interval{a, b};
    } else {
      const double root = -k0 / k1;
      double lo = a, hi = b;
      if (k1 > 0.0)
        lo = root > a ? root : a;
      else
        hi = root < b ? root : b;
      if (lo < hi) out[n++] = Interval{lo, hi};
    }
  } else {
    // crossings of the polygon's edges with the line fixed = c (half-open
    // rule on the fixed coordinate, as CountCrossedLines_), sorted along it
    const int nv = int(s[2]);
    const double* xy = s + 3;
    double cr[kMaxIntervals];
    int m = 0;
    for (int e = 0; e + 1 < nv && m < kMaxIntervals; ++e) {
      const double vf = vertical ? xy[2 * e] : xy[2 * e + 1];
      const double wf = vertical ? xy[2 * e + 2] : xy[2 * e + 3];
      const double vs = vertical ? xy[2 * e + 1] : xy[2 * e];
      const double ws = vertical ? xy[2 * e + 3] : xy[2 * e + 2];
      if ((vf < c && c <= wf) || (wf < c && c <= vf)) {
        const double t = (c - vf) / (wf - vf);
        cr[m++] = (1.0 - t) * vs + t * ws;
      }
    }
    for (int i = 1; i < m; ++i) {
      const double t = cr[i];
      int j = i - 1;
      while (j >= 0 && cr[j] > t) {
        cr[j + 1] = cr[j];
        --j;
      }
      cr[j + 1] = t;
    }
    for (int i = 0; i + 1 < m && n < kMaxIntervals; i += 2) {
      double lo = cr[i] > a ? cr[i] : a;
      double hi = cr[i + 1] < b ? cr[i + 1] : b;
      if (lo < hi) out[n++] = Interval{lo, hi};
    }
  }
  if (s[1] != 0.0) {
    // complement within [a, b]
    Interval inv[kMaxIntervals];
    int k = 0;
    double pos = a;
    for (int i = 0; i < n && k < kMaxIntervals; ++i) {
      if (out[i].lo > pos) inv[k++] = Interval{pos, out[i].lo};
      pos = out[i].hi;
    }
    if (pos < b && k < kMaxIntervals) inv[k++] = Interval{pos, b};
    for (int i = 0; i < k; ++i) out[i] = inv[i];
    n = k;
  }
  return n;
}

// Covered intervals of the segment {fixed coordinate = c, free coordinate in
// [a, b]} by the union of the shapes (nwords doubles of records), merged and
// sorted (free-coordinate units).  `vertical`: the segment is x = c (free
// coordinate y); else y = c.
int CoveredIntervals(double c, double a, double b, bool vertical, int nwords,
                     const double* shapes, Interval* out) {
  Interval iv[kMaxIntervals];
  int n = 0;
  for (int w = 0; w < nwords && n < kMaxIntervals; w += ShapeWords(shapes + w)) {
    Interval part[kMaxIntervals];
    const int k = ShapeIntervals(shapes + w, c, a, b, vertical, part);
    for (int i = 0; i < k && n < kMaxIntervals; ++i) iv[n++] = part[i];
  }
  // insertion sort by lower end (stable)
  for (int i = 1; i < n; ++i) {
    Interval t = iv[i];
    int j = i - 1;
    while (j >= 0 && iv[j].lo > t.lo) {
      iv[j + 1] = iv[j];
      --j;
    }
    iv[j + 1] = t;
  }
  int m = 0;
  for (int i = 0; i < n; ++i) {
    if (m > 0 && iv[i].lo <= out[m - 1].hi) {
      if (iv[i].hi > out[m - 1].hi) out[m - 1].hi = iv[i].hi;
    } else {
      out[m++] = iv[i];
    }
  }
  return m;
}

// Fluid fraction of a face from its covered intervals.
double FaceFraction(const Interval* iv, int n, double a, double b) {
  double cov = 0.0;
  for (int i = 0; i < n; ++i) cov = cov + (iv[i].hi - iv[i].lo);
  const double len = b - a;
  return (len - cov) / len;
}

// A point on the cell perimeter: edge e (0 bottom, 1 right, 2 top, 3 left,
// walked counter-clockwise) and the distance t in [0, 1) (cell units) from
// the edge's start corner; t = 1 is stored as t = 0 of the next edge.
struct PerimPoint {
  int e;
  double t;
};

PerimPoint MakePoint(int e, double t) {
  if (t >= 1.0) return PerimPoint{(e + 1) % 4, 0.0};
  return PerimPoint{e, t};
}

bool Same(const PerimPoint& a, const PerimPoint& b) { return a.e == b.e && a.t == b.t; }

// Perimeter length walked forward from a to b (cell units, cyclic).
double ForwardLength(const PerimPoint& a, const PerimPoint& b) {
  if (b.e == a.e && b.t >= a.t) return b.t - a.t;
  return (1.0 - a.t) + double((b.e - a.e - 1 + 4) % 4) + b.t;
}

// Cell-local coordinates (u, v) in [-0.5, 0.5]^2 of a perimeter point.
void PerimUV(const PerimPoint& p, double& u, double& v) {
  switch (p.e) {
  case 0:
    u = -0.5 + p.t;
    v = -0.5;
    break;
  case 1:
    u = 0.5;
    v = -0.5 + p.t;
    break;
  case 2:
    u = 0.5 - p.t;
    v = 0.5;
    break;
  default:
    u = -0.5;
    v = 0.5 - p.t;
    break;
  }
}

struct CellGeom {
  double alpha;
  double nx, ny;  // boundary normal into the fluid (unit), 0 if none
  double cx, cy;  // boundary centroid, cell units relative to the centre
};

// Position of v on a cell edge [a, b] of length h as a fraction of the edge,
// walked from a (EdgeFrac) or from b (EdgeFracRev): the ends exactly 0 and 1
// -- an interval clamped to an edge end stops there, and the perimeter walk
// must see it meet the next edge's interval (a - b + h need not round to 0)
// -- else (v - a) / h or (b - v) / h.
inline double EdgeFrac(double v, double a, double b, double h) {
  if (v == a) return 0.0;
  if (v == b) return 1.0;
  return (v - a) / h;
}
inline double EdgeFracRev(double v, double a, double b, double h) {
  if (v == b) return 0.0;
  if (v == a) return 1.0;
  return (b - v) / h;
}

// Volume fraction, normal and centroid of the cell [xa, xa+dx] x [ya, ya+dy].
// Covered arcs of the perimeter are joined by straight chords; the fluid
// region is the polygon made of the fluid perimeter arcs and the chords.
CellGeom ComputeCell(double xa, double ya, double dx, double dy, int nwords,
                     const double* shapes) {
  const double xb = xa + dx, yb = ya + dy;
  PerimPoint lo[256], hi[256];
  int nc = 0;
  Interval iv[64];
  // bottom: y = ya, walked with x increasing
  int n = CoveredIntervals(ya, xa, xb, false, nwords, shapes, iv);
  for (int i = 0; i < n; ++i) {
    lo[nc] = MakePoint(0, EdgeFrac(iv[i].lo, xa, xb, dx));
    hi[nc] = MakePoint(0, EdgeFrac(iv[i].hi, xa, xb, dx));
    ++nc;
  }
  // right: x = xb, y increasing
  n = CoveredIntervals(xb, ya, yb, true, nwords, shapes, iv);
  for (int i = 0; i < n; ++i) {
    lo[nc] = MakePoint(1, EdgeFrac(iv[i].lo, ya, yb, dy));
    hi[nc] = MakePoint(1, EdgeFrac(iv[i].hi, ya, yb, dy));
    ++nc;
  }
  // top: y = yb, x decreasing
  n = CoveredIntervals(yb, xa, xb, false, nwords, shapes, iv);
  for (int i = n - 1; i >= 0; --i) {
    lo[nc] = MakePoint(2, EdgeFracRev(iv[i].hi, xa, xb, dx));
    hi[nc] = MakePoint(2, EdgeFracRev(iv[i].lo, xa, xb, dx));
    ++nc;
  }
  // left: x = xa, y decreasing
  n = CoveredIntervals(xa, ya, yb, true, nwords, shapes, iv);
  for (int i = n - 1; i >= 0; --i) {
    lo[nc] = MakePoint(3, EdgeFracRev(iv[i].hi, ya, yb, dy));
    hi[nc] = MakePoint(3, EdgeFracRev(iv[i].lo, ya, yb, dy));
    ++nc;
  }
  CellGeom g{1.0, 0.0, 0.0, 0.0, 0.0};
  if (nc == 0) return g;
  // join arcs that touch at a corner
  int m = 0;
  for (int i = 0; i < nc; ++i) {
    if (m > 0 && Same(hi[m - 1], lo[i])) {
      hi[m - 1] = hi[i];
    } else {
      lo[m] = lo[i];
      hi[m] = hi[i];
      ++m;
    }
  }
  if (m > 1 && Same(hi[m - 1], lo[0])) {  // the last arc runs on into the first
    lo[0] = lo[m - 1];
    --m;
  }
  double covered = 0.0;
  for (int i = 0; i < m; ++i) covered = covered + ForwardLength(lo[i], hi[i]);
  if (m == 1 && Same(lo[0], hi[0])) covered = 4.0;
  if (covered >= 4.0) {
    g.alpha = 0.0;
    return g;
  }
  // polygon: for each covered arc its chord (lo -> hi), then the corners of
  // the fluid arc up to the next covered arc
  double pu[512], pv[512];
  int np = 0;
  double snx = 0.0, sny = 0.0, sl = 0.0, scx = 0.0, scy = 0.0;
  for (int j = 0; j < m; ++j) {
    double ua, va, ub, vb;
    PerimUV(lo[j], ua, va);
    PerimUV(hi[j], ub, vb);
    pu[np] = ua;
    pv[np] = va;
    ++np;
    pu[np] = ub;
    pv[np] = vb;
    ++np;
    // chord and its left normal (into the fluid), physical units
    const double lx = (ub - ua) * dx, ly = (vb - va) * dy;
    const double len = std::sqrt(lx * lx + ly * ly);
    snx = snx - ly;
    sny = sny + lx;
    sl = sl + len;
    scx = scx + 0.5 * (ua + ub) * len;
    scy = scy + 0.5 * (va + vb) * len;
    // corners strictly between hi[j] and the next arc's lo
    const PerimPoint p = hi[j];
    const PerimPoint q = lo[(j + 1) % m];
    if (!(q.e == p.e && q.t > p.t)) {
      for (int c = (p.e + 1) % 4;; c = (c + 1) % 4) {
        if (c == q.e) {
          if (q.t > 0.0) {
            PerimUV(PerimPoint{c, 0.0}, pu[np], pv[np]);
            ++np;
          }
          break;
        }
        PerimUV(PerimPoint{c, 0.0}, pu[np], pv[np]);
        ++np;
      }
    }
  }
  double a2 = 0.0;
  for (int i = 0; i < np; ++i) {
    const int k = (i + 1 < np) ? i + 1 : 0;
    a2 = a2 + (pu[i] * pv[k] - pu[k] * pv[i]);
  }
  double alpha = 0.5 * a2;
  alpha = alpha < 0.0 ? 0.0 : alpha;
  alpha = alpha > 1.0 ? 1.0 : alpha;
  g.alpha = alpha;
  const double nn = std::sqrt(snx * snx + sny * sny);
  if (nn > 0.0) {
    g.nx = snx / nn;
    g.ny = sny / nn;
  }
  if (sl > 0.0) {
    g.cx = scx / sl;
    g.cy = scy / sl;
  }
  return g;
}

}  // namespace

extern "C" {

// Geometry of the union of shapes (nwords doubles of shape records) on an
// nx x ny grid of cells [x0 + i dx, x0 + (i+1) dx] x [y0 + j dy, ...] grown
// by G ghost layers.  Outputs (component-major, x fastest, over the grown
// boxes): alpha [ny+2G][nx+2G]; betax [ny+2G][nx+2G+1] (face i between
// cells i-1 and i); betay [ny+2G+1][nx+2G]; normal [2][ny+2G][nx+2G] (into
// the fluid); center [2][ny+2G][nx+2G] (cell units).
void orc_cc_geometry_shapes(int nx, int ny, double x0, double y0, double dx, double dy, int G,
                            int nwords, const double* shapes, double* alpha, double* betax,
                            double* betay, double* normal, double* center) {
  const int NX = nx + 2 * G, NY = ny + 2 * G;
  const int64_t cells = int64_t(NX) * NY;
#pragma omp parallel for schedule(dynamic, 16)
  for (int jj = 0; jj < NY; ++jj) {
    Interval iv[64];
    for (int ii = 0; ii < NX; ++ii) {
      const double xa = x0 + double(ii - G) * dx;
      const double ya = y0 + double(jj - G) * dy;
      const CellGeom g = ComputeCell(xa, ya, dx, dy, nwords, shapes);
      const int64_t c = int64_t(jj) * NX + ii;
      alpha[c] = g.alpha;
      normal[c] = g.nx;
      normal[cells + c] = g.ny;
      center[c] = g.cx;
      center[cells + c] = g.cy;
    }
    for (int ii = 0; ii <= NX; ++ii) {
      const double xf = x0 + double(ii - G) * dx;
      const double ya = y0 + double(jj - G) * dy;
      const int n = CoveredIntervals(xf, ya, ya + dy, true, nwords, shapes, iv);
      betax[int64_t(jj) * (NX + 1) + ii] = FaceFraction(iv, n, ya, ya + dy);
    }
  }
#pragma omp parallel for schedule(dynamic, 16)
  for (int jj = 0; jj <= NY; ++jj) {
    Interval iv[64];
    for (int ii = 0; ii < NX; ++ii) {
      const double yf = y0 + double(jj - G) * dy;
      const double xa = x0 + double(ii - G) * dx;
      const int n = CoveredIntervals(yf, xa, xa + dx, false, nwords, shapes, iv);
      betay[int64_t(jj) * NX + ii] = FaceFraction(iv, n, xa, xa + dx);
    }
  }
  // A face can only carry flux between two cells that hold fluid: close the
  // faces next to a cell without volume (a thin fluid gap between two
  // circles can leave fluid on a face whose chord polygon has no area).
  for (int jj = 0; jj < NY; ++jj) {
    for (int ii = 1; ii < NX; ++ii) {
      if (alpha[int64_t(jj) * NX + ii - 1] <= 0.0 || alpha[int64_t(jj) * NX + ii] <= 0.0)
        betax[int64_t(jj) * (NX + 1) + ii] = 0.0;
    }
  }
  for (int jj = 1; jj < NY; ++jj) {
    for (int ii = 0; ii < NX; ++ii) {
      if (alpha[int64_t(jj - 1) * NX + ii] <= 0.0 || alpha[int64_t(jj) * NX + ii] <= 0.0)
        betay[int64_t(jj) * NX + ii] = 0.0;
    }
  }
}

// The same for a union of ncirc circles (cx, cy, r triples).
void orc_cc_geometry(int nx, int ny, double x0, double y0, double dx, double dy, int G,
                     int ncirc, const double* circ, double* alpha, double* betax,
                     double* betay, double* normal, double* center) {
  std::vector<double> words;
  for (int k = 0; k < ncirc; ++k) {
    const double rec[5] = {0.0, 0.0, circ[3 * k], circ[3 * k + 1], circ[3 * k + 2]};
    words.insert(words.end(), rec, rec + 5);
  }
  orc_cc_geometry_shapes(nx, ny, x0, y0, dx, dy, G, int(words.size()), words.data(), alpha,
                         betax, betay, normal, center);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// KBN cut-cell update on a uniform 2-D grid.

namespace {

constexpr int kG = 3;  // ghost layers of the geometry and state scratch

// Periodic image, transmissive boundary cell or reflective mirror cell of
// index i (extent n); see SourceIndex of the uniform grid.
inline int SourceIndexCc(int i, int n, int bc) {
  if (i >= 0 && i < n) return i;
  if (bc == 0) return ((i % n) + n) % n;
  if (bc == 2) return i < 0 ? -1 - i : 2 * n - 1 - i;
  return i < 0 ? 0 : n - 1;
}

struct CcGrid {
  int nx, ny;
  int bc[2];
  double dx[2];
  // geometry over the grown box (kG ghost layers)
  const double* alpha;     // [NY][NX]
  const double* beta[2];   // x faces [NY][NX+1], y faces [NY+1][NX]
  const double* normal;    // [2][NY][NX]
  const double* center;    // [2][NY][NX]
  int NX() const { return nx + 2 * kG; }
  int NY() const { return ny + 2 * kG; }
  int64_t C(int i, int j) const { return int64_t(j + kG) * NX() + (i + kG); }
  // face f (between cells f-1 and f along d) of the transverse index t
  int64_t F(int d, int f, int t) const {
    return d == 0 ? int64_t(t + kG) * (NX() + 1) + (f + kG)
                  : int64_t(f + kG) * NX() + (t + kG);
  }
  double Alpha(int i, int j) const { return alpha[C(i, j)]; }
  double Beta(int d, int f, int t) const { return beta[d][F(d, f, t)]; }
};

// Shielded fractions of face f along d (FillCutCellData__, FillCutCellData.cpp:28-118).
struct Shielded {
  double us, sL, sR, ds, us_rel, sL_rel, sR_rel, ds_rel;
};

Shielded ShieldedFractions(double betaL, double betaM, double betaR) {
  Shielded s;
  const double dBetaL = std::max(0.0, betaM - betaL);
  const double dBetaR = std::max(0.0, betaM - betaR);
  s.us = std::max(0.0, betaM - std::max(dBetaL, dBetaR));
  s.ds = std::min(dBetaL, dBetaR);
  s.sL = dBetaL - s.ds;
  s.sR = dBetaR - s.ds;
  betaM = betaM > 0 ? betaM : 1.0;
  s.us_rel = s.us / betaM;
  s.ds_rel = s.ds / betaM;
  s.sL_rel = s.sL / betaM;
  s.sR_rel = s.sR / betaM;
  return s;
}

Shielded FaceShielded(const CcGrid& g, int d, int f, int t) {
  return ShieldedFractions(g.Beta(d, f - 1, t), g.Beta(d, f, t), g.Beta(d, f + 1, t));
}

// IsCutCell_ (src/CutCellData.cpp:227-246).
bool IsCutCell(const CcGrid& g, int i, int j) {
  const double a = g.Alpha(i, j);
  if (a <= 0.0) return false;
  if (a < 1.0) return true;
  if (g.Beta(0, i, j) < 1.0 || g.Beta(0, i + 1, j) < 1.0) return true;
  if (g.Beta(1, j, i) < 1.0 || g.Beta(1, j + 1, i) < 1.0) return true;
  return false;
}

using C2 = Complete<2>;

// MakeRotation (include/fub/ext/Eigen.hpp:104-115) applied to the momentum:
// the rotation taking a to b.
void RotateMomentum(C2& q, const double* a, const double* b) {
  if (a[0] == -b[0] && a[1] == -b[1]) {
    q.m[0] = -q.m[0];
    q.m[1] = -q.m[1];
    return;
  }
  const double s = a[0] * b[1] - a[1] * b[0];
  const double c = a[0] * b[0] + a[1] * b[1];
  const double m0 = q.m[0], m1 = q.m[1];
  q.m[0] = c * m0 + (-s) * m1;
  q.m[1] = s * m0 + c * m1;
}

// Reflect about the unit normal e_x (PerfectGas.cpp:240-252):
// m - 2 (m . n) n.
void ReflectX(C2& r, const C2& q) {
  r = q;
  const double dot = q.m[0] * 1.0 + q.m[1] * 0.0;
  const double n0 = dot * 1.0, n1 = dot * 0.0;
  r.m[0] = q.m[0] - 2 * n0;
  r.m[1] = q.m[1] - 2 * n1;
}

// HLL solution of the half problem (reflected | state) at the wall, rotated
// back (KbnStabilisation.hpp:188-210 and 229-238, mask == 0).
C2 WallSolution(const Gas& eq, const C2& state, const double* normal) {
  const double unit[2] = {1.0, 0.0};
  C2 rot = state;
  RotateMomentum(rot, normal, unit);
  C2 refl;
  ReflectX(refl, rot);
  C2 sol;
  HllRiemannState<2>(eq, sol, refl, rot, 0);
  RotateMomentum(sol, unit, normal);
  return sol;
}

// Masked MUSCL-Hancock + HLLE flux of face f (MusclHancockMethod.hpp:487-571,
// HllMethod.hpp:295-335) for one lane.
void MaskedMusclFlux(const Gas& eq, double* nf, const C2* st, const double* alpha,
                     double beta, int limiter, double lambda_half, int dir) {
  constexpr int K = 4;
  const bool valid = beta > 0.0;
  if (!valid) {
    for (int k = 0; k < K; ++k) nf[k] = 0.0;
    return;
  }
  double u[4][K];
  for (int s = 0; s < 4; ++s) AsCons<2>(u[s], st[s]);
  C2 rec[2];
  for (int side = 0; side < 2; ++side) {
    const int c = side == 0 ? 1 : 2;
    const bool smask = alpha[c - 1] > 0.0 && alpha[c] > 0.0 && alpha[c + 1] > 0.0;
    double uL[K], uR[K];
    for (int k = 0; k < K; ++k) {
      const double sL = smask ? u[c][k] - u[c - 1][k] : 0.0;
      const double sR = smask ? u[c + 1][k] - u[c][k] : 0.0;
      double slope;
      if (limiter == kMinMod) {
        slope = MinMod(sL, sR);
      } else if (limiter == kNoLimiter) {
        slope = 0.5 * (sL + sR);  // NoLimiter, masked form (MusclHancockMethod.hpp:56-68)
      } else if (limiter == kNoGradient) {
        slope = 0.0;
      } else {
        slope = VanLeer(sL, sR);
      }
      uL[k] = u[c][k] - 0.5 * slope;
      uR[k] = u[c][k] + 0.5 * slope;
    }
    C2 qL, qR;
    CompleteFromConsMasked<2>(eq, qL, uL, true);
    CompleteFromConsMasked<2>(eq, qR, uR, true);
    double fL[K], fR[K];
    FluxMasked<2>(fL, qL, true, dir);
    FluxMasked<2>(fR, qR, true, dir);
    double w[K];
    const double* base = side == 0 ? uR : uL;
    for (int k = 0; k < K; ++k) w[k] = base[k] + lambda_half * (fL[k] - fR[k]);
    CompleteFromConsMasked<2>(eq, rec[side], w, true);
  }
  double s0, s1;
  EinfeldtMasked<2>(eq, rec[0], rec[1], true, dir, s0, s1);
  double fL[K], fR[K], qL[K], qR[K];
  FluxMasked<2>(fL, rec[0], true, dir);
  FluxMasked<2>(fR, rec[1], true, dir);
  AsCons<2>(qL, rec[0]);
  AsCons<2>(qR, rec[1]);
  const double sL = PMin(s0, 0.0);
  const double sR = PMax(s1, 0.0);
  const double sLsR = sL * sR;
  const double ds = sR - sL;
  for (int k = 0; k < K; ++k) {
    nf[k] = (sR * fL[k] - sL * fR[k] + sLsR * (qR[k] - qL[k])) / ds;
  }
}

struct CcStats {
  int64_t cut_cells = 0;
};

// Ghost-filled, masked-complete scratch of the whole grown box.
std::vector<C2> CcScratch(const CcGrid& g, const double* cons) {
  const Gas eq;
  std::vector<C2> sc(size_t(g.NX()) * g.NY());
  const int64_t n = int64_t(g.nx) * g.ny;
  for (int jj = -kG; jj < g.ny + kG; ++jj) {
    for (int ii = -kG; ii < g.nx + kG; ++ii) {
      const int si = SourceIndexCc(ii, g.nx, g.bc[0]);
      const int sj = SourceIndexCc(jj, g.ny, g.bc[1]);
      double u[4];
      for (int c = 0; c < 4; ++c) u[c] = cons[c * n + int64_t(sj) * g.nx + si];
      C2 q;
      CompleteFromConsMasked<2>(eq, q, u, g.Alpha(ii, jj) > 0.0);
      // reflective walls (cutcell::ReflectiveBoundary, ReflectiveBoundary.hpp:
      // 72-122): Reflect of the mirror cell's state, x then y, or zeros where
      // the mirror cell has no volume (the ghost's own alpha masks above)
      const bool rx = g.bc[0] == 2 && (ii < 0 || ii >= g.nx);
      const bool ry = g.bc[1] == 2 && (jj < 0 || jj >= g.ny);
      if (rx) ReflectMomentum<2>(q.m, 0);
      if (ry) ReflectMomentum<2>(q.m, 1);
      if ((rx || ry) && !(g.Alpha(si, sj) > 0.0)) q = C2{};
      sc[size_t(g.C(ii, jj))] = q;
    }
  }
  return sc;
}

}  // namespace

namespace {

inline void CellAt(int d, int c, int t, int& i, int& j) {
  if (d == 0) {
    i = c;
    j = t;
  } else {
    i = t;
    j = c;
  }
}

// KbnCutCellMethod::PreAdvanceHierarchy over the cells [-1, n+1)^2.
void ReferenceStates(const CcGrid& g, const std::vector<C2>& sc, std::vector<C2>& refs) {
  const Gas eq;
  for (int j = -1; j < g.ny + 1; ++j) {
    for (int i = -1; i < g.nx + 1; ++i) {
      if (!IsCutCell(g, i, j)) continue;
      const C2& q = sc[size_t(g.C(i, j))];
      if (!(q.rho > 0.0)) continue;
      const int64_t c = g.C(i, j);
      const double n[2] = {g.normal[c], g.normal[int64_t(g.NX()) * g.NY() + c]};
      refs[size_t(c)] = WallSolution(eq, q, n);
    }
  }
}

// ComputeBoundaryFlux (KbnStabilisation.hpp:212-244), mask == 0.
void BoundaryFlux(const Gas& eq, double* fb, const C2& state, const C2& ref,
                  const double* normal, int dir) {
  Flux<2>(fb, ref, dir);
  const C2 sol = WallSolution(eq, state, normal);
  fb[1 + dir] += sol.p - ref.p;
}

// One KBN sweep of the interior along `dir` with time step dt.
void CcSweep(const CcGrid& g, const double* cons_in, double* cons_out,
             const std::vector<C2>& refs, double dt, int dir, int limiter) {
  const Gas eq;
  const std::vector<C2> sc = CcScratch(g, cons_in);
  const int nd = dir == 0 ? g.nx : g.ny;
  const int nt = dir == 0 ? g.ny : g.nx;
  const double dx = g.dx[dir];
  const double lambda_half = 0.5 * dt / dx;
  const double dt_dx = dt / dx;
  const int64_t ncell = int64_t(g.nx) * g.ny;
  const int64_t plane = int64_t(g.NX()) * g.NY();
#pragma omp parallel for schedule(static)
  for (int t = 0; t < nt; ++t) {
    // boundary fluxes of the cells -1 .. nd
    std::vector<double> FB(size_t(nd + 2) * 4, 0.0);
    for (int c = -1; c <= nd; ++c) {
      int i, j;
      CellAt(dir, c, t, i, j);
      if (!IsCutCell(g, i, j)) continue;
      const int64_t ci = g.C(i, j);
      const double n[2] = {g.normal[ci], g.normal[plane + ci]};
      BoundaryFlux(eq, &FB[size_t(c + 1) * 4], sc[size_t(ci)], refs[size_t(ci)], n, dir);
    }
    // regular (masked MUSCL) and stabilised fluxes of the faces 0 .. nd
    std::vector<double> f(size_t(nd + 1) * 4), fs(size_t(nd + 1) * 4),
        fsL(size_t(nd + 1) * 4), fsR(size_t(nd + 1) * 4);
    for (int face = 0; face <= nd; ++face) {
      C2 st[4];
      double al[4];
      for (int q = 0; q < 4; ++q) {
        int i, j;
        CellAt(dir, face - 2 + q, t, i, j);
        st[q] = sc[size_t(g.C(i, j))];
        al[q] = g.Alpha(i, j);
      }
      double* nf = &f[size_t(face) * 4];
      MaskedMusclFlux(eq, nf, st, al, g.Beta(dir, face, t), limiter, lambda_half, dir);
      // ComputeStableFluxes_Row (KbnStabilisation.cpp:55-105)
      int il, jl, ir, jr;
      CellAt(dir, face - 1, t, il, jl);
      CellAt(dir, face, t, ir, jr);
      const double centerL = g.center[int64_t(dir) * plane + g.C(il, jl)];
      const double centerR = g.center[int64_t(dir) * plane + g.C(ir, jr)];
      const Shielded sh = FaceShielded(g, dir, face, t);
      const double dL = std::clamp(0.5 - centerL, 0.0, 1.0);
      const double dR = std::clamp(0.5 + centerR, 0.0, 1.0);
      for (int k = 0; k < 4; ++k) {
        const double fk = nf[k];
        const double sLk = dL * fk + (1.0 - dL) * FB[size_t(face) * 4 + k];
        const double sRk = dR * fk + (1.0 - dR) * FB[size_t(face + 1) * 4 + k];
        fsL[size_t(face) * 4 + k] = sLk;
        fsR[size_t(face) * 4 + k] = sRk;
        fs[size_t(face) * 4 + k] = sh.us_rel * fk + sh.sL_rel * sLk + sh.sR_rel * sRk;
      }
    }
    // UpdateConservatively_Row (src/AMReX/cutcell/TimeIntegrator.cpp:65-221)
    for (int c = 0; c < nd; ++c) {
      int i, j;
      CellAt(dir, c, t, i, j);
      const double alpha = g.Alpha(i, j);
      const int64_t out = int64_t(j) * g.nx + i;
      if (alpha == 0.0) {
        for (int k = 0; k < 4; ++k) cons_out[k * ncell + out] = 0.0;
        continue;
      }
      const double betaL = g.Beta(dir, c, t);
      const double betaR = g.Beta(dir, c + 1, t);
      const Shielded shL = FaceShielded(g, dir, c, t);
      const Shielded shR = FaceShielded(g, dir, c + 1, t);
      const double center = g.center[int64_t(dir) * plane + g.C(i, j)];
      for (int k = 0; k < 4; ++k) {
        const double prev = cons_in[k * ncell + out];
        const double fLs = fs[size_t(c) * 4 + k], fRs = fs[size_t(c + 1) * 4 + k];
        const double fLu = f[size_t(c) * 4 + k], fRu = f[size_t(c + 1) * 4 + k];
        const double fB = FB[size_t(c + 1) * 4 + k];
        const double regular = prev + dt_dx * (fLs - fRs);
        double next;
        if (betaL == betaR) {
          next = regular;
        } else if (betaL > betaR) {
          const double bus = shL.us / alpha;
          const double bsL = shL.sL / alpha;
          const double dist = 0.5 + center;
          const double dBeta = std::clamp((shL.sR * dist) / alpha, 0.0, 1.0);
          const double dF_us = fLu - fRs;
          const double dF_sL = fsL[size_t(c) * 4 + k] - fRs;
          const double dB = fLu - fB;
          next = prev + dt_dx * bus * dF_us + dt_dx * bsL * dF_sL + dt_dx * dBeta * dB;
        } else {
          const double bus = shR.us / alpha;
          const double bsR = shR.sR / alpha;
          const double dist = 0.5 - center;
          const double dBeta = std::clamp((shR.sL * dist) / alpha, 0.0, 1.0);
          const double dF_us = fLs - fRu;
          const double dF_sR = fLs - fsR[size_t(c + 1) * 4 + k];
          const double dB = fB - fRu;
          next = prev + dt_dx * bus * dF_us + dt_dx * bsR * dF_sR + dt_dx * dBeta * dB;
        }
        cons_out[k * ncell + out] = next;
      }
    }
  }
}

// KbnCutCellMethod::ComputeStableDt: faces with beta > 0, masked Einfeldt
// speeds of the two cells (KbnStabilisation.hpp:275-345, HllMethod.hpp:349-365).
double CcStableDt(const CcGrid& g, const double* cons, int dir) {
  const Gas eq;
  const std::vector<C2> sc = CcScratch(g, cons);
  const int nd = dir == 0 ? g.nx : g.ny;
  const int nt = dir == 0 ? g.ny : g.nx;
  double min_dt = std::numeric_limits<double>::infinity();
  for (int t = 0; t < nt; ++t) {
    for (int face = 0; face <= nd; ++face) {
      if (!(g.Beta(dir, face, t) > 0.0)) continue;
      int il, jl, ir, jr;
      CellAt(dir, face - 1, t, il, jl);
      CellAt(dir, face, t, ir, jr);
      double s0, s1;
      EinfeldtMasked<2>(eq, sc[size_t(g.C(il, jl))], sc[size_t(g.C(ir, jr))], true, dir, s0, s1);
      const double mx = PMax(PMax(0.0, std::abs(s0)), std::abs(s1));
      min_dt = std::min(min_dt, g.dx[dir] / mx);
    }
  }
  return min_dt;
}

CcGrid MakeCcGrid(const int32_t* n, const int32_t* bc, const double* dx,
                  const double* alpha, const double* betax, const double* betay,
                  const double* normal, const double* center) {
  CcGrid g;
  g.nx = n[0];
  g.ny = n[1];
  g.bc[0] = bc[0];
  g.bc[1] = bc[1];
  g.dx[0] = dx[0];
  g.dx[1] = dx[1];
  g.alpha = alpha;
  g.beta[0] = betax;
  g.beta[1] = betay;
  g.normal = normal;
  g.center = center;
  return g;
}

}  // namespace

extern "C" {

int orc_cc_ghost_layers(void) { return kG; }

// Shielded fractions of every face of the grown box whose two neighbours
// along the direction exist (others are left untouched): outputs have the
// layout of beta[dir]; order us, sL, sR, us_rel, sL_rel, sR_rel.
void orc_cc_shielded(int nx, int ny, int dir, const double* betax, const double* betay,
                     double* us, double* sL, double* sR, double* us_rel, double* sL_rel,
                     double* sR_rel) {
  const int32_t n[2] = {nx, ny};
  const int32_t bc[2] = {1, 1};
  const double dx[2] = {1.0, 1.0};
  const CcGrid g = MakeCcGrid(n, bc, dx, nullptr, betax, betay, nullptr, nullptr);
  const int nd = dir == 0 ? nx : ny;
  const int nt = dir == 0 ? ny : nx;
  for (int t = -kG; t < nt + kG; ++t) {
    for (int f = -kG + 1; f <= nd + kG - 1; ++f) {
      const Shielded sh = FaceShielded(g, dir, f, t);
      const int64_t idx = g.F(dir, f, t);
      us[idx] = sh.us;
      sL[idx] = sh.sL;
      sR[idx] = sh.sR;
      us_rel[idx] = sh.us_rel;
      sL_rel[idx] = sh.sL_rel;
      sR_rel[idx] = sh.sR_rel;
    }
  }
}

// Cut-cell flags (IsCutCell) of the interior cells, [ny][nx].
void orc_cc_cutcells(const int32_t* n, const double* alpha, const double* betax,
                     const double* betay, int32_t* flags) {
  const int32_t bc[2] = {1, 1};
  const double dx[2] = {1.0, 1.0};
  const CcGrid g = MakeCcGrid(n, bc, dx, alpha, betax, betay, nullptr, nullptr);
  for (int j = 0; j < g.ny; ++j)
    for (int i = 0; i < g.nx; ++i) flags[int64_t(j) * g.nx + i] = IsCutCell(g, i, j) ? 1 : 0;
}

// Reference states of the cut cells in [-1, n+1)^2 (over the grown box
// layout, Complete components [6][NY][NX]; other cells are zero).
void orc_cc_reference_states(const int32_t* n, const int32_t* bc, const double* dx,
                             const double* alpha, const double* betax, const double* betay,
                             const double* normal, const double* center, const double* cons,
                             double* refs_out) {
  const CcGrid g = MakeCcGrid(n, bc, dx, alpha, betax, betay, normal, center);
  const std::vector<C2> sc = CcScratch(g, cons);
  std::vector<C2> refs(sc.size(), C2{});
  for (auto& r : refs) r = C2{0.0, {0.0, 0.0}, 0.0, 0.0, 0.0};
  ReferenceStates(g, sc, refs);
  const int64_t plane = int64_t(g.NX()) * g.NY();
  for (int64_t c = 0; c < plane; ++c) {
    refs_out[c] = refs[size_t(c)].rho;
    refs_out[plane + c] = refs[size_t(c)].m[0];
    refs_out[2 * plane + c] = refs[size_t(c)].m[1];
    refs_out[3 * plane + c] = refs[size_t(c)].E;
    refs_out[4 * plane + c] = refs[size_t(c)].p;
    refs_out[5 * plane + c] = refs[size_t(c)].c;
  }
}

// One KBN sweep with the reference states of `cons_ref_src` (the state at the
// start of the step).
void orc_cc_sweep(const int32_t* n, const int32_t* bc, const double* dx, const double* alpha,
                  const double* betax, const double* betay, const double* normal,
                  const double* center, const double* cons_ref_src, const double* cons_in,
                  double* cons_out, double dt, int dir, int limiter, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  const CcGrid g = MakeCcGrid(n, bc, dx, alpha, betax, betay, normal, center);
  std::vector<C2> refs(size_t(g.NX()) * g.NY(), C2{0.0, {0.0, 0.0}, 0.0, 0.0, 0.0});
  ReferenceStates(g, CcScratch(g, cons_ref_src), refs);
  CcSweep(g, cons_in, cons_out, refs, dt, dir, limiter);
}

double orc_cc_stable_dt(const int32_t* n, const int32_t* bc, const double* dx,
                        const double* alpha, const double* betax, const double* betay,
                        const double* cons, int dir) {
  const CcGrid g = MakeCcGrid(n, bc, dx, alpha, betax, betay, nullptr, nullptr);
  if (dir >= 0) return CcStableDt(g, cons, dir);
  return std::min(CcStableDt(g, cons, 0), CcStableDt(g, cons, 1));
}

// Strang-split KBN run (RunSimulation without outputs; the reference states
// are recomputed at the start of every step, the per-sweep check restarts a
// step with the failed dt).  Returns the number of steps.
int orc_cc_run(const int32_t* n, const int32_t* bc, const double* dx, const double* alpha,
               const double* betax, const double* betay, const double* normal,
               const double* center, double* cons, double cfl, double t_end, int max_steps,
               int limiter, double* dt_log, int* restarts_out, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  const CcGrid g = MakeCcGrid(n, bc, dx, alpha, betax, betay, normal, center);
  const size_t total = size_t(g.nx) * g.ny * 4;
  std::vector<double> backup(total);
  double t = 0.0;
  int step = 0, restarts = 0;
  bool have_failure = false;
  double failure_dt = 0.0;
  while (t + 1e-12 < t_end && (max_steps < 0 || step < max_steps)) {
    const double stable =
        have_failure ? failure_dt : std::min(CcStableDt(g, cons, 0), CcStableDt(g, cons, 1));
    const double dt = std::min(t_end - t, cfl * stable);
    std::memcpy(backup.data(), cons, total * sizeof(double));
    std::vector<C2> refs(size_t(g.NX()) * g.NY(), C2{0.0, {0.0, 0.0}, 0.0, 0.0, 0.0});
    ReferenceStates(g, CcScratch(g, cons), refs);
    const int odd = step % 2;
    const int d0 = odd ? 1 : 0, d1 = odd ? 0 : 1;
    const int seq[4] = {d0, d1, d1, d0};
    bool failed = false;
    for (int q = 0; q < 4 && !failed; ++q) {
      const double level = CcStableDt(g, cons, seq[q]);
      if (level < 0.5 * dt) {
        failed = true;
        failure_dt = level;
        break;
      }
      std::vector<double> out(total);
      CcSweep(g, cons, out.data(), refs, 0.5 * dt, seq[q], limiter);
      std::memcpy(cons, out.data(), total * sizeof(double));
    }
    if (failed) {
      std::memcpy(cons, backup.data(), total * sizeof(double));
      have_failure = true;
      ++restarts;
      continue;
    }
    have_failure = false;
    if (dt_log) dt_log[step] = dt;
    t = t + dt;
    ++step;
  }
  if (restarts_out) *restarts_out = restarts;
  return step;
}

}  // extern "C"
