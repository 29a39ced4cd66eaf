// fvs_cutcell_geometry.cuh -- FP64 cut-cell geometry of a union of shapes
// (the embedded body is the union of their insides), one cell or face per
// thread.
//
// Shape records (flat doubles; the forms of the reference's
// include/fub/geometry/*: Ball, Halfspace, Polygon, Invert, PolymorphicUnion):
//   circle     [0, inverted, cx, cy, r]     inside: |x - c| < r
//   halfspace  [1, inverted, nx, ny, o]     inside: n . x - o > 0, n a unit vector
//                                           (src/geometry/Halfspace.cpp)
//   polygon    [2, inverted, nv, x_0, y_0, ..., x_{nv-1}, y_{nv-1}]
//              closed (last vertex = first), inside by the even-odd rule
//              (src/geometry/Polygon.cpp)
// inverted != 0: the shape's outside (Invert).
//
// AMReX's EB2 geometry generator, which the reference feeds these shapes to
// and reads its cut-cell data from (src/AMReX/cutcell/PatchHierarchy.cpp:
// 507-547), is not part of the reference tree; this is the library's own
// generator:
//  - face fraction beta: fluid length of the face / face length, from the
//    exact intervals the shapes cover on the face;
//  - volume fraction alpha: area of the polygon formed by the fluid parts of
//    the cell's perimeter with every covered perimeter piece replaced by the
//    straight chord joining its ends (shoelace formula, cell units);
//  - boundary normal: sum of the chords' left normals (pointing into the
//    fluid, the sign convention of fub's GetBoundaryNormal,
//    src/CutCellData.cpp:90-105), normalised;
//  - boundary centroid: length-weighted chord midpoints, in cell units
//    relative to the cell centre (the convention used as 0.5 +- x_B in
//    src/AMReX/cutcell/TimeIntegrator.cpp:180,202);
//  - a face next to a cell without volume is closed (beta = 0).
// The translation unit is compiled with -fmad=false so the results match the
// CPU oracle's restatement bit for bit.
#pragma once

namespace fvs {
namespace ccgeom {

constexpr int kMaxIntervals = 64;  // intervals per segment, crossings per line

struct Iv {
  double lo, hi;
};

__device__ __forceinline__ int ShapeWords(const double* s) {
  return s[0] == 2.0 ? 3 + 2 * int(s[2]) : 5;
}

// Intervals of [a, b] (sorted, disjoint) inside one shape on the segment
// {fixed = c, free in [a, b]}; `vertical`: x = c.
__device__ inline int ShapeIntervals(const double* __restrict__ s, double c, double a, double b,
                                     bool vertical, Iv* out) {
  int n = 0;
  const int kind = int(s[0]);
  if (kind == 0) {
    const double cx = s[2], cy = s[3], r = s[4];
    const double d = vertical ? (c - cx) : (c - cy);
    if (fabs(d) < r) {
      const double h = sqrt(r * r - d * d);
      const double m = vertical ? cy : cx;
      double lo = m - h, hi = m + h;
      lo = lo > a ? lo : a;
      hi = hi < b ? hi : b;
      if (lo < hi) {
        out[n].lo = lo;
        out[n].hi = hi;
        ++n;
      }
    }
  } else if (kind == 1) {
    // phi(free) = k1 * free + k0 > 0 inside
    const double nx = s[2], ny = s[3], o = s[4];
    const double k1 = vertical ? ny : nx;
    const double k0 = (vertical ? nx : ny) * c - o;
    if (k1 == 0.0) {
      if (k0 > 0.0) {
        out[n].lo = a;
        out[n].hi = b;
        ++n;
      }
    } else {
      const double root = -k0 / k1;
      double lo = a, hi = b;
      if (k1 > 0.0)
        lo = root > a ? root : a;
      else
        hi = root < b ? root : b;
      if (lo < hi) {
        out[n].lo = lo;
        out[n].hi = hi;
        ++n;
      }
    }
  } else {
    // crossings of the polygon's edges with the line fixed = c (half-open
    // rule on the fixed coordinate), sorted along the line
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
      const double lo = cr[i] > a ? cr[i] : a;
      const double hi = cr[i + 1] < b ? cr[i + 1] : b;
      if (lo < hi) {
        out[n].lo = lo;
        out[n].hi = hi;
        ++n;
      }
    }
  }
  if (s[1] != 0.0) {
    // complement within [a, b]
    Iv inv[kMaxIntervals];
    int k = 0;
    double pos = a;
    for (int i = 0; i < n && k < kMaxIntervals; ++i) {
      if (out[i].lo > pos) {
        inv[k].lo = pos;
        inv[k].hi = out[i].lo;
        ++k;
      }
      pos = out[i].hi;
    }
    if (pos < b && k < kMaxIntervals) {
      inv[k].lo = pos;
      inv[k].hi = b;
      ++k;
    }
    for (int i = 0; i < k; ++i) out[i] = inv[i];
    n = k;
  }
  return n;
}

// Merged covered intervals of the segment {fixed = c, free in [a, b]} by the
// union of the shapes (nwords doubles of records).
__device__ inline int Covered(double c, double a, double b, bool vertical, int nwords,
                              const double* __restrict__ shapes, Iv* out) {
  Iv iv[kMaxIntervals];
  int n = 0;
  for (int w = 0; w < nwords && n < kMaxIntervals; w += ShapeWords(shapes + w)) {
    Iv part[kMaxIntervals];
    const int k = ShapeIntervals(shapes + w, c, a, b, vertical, part);
    for (int i = 0; i < k && n < kMaxIntervals; ++i) iv[n++] = part[i];
  }
  for (int i = 1; i < n; ++i) {
    const Iv t = iv[i];
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

__device__ __forceinline__ double FaceFraction(const Iv* iv, int n, double a, double b) {
  double cov = 0.0;
  for (int i = 0; i < n; ++i) cov = cov + (iv[i].hi - iv[i].lo);
  const double len = b - a;
  return (len - cov) / len;
}

// perimeter position: edge (0 bottom, 1 right, 2 top, 3 left; counter-
// clockwise) and distance in [0, 1) from the edge's first corner
struct PP {
  int e;
  double t;
};

__device__ __forceinline__ PP Pt(int e, double t) {
  PP p;
  if (t >= 1.0) {
    p.e = (e + 1) & 3;
    p.t = 0.0;
  } else {
    p.e = e;
    p.t = t;
  }
  return p;
}

__device__ __forceinline__ bool Eq(const PP& a, const PP& b) { return a.e == b.e && a.t == b.t; }

__device__ __forceinline__ double Fwd(const PP& a, const PP& b) {
  if (b.e == a.e && b.t >= a.t) return b.t - a.t;
  return (1.0 - a.t) + double((b.e - a.e - 1 + 4) % 4) + b.t;
}

__device__ __forceinline__ void UV(const PP& p, double& u, double& v) {
  if (p.e == 0) {
    u = -0.5 + p.t;
    v = -0.5;
  } else if (p.e == 1) {
    u = 0.5;
    v = -0.5 + p.t;
  } else if (p.e == 2) {
    u = 0.5 - p.t;
    v = 0.5;
  } else {
    u = -0.5;
    v = 0.5 - p.t;
  }
}

// Position of v on a cell edge [a, b] of length h as a fraction of the edge,
// walked from a (EdgeFrac) or from b (EdgeFracRev): the ends exactly 0 and 1
// -- an interval clamped to an edge end stops there, and the perimeter walk
// must see it meet the next edge's interval (a - b + h need not round to 0)
// -- else (v - a) / h or (b - v) / h.
__device__ __forceinline__ double EdgeFrac(double v, double a, double b, double h) {
  if (v == a) return 0.0;
  if (v == b) return 1.0;
  return (v - a) / h;
}
__device__ __forceinline__ double EdgeFracRev(double v, double a, double b, double h) {
  if (v == b) return 0.0;
  if (v == a) return 1.0;
  return (b - v) / h;
}

struct Cell {
  double alpha, nx, ny, cx, cy;
};

__device__ inline Cell CellGeometry(double xa, double ya, double dx, double dy, int nwords,
                                    const double* __restrict__ shapes) {
  const double xb = xa + dx, yb = ya + dy;
  constexpr int kArcs = 4 * kMaxIntervals;
  PP lo[kArcs], hi[kArcs];
  int nc = 0;
  Iv iv[kMaxIntervals];
  int n = Covered(ya, xa, xb, false, nwords, shapes, iv);
  for (int i = 0; i < n && nc < kArcs; ++i, ++nc) {
    lo[nc] = Pt(0, EdgeFrac(iv[i].lo, xa, xb, dx));
    hi[nc] = Pt(0, EdgeFrac(iv[i].hi, xa, xb, dx));
  }
  n = Covered(xb, ya, yb, true, nwords, shapes, iv);
  for (int i = 0; i < n && nc < kArcs; ++i, ++nc) {
    lo[nc] = Pt(1, EdgeFrac(iv[i].lo, ya, yb, dy));
    hi[nc] = Pt(1, EdgeFrac(iv[i].hi, ya, yb, dy));
  }
  n = Covered(yb, xa, xb, false, nwords, shapes, iv);
  for (int i = n - 1; i >= 0 && nc < kArcs; --i, ++nc) {
    lo[nc] = Pt(2, EdgeFracRev(iv[i].hi, xa, xb, dx));
    hi[nc] = Pt(2, EdgeFracRev(iv[i].lo, xa, xb, dx));
  }
  n = Covered(xa, ya, yb, true, nwords, shapes, iv);
  for (int i = n - 1; i >= 0 && nc < kArcs; --i, ++nc) {
    lo[nc] = Pt(3, EdgeFracRev(iv[i].hi, ya, yb, dy));
    hi[nc] = Pt(3, EdgeFracRev(iv[i].lo, ya, yb, dy));
  }
  Cell g{1.0, 0.0, 0.0, 0.0, 0.0};
  if (nc == 0) return g;
  int m = 0;
  for (int i = 0; i < nc; ++i) {
    if (m > 0 && Eq(hi[m - 1], lo[i])) {
      hi[m - 1] = hi[i];
    } else {
      lo[m] = lo[i];
      hi[m] = hi[i];
      ++m;
    }
  }
  if (m > 1 && Eq(hi[m - 1], lo[0])) {
    lo[0] = lo[m - 1];
    --m;
  }
  double covered = 0.0;
  for (int i = 0; i < m; ++i) covered = covered + Fwd(lo[i], hi[i]);
  if (m == 1 && Eq(lo[0], hi[0])) covered = 4.0;
  if (covered >= 4.0) {
    g.alpha = 0.0;
    return g;
  }
  // shoelace over: chord start, chord end, corners of the following fluid arc
  double a2 = 0.0;
  double fu = 0.0, fv = 0.0;  // first vertex
  double pu = 0.0, pv = 0.0;  // previous vertex
  bool first = true;
  auto vertex = [&](double u, double v) {
    if (first) {
      fu = u;
      fv = v;
      first = false;
    } else {
      a2 = a2 + (pu * v - u * pv);
    }
    pu = u;
    pv = v;
  };
  double snx = 0.0, sny = 0.0, sl = 0.0, scx = 0.0, scy = 0.0;
  for (int j = 0; j < m; ++j) {
    double ua, va, ub, vb;
    UV(lo[j], ua, va);
    UV(hi[j], ub, vb);
    vertex(ua, va);
    vertex(ub, vb);
    const double lx = (ub - ua) * dx, ly = (vb - va) * dy;
    const double len = sqrt(lx * lx + ly * ly);
    snx = snx - ly;
    sny = sny + lx;
    sl = sl + len;
    scx = scx + 0.5 * (ua + ub) * len;
    scy = scy + 0.5 * (va + vb) * len;
    const PP p = hi[j];
    const PP q = lo[(j + 1) % m];
    if (!(q.e == p.e && q.t > p.t)) {
      for (int c = (p.e + 1) & 3;; c = (c + 1) & 3) {
        double u, v;
        if (c == q.e) {
          if (q.t > 0.0) {
            UV(PP{c, 0.0}, u, v);
            vertex(u, v);
          }
          break;
        }
        UV(PP{c, 0.0}, u, v);
        vertex(u, v);
      }
    }
  }
  a2 = a2 + (pu * fv - fu * pv);  // closing edge
  double alpha = 0.5 * a2;
  alpha = alpha < 0.0 ? 0.0 : alpha;
  alpha = alpha > 1.0 ? 1.0 : alpha;
  g.alpha = alpha;
  const double nn = sqrt(snx * snx + sny * sny);
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

}  // namespace ccgeom
}  // namespace fvs
