// fvs_cutcell_geometry.cuh -- FP64 cut-cell geometry of a union of circles
// (the embedded body is the inside of the circles), one cell or face per
// thread.
//
// AMReX's EB2 geometry generator, which the reference reads its cut-cell
// data from (src/AMReX/cutcell/PatchHierarchy.cpp:507-547), is not part of
// the reference tree; this is the library's own generator:
//  - face fraction beta: fluid length of the face / face length, from the
//    exact intervals the circles cover on the face;
//  - volume fraction alpha: area of the polygon formed by the fluid parts of
//    the cell's perimeter with every covered perimeter arc replaced by the
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

constexpr int kMaxCircles = 64;

struct Iv {
  double lo, hi;
};

// Merged covered intervals of the segment {fixed = c, free in [a, b]}.
__device__ __forceinline__ int Covered(double c, double a, double b, bool vertical, int ncirc,
                                       const double* __restrict__ circ, Iv* out) {
  Iv iv[16];
  int n = 0;
  for (int k = 0; k < ncirc && n < 16; ++k) {
    const double cx = circ[3 * k], cy = circ[3 * k + 1], r = circ[3 * k + 2];
    const double d = vertical ? (c - cx) : (c - cy);
    if (fabs(d) < r) {
      const double s = sqrt(r * r - d * d);
      const double m = vertical ? cy : cx;
      double lo = m - s, hi = m + s;
      lo = lo > a ? lo : a;
      hi = hi < b ? hi : b;
      if (lo < hi) {
        iv[n].lo = lo;
        iv[n].hi = hi;
        ++n;
      }
    }
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

struct Cell {
  double alpha, nx, ny, cx, cy;
};

__device__ __forceinline__ Cell CellGeometry(double xa, double ya, double dx, double dy,
                                             int ncirc, const double* __restrict__ circ) {
  const double xb = xa + dx, yb = ya + dy;
  constexpr int kArcs = 64;
  PP lo[kArcs], hi[kArcs];
  int nc = 0;
  Iv iv[16];
  int n = Covered(ya, xa, xb, false, ncirc, circ, iv);
  for (int i = 0; i < n && nc < kArcs; ++i, ++nc) {
    lo[nc] = Pt(0, (iv[i].lo - xa) / dx);
    hi[nc] = Pt(0, (iv[i].hi - xa) / dx);
  }
  n = Covered(xb, ya, yb, true, ncirc, circ, iv);
  for (int i = 0; i < n && nc < kArcs; ++i, ++nc) {
    lo[nc] = Pt(1, (iv[i].lo - ya) / dy);
    hi[nc] = Pt(1, (iv[i].hi - ya) / dy);
  }
  n = Covered(yb, xa, xb, false, ncirc, circ, iv);
  for (int i = n - 1; i >= 0 && nc < kArcs; --i, ++nc) {
    lo[nc] = Pt(2, (xb - iv[i].hi) / dx);
    hi[nc] = Pt(2, (xb - iv[i].lo) / dx);
  }
  n = Covered(xa, ya, yb, true, ncirc, circ, iv);
  for (int i = n - 1; i >= 0 && nc < kArcs; --i, ++nc) {
    lo[nc] = Pt(3, (yb - iv[i].hi) / dy);
    hi[nc] = Pt(3, (yb - iv[i].lo) / dy);
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
