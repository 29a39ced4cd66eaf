"""CPU checks of the oracle's cut-cell geometry for general shapes (circles,
half-spaces, polygons, inverted shapes, unions -- the reference's
include/fub/geometry/* forms).  A straight boundary is reconstructed exactly
by the chord polygon, so against a half-space the volume fractions, face
fractions, normals and centroids have closed forms; polygons follow the
reference's even-odd inside rule; circles given as shapes reproduce the
circle generator bit for bit."""
import math

import numpy as np
import pytest

N = 48


def _clip_area(f, x0, y0, h):
    """Area fraction of the cell [x0, x0+h] x [y0, y0+h] where f <= 0 (f affine)."""
    pts = [(x0, y0), (x0 + h, y0), (x0 + h, y0 + h), (x0, y0 + h)]
    out = []
    for i in range(4):
        p, q = pts[i], pts[(i + 1) % 4]
        fp, fq = f(*p), f(*q)
        if fp <= 0:
            out.append(p)
        if (fp <= 0) != (fq <= 0):
            t = fp / (fp - fq)
            out.append((p[0] + t * (q[0] - p[0]), p[1] + t * (q[1] - p[1])))
    if len(out) < 3:
        return 0.0
    a = sum(out[i][0] * out[(i + 1) % len(out)][1] - out[(i + 1) % len(out)][0] * out[i][1]
            for i in range(len(out)))
    return abs(a) / 2 / (h * h)


def test_circles_as_shapes_bit_exact(orc):
    circles = [[0.5, 0.5, 0.2], [0.3, 0.72, 0.11], [0.95, 0.1, 0.2]]
    a = orc.CutCellGeometry(N, N, circles)
    b = orc.CutCellGeometry(N, N, shapes=[{"kind": "circle", "p": c} for c in circles])
    for k in ("alpha", "betax", "betay", "normal", "center"):
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k), err_msg=k)


@pytest.mark.parametrize("nrm,off", [((-3.0, 4.0), 0.1), ((1.0, 0.0), 0.37), ((2.0, 1.0), 0.9)])
def test_halfspace_closed_forms(orc, nrm, off):
    g = orc.CutCellGeometry(N, N, shapes=[{"kind": "halfspace", "p": (*nrm, off)}])
    G = g.G
    nn = math.hypot(*nrm)
    ux, uy = nrm[0] / nn, nrm[1] / nn
    f = lambda x, y: ux * x + uy * y - off  # body where f > 0
    h = 1.0 / N
    alpha = g.alpha[G:-G, G:-G]
    exact = np.array([[_clip_area(f, i * h, j * h, h) for i in range(N)] for j in range(N)])
    np.testing.assert_allclose(alpha, exact, rtol=0, atol=1e-12)
    cut = (alpha > 1e-9) & (alpha < 1 - 1e-9)
    assert cut.any()
    # the boundary normal points into the fluid, -n
    np.testing.assert_allclose(g.normal[0, G:-G, G:-G][cut], -ux, atol=1e-12)
    np.testing.assert_allclose(g.normal[1, G:-G, G:-G][cut], -uy, atol=1e-12)
    # the boundary centroid lies on the line (cell units about the centre)
    jj, ii = np.nonzero(cut)
    xc = (ii + 0.5 + g.center[0, G:-G, G:-G][cut]) * h
    yc = (jj + 0.5 + g.center[1, G:-G, G:-G][cut]) * h
    np.testing.assert_allclose(f(xc, yc), 0.0, atol=1e-12)
    # x faces: fluid length fraction of the segment x = i h, y in cell j
    for j in range(0, N, 7):
        for i in range(0, N + 1, 5):
            x, y0, y1 = i * h, j * h, (j + 1) * h
            fa, fb = f(x, y0), f(x, y1)
            if fa <= 0 and fb <= 0:
                ref = 1.0
            elif fa > 0 and fb > 0:
                ref = 0.0
            else:
                t = fa / (fa - fb)
                ref = t if fa <= 0 else 1 - t
            assert abs(g.betax[j + G, i + G] - ref) < 1e-12 or g.alpha[j + G, i + G] == 0 or \
                g.alpha[j + G, i + G - 1] == 0


def _inside_even_odd(xy, x, y):
    """The reference's even-odd rule (Polygon::ComputeDistanceTo): crossings
    of the edges with the ray to the left of the point."""
    c = 0
    for (vx, vy), (wx, wy) in zip(xy[:-1], xy[1:]):
        if (vy < y <= wy) or (wy < y <= vy):
            t = (y - vy) / (wy - vy)
            if (1 - t) * vx + t * wx < x:
                c += 1
    return c % 2 == 1


def _star(n=7, r0=0.3, r1=0.14):
    pts = []
    for k in range(2 * n):
        r = r0 if k % 2 == 0 else r1
        t = 0.2 + math.pi * k / n
        pts.append((0.5 + r * math.cos(t), 0.47 + r * math.sin(t)))
    return pts + [pts[0]]


def test_polygon_inside_rule_and_complement(orc):
    xy = _star()
    g = orc.CutCellGeometry(N, N, shapes=[{"kind": "polygon", "xy": xy}])
    gi = orc.CutCellGeometry(N, N, shapes=[{"kind": "polygon", "xy": xy, "inverted": True}])
    G = g.G
    h = 1.0 / N
    a = g.alpha[G:-G, G:-G]
    ai = gi.alpha[G:-G, G:-G]
    # cells two or more cells away from every vertex see straight edges only
    # (near a sharp vertex a sub-cell spike is not resolved by the chords)
    verts = {(int(x / h), int(y / h)) for x, y in xy}
    near = {(vi + di, vj + dj) for vi, vj in verts for di in range(-2, 3) for dj in range(-2, 3)}
    for j in range(N):
        for i in range(N):
            if (i, j) in near:
                continue
            if a[j, i] in (0.0, 1.0):
                inside = _inside_even_odd(xy, (i + 0.5) * h, (j + 0.5) * h)
                assert (a[j, i] == 0.0) == inside
                assert ai[j, i] == 1.0 - a[j, i]
            else:  # crossed by one straight edge: complementary fractions
                assert abs(a[j, i] + ai[j, i] - 1.0) < 1e-12
    # the chord polygons cut only the vertex cells: areas within their area
    area = 0.5 * abs(sum(xy[k][0] * xy[k + 1][1] - xy[k + 1][0] * xy[k][1]
                         for k in range(len(xy) - 1)))
    assert abs((1.0 - a.sum() * h * h) - area) < len(near) * h * h
    assert abs(ai.sum() * h * h - area) < len(near) * h * h


def test_union_of_shapes(orc):
    """A ramp (half-space) and a circle: covered where either covers; faces
    are the union of the covered intervals."""
    shapes = [{"kind": "halfspace", "p": (-1.0, 3.0, -0.2)},  # body above the line
              {"kind": "circle", "p": (0.6, 0.45, 0.12)}]
    u = orc.CutCellGeometry(N, N, shapes=shapes)
    a = orc.CutCellGeometry(N, N, shapes=shapes[:1])
    b = orc.CutCellGeometry(N, N, shapes=shapes[1:])
    G = u.G
    full_a = a.alpha == 0
    full_b = b.alpha == 0
    assert np.all(u.alpha[full_a | full_b] == 0)
    both_fluid = (a.alpha == 1) & (b.alpha == 1)
    assert np.all(u.alpha[both_fluid] == 1)
    np.testing.assert_array_less(u.betax - 1e-15, np.minimum(a.betax, b.betax) + 1e-15)


def test_polygon_known_answer_of_the_reference(orc):
    """The reference's polygon test (tests/test.Geometry.Polygon.cpp): the
    triangle (0.1, 0.1), (0.2, 0.1), (0.15, 0.2) has (0.11, 0.105) inside
    (distance > 0) and (0.09, 0.1) outside.  The reference hands that distance
    to AMReX's EB generator as the implicit function
    (include/fub/AMReX/Geometry.hpp:37-45), positive in the body, so here the
    first point's cell is covered (alpha 0) and the second one's fluid."""
    n = 1000
    xy = [(0.1, 0.1), (0.2, 0.1), (0.15, 0.2), (0.1, 0.1)]
    g = orc.CutCellGeometry(n, n, shapes=[{"kind": "polygon", "xy": xy}])
    G = g.G

    def cell(x, y):
        return int(y * n) + G, int(x * n) + G

    assert g.alpha[cell(0.11, 0.105)] == 0.0
    assert g.alpha[cell(0.09, 0.1)] == 1.0


def _clip_convex(poly, f):
    """The part of a convex polygon where the affine f <= 0."""
    out = []
    for k in range(len(poly)):
        p, q = poly[k], poly[(k + 1) % len(poly)]
        fp, fq = f(*p), f(*q)
        if fp <= 0:
            out.append(p)
        if (fp <= 0) != (fq <= 0):
            t = fp / (fp - fq)
            out.append((p[0] + t * (q[0] - p[0]), p[1] + t * (q[1] - p[1])))
    return out


def _area(poly):
    if len(poly) < 3:
        return 0.0
    return 0.5 * abs(sum(poly[k][0] * poly[(k + 1) % len(poly)][1]
                         - poly[(k + 1) % len(poly)][0] * poly[k][1] for k in range(len(poly))))


# The wedge of the reference's tests/test.AMReX.EB.plane_nan.cpp:32-53 on its
# 64 x 64 grid over [-0.5, 0.5] x [0, 1]: the complement of the intersection
# of the two planes through p0 = (0, 0.1) along p1 - p0 = (-1, 0.9) and
# p2 - p0 = (1, 0.9) leaves as body the cone y < 0.1 - 0.9 |x| (a wedge on
# the lower wall, its apex on the grid line x = 0).  Here it is the polygon
# of the cone cut off below the domain.
WEDGE_X0, WEDGE_N = -0.5, 64
WEDGE = [{"kind": "polygon", "xy": [(0.0, 0.1), (1.0, -0.8), (-1.0, -0.8), (0.0, 0.1)]}]


def test_wedge_of_the_reference_plane_nan_case(orc):
    """That test builds the wedge with floating-point exceptions enabled: no
    NaN may appear.  Here every array is finite, the fractions lie in [0, 1],
    no cut cell has a zero volume (the property tests/test.AMReX.EB.Cylinder.cpp
    prints violations of), and since the apex lies on a cell edge every cell is
    crossed by at most one straight edge: alpha equals the exact fluid area."""
    n, h = WEDGE_N, 1.0 / WEDGE_N
    g = orc.CutCellGeometry(n, n, x0=WEDGE_X0, y0=0.0, shapes=WEDGE)
    G = g.G
    for key in ("alpha", "betax", "betay", "normal", "center"):
        assert np.isfinite(getattr(g, key)).all(), key
    for key in ("alpha", "betax", "betay"):
        a = getattr(g, key)
        assert a.min() >= 0.0 and a.max() <= 1.0, key
    alpha = g.alpha[G:-G, G:-G]
    cut = g.cut_cells().astype(bool)
    assert cut.sum() > 0 and (alpha[cut] > 0.0).all()
    lines = [lambda x, y: y - (0.1 + 0.9 * x), lambda x, y: y - (0.1 - 0.9 * x)]  # body <= 0
    for j in range(n):
        for i in range(n):
            x0, y0 = WEDGE_X0 + i * h, j * h
            body = [(x0, y0), (x0 + h, y0), (x0 + h, y0 + h), (x0, y0 + h)]
            for f in lines:
                body = _clip_convex(body, f)
            exact = 1.0 - _area(body) / (h * h)
            assert abs(alpha[j, i] - exact) < 1e-12, (i, j, alpha[j, i], exact)
    # the two apex cells either side of x = 0
    ja, ia = int(0.1 / h), n // 2
    assert 0.0 < alpha[ja, ia - 1] < 1.0 and abs(alpha[ja, ia - 1] - alpha[ja, ia]) < 1e-12
