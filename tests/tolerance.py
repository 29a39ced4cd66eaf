"""Per-cell tolerance of the FP64 flavours that are not bit-identical to the
oracle (fast FP64 with FMA contraction and refined reciprocals, double-float).

The stated tolerance is 1e-12 relative per cell.  Density and energy are
positive, so for them the check is purely relative:
    |a - b| <= rtol * |b|.
Momentum components cross zero, where a relative bound means nothing; for
them the bound is relative to the cell's value plus the component's largest
magnitude over the grid:
    |a - b| <= rtol * (|b| + max |b_m|).
"""
import numpy as np


def positive_components(rank):
    """Indices of density and energy among the rank+2 conservative components."""
    return (0, rank + 1)


def assert_close_fp64(a, b, rank, rtol=1e-12, what=""):
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    ncomp = b.shape[0]
    assert ncomp == rank + 2, (ncomp, rank)
    worst = []
    for c in range(ncomp):
        ac = a[c].ravel()
        bc = b[c].ravel()
        err = np.abs(ac - bc)
        if c in positive_components(rank):
            assert np.all(bc > 0), f"{what} component {c} not positive"
            scale = np.abs(bc)
        else:
            scale = np.abs(bc) + np.abs(bc).max()
        rel = err / np.where(scale > 0, scale, 1.0)
        worst.append(float(rel.max()) if rel.size else 0.0)
        bad = rel > rtol
        assert not bad.any(), (f"{what} component {c}: {int(bad.sum())} cells beyond "
                               f"{rtol:g}, max rel err {rel.max():.3e}")
    return worst
