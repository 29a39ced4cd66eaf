"""ctypes bindings of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product package.  The oracle is a
scalar C++17 restatement of maikel/FiniteVolumeSolver's perfect-gas patch
update (see fvs_oracle.hpp for the file:line citations).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

MUSCL_HLLE, HLLE, GODUNOV, MUSCL_GODUNOV, HLLEM, MUSCL_HLLEM = 0, 1, 2, 3, 4, 5
MUSCL_CHAR, MUSCL_PRIM = 6, 7
VAN_LEER, MINMOD, NO_LIMITER, NO_GRADIENT = 0, 1, 2, 3
GUESS_MEAN, GUESS_PVRS_TR, GUESS_GIVEN = 0, 1, 2


class OrcMethod(C.Structure):
    _fields_ = [("method", C.c_int32), ("limiter", C.c_int32), ("guess", C.c_int32),
                ("max_iterations", C.c_int32), ("tol", C.c_double)]


def method(kind=MUSCL_HLLE, limiter=VAN_LEER, guess=GUESS_MEAN, max_iterations=5000,
           tol=1e-7) -> OrcMethod:
    return OrcMethod(kind, limiter, guess, max_iterations, tol)


_lib = None
_P = C.POINTER(C.c_double)
_I32 = C.POINTER(C.c_int32)
_I64 = C.POINTER(C.c_int64)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(str(path))
        M = C.POINTER(OrcMethod)
        L.orc_complete_from_cons.argtypes = [C.c_int, C.c_int64, _P, _P]
        L.orc_compute_numeric_fluxes.argtypes = [M, C.c_int, _P, _I32, _I32, _P, _I32, _I32,
                                                 C.c_double, C.c_double, C.c_int, _I64, _I64]
        L.orc_compute_numeric_fluxes.restype = C.c_int
        L.orc_compute_stable_dt.argtypes = [M, C.c_int, _P, _I32, _I32, C.c_double, C.c_int,
                                            C.c_int]
        L.orc_compute_stable_dt.restype = C.c_double
        L.orc_update_conservatively.argtypes = [_P, _I32, _I32, _P, _I32, _I32, _P, _I32, _I32,
                                                C.c_int, C.c_double, C.c_double, C.c_int]
        L.orc_grid_sweep.argtypes = [M, C.c_int, _I32, _I32, _P, _P, _P, C.c_double, C.c_int,
                                     C.c_int, _I64, _I64]
        L.orc_grid_stable_dt.argtypes = [M, C.c_int, _I32, _I32, _P, _P, C.c_int, C.c_int,
                                         C.c_int]
        L.orc_grid_stable_dt.restype = C.c_double
        L.orc_grid_step.argtypes = [M, C.c_int, _I32, _I32, _P, _P, C.c_double, C.c_int,
                                    C.c_int]
        L.orc_grid_step.restype = C.c_int
        L.orc_run.argtypes = [M, C.c_int, _I32, _I32, _P, _P, C.c_double, C.c_double, C.c_int,
                              C.c_int, _P, C.c_int, _P, C.POINTER(C.c_int), C.c_int, _I64, _I64]
        L.orc_run.restype = C.c_int
        L.orc_exact_star.argtypes = [C.c_int64, _P, _P, _P, _P, _P, _P, C.c_int, _P, C.c_double,
                                     C.c_int, _P, _P, _I32, _I32]
        L.orc_max_threads.restype = C.c_int
        _lib = L
    return _lib


def _d(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_P)


def _i3(v):
    a = (C.c_int32 * 3)(*[int(x) for x in v])
    return a


def _pad3(v, fill):
    v = list(v)
    return v + [fill] * (3 - len(v))


def max_threads() -> int:
    return int(lib().orc_max_threads())


def complete_from_cons(rank: int, cons: np.ndarray) -> np.ndarray:
    """cons: (rank+2, n) -> complete (rank+4, n)."""
    cons = np.ascontiguousarray(cons, dtype=np.float64)
    n = cons.shape[1]
    out = np.zeros((rank + 4, n))
    lib().orc_complete_from_cons(rank, n, _d(cons), _d(out))
    return out


def compute_numeric_fluxes(m: OrcMethod, rank, states, cell_box, face_box, dt, dx, dir):
    """states: (rank+4, nz, ny, nx) over cell_box; returns fluxes over face_box."""
    states = np.ascontiguousarray(states, dtype=np.float64)
    flo, fhi = _pad3(face_box[0], 0), _pad3(face_box[1], 1)
    clo, chi = _pad3(cell_box[0], 0), _pad3(cell_box[1], 1)
    shape = (rank + 2, fhi[2] - flo[2], fhi[1] - flo[1], fhi[0] - flo[0])
    fluxes = np.zeros(shape)
    it = C.c_int64(0)
    fl = C.c_int64(0)
    lib().orc_compute_numeric_fluxes(C.byref(m), rank, _d(fluxes), _i3(flo), _i3(fhi),
                                     _d(states), _i3(clo), _i3(chi), dt, dx, dir,
                                     C.byref(it), C.byref(fl))
    return fluxes


def compute_stable_dt(m: OrcMethod, rank, states, cell_box, dx, dir, window_rule=1):
    states = np.ascontiguousarray(states, dtype=np.float64)
    clo, chi = _pad3(cell_box[0], 0), _pad3(cell_box[1], 1)
    return lib().orc_compute_stable_dt(C.byref(m), rank, _d(states), _i3(clo), _i3(chi), dx,
                                       dir, window_rule)


def update_conservatively(next_box, prev, prev_box, fluxes, face_box, dt, dx, dir):
    prev = np.ascontiguousarray(prev, dtype=np.float64)
    fluxes = np.ascontiguousarray(fluxes, dtype=np.float64)
    nlo, nhi = _pad3(next_box[0], 0), _pad3(next_box[1], 1)
    ncomp = prev.shape[0]
    out = np.full((ncomp, nhi[2] - nlo[2], nhi[1] - nlo[1], nhi[0] - nlo[0]), np.nan)
    lib().orc_update_conservatively(
        _d(out), _i3(nlo), _i3(nhi), _d(prev), _i3(_pad3(prev_box[0], 0)),
        _i3(_pad3(prev_box[1], 1)), _d(fluxes), _i3(_pad3(face_box[0], 0)),
        _i3(_pad3(face_box[1], 1)), ncomp, dt, dx, dir)
    return out


class Grid:
    """A uniform single-patch grid; cons arrays are (rank+2, nz, ny, nx)."""

    def __init__(self, rank, n, bc, dx):
        self.rank = rank
        self.n = _pad3(n, 1)
        self.bc = _pad3(bc, 0)
        self.dx = np.array(_pad3(dx, 1.0), dtype=np.float64)

    def _args(self):
        return _i3(self.n), _i3(self.bc), _d(self.dx)

    def sweep(self, m, cons, dt, dir, nthreads=0):
        cons = np.ascontiguousarray(cons, dtype=np.float64)
        out = np.empty_like(cons)
        n, bc, dx = self._args()
        lib().orc_grid_sweep(C.byref(m), self.rank, n, bc, dx, _d(cons), _d(out), dt, dir,
                             nthreads, None, None)
        return out

    def stable_dt(self, m, cons, dir=-1, rule=0, nthreads=0):
        cons = np.ascontiguousarray(cons, dtype=np.float64)
        n, bc, dx = self._args()
        return lib().orc_grid_stable_dt(C.byref(m), self.rank, n, bc, dx, _d(cons), dir, rule,
                                        nthreads)

    def step(self, m, cons, dt, cycle, nthreads=0):
        cons = np.array(cons, dtype=np.float64, copy=True, order="C")
        n, bc, dx = self._args()
        lib().orc_grid_step(C.byref(m), self.rank, n, bc, dx, _d(cons), dt, cycle, nthreads)
        return cons

    def run(self, m, cons, cfl, t_end, max_steps=-1, dt_rule=0, dt_override=None,
            nthreads=0):
        cons = np.array(cons, dtype=np.float64, copy=True, order="C")
        n, bc, dx = self._args()
        cap = max_steps if max_steps >= 0 else 100000
        log = np.zeros(max(cap, 1))
        restarts = C.c_int(0)
        if dt_override is not None:
            dto = np.ascontiguousarray(dt_override, dtype=np.float64)
            dptr, nov = _d(dto), len(dto)
        else:
            dptr, nov = None, 0
        steps = lib().orc_run(C.byref(m), self.rank, n, bc, dx, _d(cons), cfl, t_end,
                              max_steps, dt_rule, dptr, nov, _d(log), C.byref(restarts),
                              nthreads, None, None)
        return cons, log[:steps].copy(), restarts.value


def exact_star(rhoL, uL, pL, rhoR, uR, pR, guess=GUESS_MEAN, given=None, tol=1e-7,
               max_iterations=5000):
    arrs = [np.ascontiguousarray(np.atleast_1d(x), dtype=np.float64)
            for x in (rhoL, uL, pL, rhoR, uR, pR)]
    n = len(arrs[0])
    ps, us = np.zeros(n), np.zeros(n)
    it = np.zeros(n, dtype=np.int32)
    cv = np.zeros(n, dtype=np.int32)
    g = None if given is None else np.ascontiguousarray(given, dtype=np.float64)
    lib().orc_exact_star(n, *[_d(a) for a in arrs], guess, None if g is None else _d(g), tol,
                         max_iterations, _d(ps), _d(us), it.ctypes.data_as(_I32),
                         cv.ctypes.data_as(_I32))
    return ps, us, it, cv


# ---------------------------------------------------------------------------
# KBN cut-cell (2-D)

def _cc_lib():
    L = lib()
    if not getattr(L, "_cc_ready", False):
        I = C.c_int
        L.orc_cc_ghost_layers.restype = C.c_int
        L.orc_cc_geometry.argtypes = [I, I, C.c_double, C.c_double, C.c_double, C.c_double, I, I,
                                      _P, _P, _P, _P, _P, _P]
        L.orc_cc_geometry_shapes.argtypes = [I, I, C.c_double, C.c_double, C.c_double,
                                             C.c_double, I, I, _P, _P, _P, _P, _P, _P]
        L.orc_cc_shielded.argtypes = [I, I, I, _P, _P, _P, _P, _P, _P, _P, _P]
        L.orc_cc_cutcells.argtypes = [_I32, _P, _P, _P, _I32]
        L.orc_cc_reference_states.argtypes = [_I32, _I32, _P, _P, _P, _P, _P, _P, _P, _P]
        L.orc_cc_sweep.argtypes = [_I32, _I32, _P, _P, _P, _P, _P, _P, _P, _P, _P, C.c_double,
                                   I, I, I]
        L.orc_cc_stable_dt.argtypes = [_I32, _I32, _P, _P, _P, _P, _P, I]
        L.orc_cc_stable_dt.restype = C.c_double
        L.orc_cc_run.argtypes = [_I32, _I32, _P, _P, _P, _P, _P, _P, _P, C.c_double, C.c_double,
                                 I, I, _P, C.POINTER(C.c_int), I]
        L.orc_cc_run.restype = C.c_int
        L._cc_ready = True
    return L


def shape_words(shapes):
    """Shape records (the oracle's and the library's flat form) of a list of
    shapes given as dicts: {"kind": "circle", "p": (cx, cy, r)},
    {"kind": "halfspace", "p": (nx, ny, offset)} (the normal is normalised
    here, as Halfspace's constructor does), {"kind": "polygon", "xy":
    [(x, y), ...]} (closed); optional "inverted": True."""
    import math
    words = []
    for s in shapes:
        inv = 1.0 if s.get("inverted") else 0.0
        if s["kind"] == "circle":
            words += [0.0, inv] + [float(v) for v in s["p"]]
        elif s["kind"] == "halfspace":
            nx, ny, o = (float(v) for v in s["p"])
            nn = math.sqrt(nx * nx + ny * ny)
            words += [1.0, inv, nx / nn, ny / nn, o]
        else:
            xy = [(float(x), float(y)) for x, y in s["xy"]]
            words += [2.0, inv, float(len(xy))] + [v for pt in xy for v in pt]
    return np.array(words, dtype=np.float64)


class CutCellGeometry:
    """FP64 geometry of a union of circles (solid inside) -- or, with
    `shapes`, of a union of shapes (shape_words) -- on an nx x ny grid grown
    by `ghost` layers: alpha [NY][NX], betax [NY][NX+1], betay [NY+1][NX],
    normal/center [2][NY][NX]."""

    def __init__(self, nx, ny, circles=None, x0=0.0, y0=0.0, dx=None, dy=None, shapes=None):
        L = _cc_lib()
        self.G = int(L.orc_cc_ghost_layers())
        self.nx, self.ny = nx, ny
        self.dx = 1.0 / nx if dx is None else dx
        self.dy = 1.0 / ny if dy is None else dy
        NX, NY = nx + 2 * self.G, ny + 2 * self.G
        self.alpha = np.zeros((NY, NX))
        self.betax = np.zeros((NY, NX + 1))
        self.betay = np.zeros((NY + 1, NX))
        self.normal = np.zeros((2, NY, NX))
        self.center = np.zeros((2, NY, NX))
        if shapes is not None:
            words = shape_words(shapes)
            L.orc_cc_geometry_shapes(nx, ny, x0, y0, self.dx, self.dy, self.G, len(words),
                                     _d(words), _d(self.alpha), _d(self.betax), _d(self.betay),
                                     _d(self.normal), _d(self.center))
            return
        circ = np.ascontiguousarray(circles, dtype=np.float64).reshape(-1, 3)
        self.circles = circ
        L.orc_cc_geometry(nx, ny, x0, y0, self.dx, self.dy, self.G, len(circ), _d(circ.ravel()),
                          _d(self.alpha), _d(self.betax), _d(self.betay), _d(self.normal),
                          _d(self.center))

    def shielded(self, dir):
        L = _cc_lib()
        shape = self.betax.shape if dir == 0 else self.betay.shape
        outs = [np.zeros(shape) for _ in range(6)]
        L.orc_cc_shielded(self.nx, self.ny, dir, _d(self.betax), _d(self.betay),
                          *[_d(o) for o in outs])
        return outs

    def cut_cells(self):
        L = _cc_lib()
        flags = np.zeros((self.ny, self.nx), dtype=np.int32)
        L.orc_cc_cutcells(_i3([self.nx, self.ny, 1]), _d(self.alpha), _d(self.betax),
                          _d(self.betay), flags.ctypes.data_as(_I32))
        return flags

    def _args(self, bc):
        dx = np.array([self.dx, self.dy])
        self._dxarr = dx
        return (_i3([self.nx, self.ny, 1]), _i3(list(bc) + [0]), _d(dx), _d(self.alpha),
                _d(self.betax), _d(self.betay))

    def reference_states(self, cons, bc=(1, 1)):
        L = _cc_lib()
        cons = np.ascontiguousarray(cons, dtype=np.float64)
        refs = np.zeros((6,) + self.alpha.shape)
        L.orc_cc_reference_states(*self._args(bc), _d(self.normal), _d(self.center), _d(cons),
                                  _d(refs))
        return refs

    def sweep(self, cons_ref_src, cons, dt, dir, bc=(1, 1), limiter=VAN_LEER, nthreads=0):
        L = _cc_lib()
        src = np.ascontiguousarray(cons_ref_src, dtype=np.float64)
        cons = np.ascontiguousarray(cons, dtype=np.float64)
        out = np.empty_like(cons)
        L.orc_cc_sweep(*self._args(bc), _d(self.normal), _d(self.center), _d(src), _d(cons),
                       _d(out), dt, dir, limiter, nthreads)
        return out

    def stable_dt(self, cons, dir=-1, bc=(1, 1)):
        L = _cc_lib()
        cons = np.ascontiguousarray(cons, dtype=np.float64)
        return L.orc_cc_stable_dt(*self._args(bc), _d(cons), dir)

    def run(self, cons, cfl, t_end, max_steps=-1, bc=(1, 1), limiter=VAN_LEER, nthreads=0):
        L = _cc_lib()
        cons = np.array(cons, dtype=np.float64, copy=True, order="C")
        cap = max_steps if max_steps >= 0 else 100000
        log = np.zeros(max(cap, 1))
        rs = C.c_int(0)
        steps = L.orc_cc_run(*self._args(bc), _d(self.normal), _d(self.center), _d(cons), cfl,
                             t_end, max_steps, limiter, _d(log), C.byref(rs), nthreads)
        return cons, log[:steps].copy(), rs.value


# ---------------------------------------------------------------------------
# Batched AMR patch set (2-D, ratio 2, MUSCL-Hancock/VanLeer + HLLE, FP64)

def amr_run(hier, cons, cfl, t_end, max_steps=-1, dt_override=None, nthreads=0):
    """Advance an AMR hierarchy (see finitevolumesolver_gb300.workloads
    .AmrHierarchy: nlevels, n0, bc, dx0, levels [npatch], boxes [npatch, 4]).
    cons: the patch interiors concatenated, each [4][ny][nx].  Returns
    (cons, dt_log, restarts)."""
    L = lib()
    if not getattr(L, "_amr_ready", False):
        I = C.c_int
        L.orc_amr_run.argtypes = [I, _I32, _I32, C.c_double, I, _I32, _I32, _P, C.c_double,
                                  C.c_double, I, _P, I, _P, C.POINTER(C.c_int), I]
        L.orc_amr_run.restype = C.c_int
        L._amr_ready = True
    cons = np.array(cons, dtype=np.float64, copy=True, order="C")
    n0 = np.asarray(hier.n0, dtype=np.int32)
    bc = np.asarray(hier.bc, dtype=np.int32)
    lv = np.ascontiguousarray(hier.levels, dtype=np.int32)
    bx = np.ascontiguousarray(hier.boxes, dtype=np.int32)
    ov = None if dt_override is None else np.ascontiguousarray(dt_override, dtype=np.float64)
    cap = max_steps if max_steps >= 0 else 100000
    log = np.zeros(max(cap, 1))
    rs = C.c_int(0)
    steps = L.orc_amr_run(int(hier.nlevels), n0.ctypes.data_as(_I32), bc.ctypes.data_as(_I32),
                          float(hier.dx0), len(lv), lv.ctypes.data_as(_I32),
                          bx.ctypes.data_as(_I32), _d(cons), float(cfl), float(t_end),
                          int(max_steps), None if ov is None else _d(ov),
                          0 if ov is None else len(ov), _d(log), C.byref(rs), int(nthreads))
    if steps < 0:
        raise ValueError("invalid AMR hierarchy")
    return cons, log[:steps].copy(), rs.value
