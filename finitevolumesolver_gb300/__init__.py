"""finitevolumesolver_gb300 -- GB300 (sm_103a) split finite-volume patch update
for the perfect-gas Euler equations.

Host-side mirror of maikel/FiniteVolumeSolver's patch-level interface for the
split update (the names, argument meaning and error behaviour follow the
reference):

  FluxMethod.ComputeNumericFluxes / ComputeStableDt / GetStencilWidth
      include/fub/flux_method/FluxMethod.hpp:115-170
  HyperbolicPatchIntegrator.UpdateConservatively
      include/fub/HyperbolicPatchIntegrator.hpp:34-54
  CompleteFromCons
      src/equations/PerfectGas.cpp:96-124
  Solver (a uniform single-level grid run by RunSimulation's loop)
      include/fub/RunSimulation.hpp:86-191,
      include/fub/solver/DimensionalSplitLevelIntegrator.hpp:204-276

Every call goes through the C ABI of libfvs_gb300.so (include/fvs_gpu.h).
Data arguments are device pointers: ints or objects with ``data_ptr()``
(e.g. CUDA tensors).  There is no CPU fallback: without the library or a GPU
the calls raise.
"""
from __future__ import annotations

import ctypes as C

from . import _capi
from ._capi import AmrDesc, Box, FvsError, GridDesc, Method, RunStats

__all__ = ["PerfectGas", "FluxMethod", "HyperbolicPatchIntegrator", "CompleteFromCons",
           "Solver", "FvsError", "make_method", "box", "lib", "LearnedGuess",
           "riemann_features", "tc_gemm_bf16", "AmrSolver"]

FLUX_METHODS = {"muscl_hlle": 0, "hlle": 1, "godunov": 2, "muscl_godunov": 3, "hllem": 4,
                "muscl_hllem": 5, "muscl_char": 6, "muscl_prim": 7}
LIMITERS = {"van_leer": 0, "minmod": 1, "none": 2, "no_limiter": 2, "no_gradient": 3}
PRECISIONS = {"fp64_exact": 0, "fp64_fast": 1, "mixed": 2, "fp64_df": 3}
GUESSES = {"mean": 0, "pvrs_tr": 1, "mlp": 2}
BCS = {"periodic": 0, "transmissive": 1, "reflective": 2}


def lib() -> C.CDLL:
    return _capi.load()


def _ptr(x) -> int:
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        if hasattr(x, "is_cuda") and not x.is_cuda:
            raise ValueError("data must live in device memory")
        return int(x.data_ptr())
    raise TypeError(f"expected a device pointer, got {type(x)!r}")


def _stream(stream) -> int:
    if stream is None:
        return 0
    if isinstance(stream, int):
        return stream
    return int(getattr(stream, "cuda_stream", stream))


def box(lo, hi) -> Box:
    """Half-open index box [lo, hi); missing dimensions become [0, 1)."""
    lo = list(lo) + [0] * (3 - len(lo))
    hi = list(hi) + [1] * (3 - len(hi))
    b = Box()
    for d in range(3):
        b.lo[d] = int(lo[d])
        b.hi[d] = int(hi[d])
    return b


def _as_box(b) -> Box:
    return b if isinstance(b, Box) else box(*b)


def make_method(flux_method="muscl_hlle", limiter="van_leer", precision="fp64_exact",
                guess="mean", max_iterations=5000, tolerance=1e-7, gamma=1.4,
                mlp_params=None) -> Method:
    m = Method()
    lib().fvs_method_default(C.byref(m))
    m.flux_method = FLUX_METHODS[flux_method] if isinstance(flux_method, str) else flux_method
    m.limiter = LIMITERS[limiter] if isinstance(limiter, str) else limiter
    m.precision = PRECISIONS[precision] if isinstance(precision, str) else precision
    m.guess = GUESSES[guess] if isinstance(guess, str) else guess
    m.max_iterations = max_iterations
    m.tolerance = tolerance
    m.gamma = gamma
    m.mlp_params = _ptr(mlp_params) or None
    return m


def exact_riemann_star(method: Method, rhoL, uL, pL, rhoR, uR, pR, pstar, ustar=None,
                       iterations=None, status=None, stream=None) -> None:
    """ExactRiemannSolver<PerfectGas<1>>::ComputeMiddleState for arrays of
    problems (device arrays, float64; iterations/status int32)."""
    n = int(rhoL.numel()) if hasattr(rhoL, "numel") else int(len(rhoL))
    _capi.check(lib().fvs_exact_riemann_star(
        C.byref(method), n, _ptr(rhoL), _ptr(uL), _ptr(pL), _ptr(rhoR), _ptr(uR), _ptr(pR),
        _ptr(pstar), _ptr(ustar), _ptr(iterations), _ptr(status), _stream(stream)))


class PerfectGas:
    """fub::PerfectGas<Rank> (include/fub/equations/PerfectGas.hpp:164-211)."""

    def __init__(self, rank: int, gamma: float = 1.4):
        if rank not in (1, 2, 3):
            raise ValueError("rank must be 1, 2 or 3")
        self.rank = rank
        self.gamma = gamma
        self.gamma_minus_1_inv = 1.0 / (gamma - 1.0)

    def n_cons(self) -> int:
        return self.rank + 2

    def n_complete(self) -> int:
        return self.rank + 4


class FluxMethod:
    """fub::FluxMethod<Base> for Base in MusclHancock<PerfectGas, Hll<Einfeldt>,
    Limiter> (the default), Hll<PerfectGas, Einfeldt>, Godunov<ExactRiemannSolver>,
    MusclHancock<PerfectGas, Godunov>, perfect_gas::Hllem, MusclHancock<PerfectGas,
    Hllem>, perfect_gas::MusclHancockCharacteristic and perfect_gas::MusclHancockPrim
    (names in FLUX_METHODS)."""

    def __init__(self, equation: PerfectGas, flux_method="muscl_hlle", limiter="van_leer",
                 precision="fp64_exact", **kw):
        self.equation = equation
        self.method = make_method(flux_method, limiter, precision, gamma=equation.gamma, **kw)

    def GetStencilWidth(self) -> int:
        return 1 if self.method.flux_method in (1, 2, 4) else 2

    def ComputeNumericFluxes(self, fluxes, face_box, states, cell_box, dt, dx, dir,
                             stream=None) -> None:
        _capi.check(lib().fvs_compute_numeric_fluxes(
            C.byref(self.method), self.equation.rank, _ptr(fluxes), _as_box(face_box),
            _ptr(states), _as_box(cell_box), float(dt), float(dx), int(dir), _stream(stream)))

    def ComputeStableDt(self, states, cell_box, dx, dir, window_rule=1, stream=None) -> float:
        out = C.c_double(0.0)
        _capi.check(lib().fvs_compute_stable_dt(
            C.byref(self.method), self.equation.rank, _ptr(states), _as_box(cell_box),
            float(dx), int(dir), int(window_rule), C.byref(out), _stream(stream)))
        return out.value


class HyperbolicPatchIntegrator:
    """fub::HyperbolicPatchIntegrator<Tag> (include/fub/HyperbolicPatchIntegrator.hpp:34-54)."""

    def UpdateConservatively(self, next, next_box, prev, prev_box, fluxes, face_box, ncomp,
                             dt, dx, dir, stream=None) -> None:
        _capi.check(lib().fvs_update_conservatively(
            _ptr(next), _as_box(next_box), _ptr(prev), _as_box(prev_box), _ptr(fluxes),
            _as_box(face_box), int(ncomp), float(dt), float(dx), int(dir), _stream(stream)))


def CompleteFromCons(equation: PerfectGas, complete, complete_box, cons, cons_box, region,
                     stream=None) -> None:
    _capi.check(lib().fvs_complete_from_cons(
        equation.rank, equation.gamma, _ptr(complete), _as_box(complete_box), _ptr(cons),
        _as_box(cons_box), _as_box(region), _stream(stream)))


class HostPatchContext:
    """The patch-level calls for patch arrays in host memory (NumPy arrays,
    C-contiguous float64, FArrayBox layout): FluxMethod.ComputeNumericFluxes,
    ComputeStableDt, HyperbolicPatchIntegrator.UpdateConservatively and
    CompleteFromCons as a CPU build of the reference calls them.  The
    context stages the boxes through device buffers on its own stream."""

    def __init__(self):
        h = C.c_void_p()
        _capi.check(lib().fvs_patch_ctx_create(C.byref(h)))
        self._h = h

    def close(self):
        if self._h:
            lib().fvs_patch_ctx_destroy(self._h)
            self._h = None

    __del__ = close

    @staticmethod
    def _np(a):
        import numpy as np
        if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
            raise TypeError("host patch arrays are C-contiguous float64 NumPy arrays")
        return a.ctypes.data

    def ComputeNumericFluxes(self, fm: "FluxMethod", fluxes, face_box, states, cell_box, dt,
                             dx, dir) -> None:
        _capi.check(lib().fvs_compute_numeric_fluxes_host(
            self._h, C.byref(fm.method), fm.equation.rank, self._np(fluxes), _as_box(face_box),
            self._np(states), _as_box(cell_box), float(dt), float(dx), int(dir)))

    def ComputeStableDt(self, fm: "FluxMethod", states, cell_box, dx, dir,
                        window_rule=1) -> float:
        out = C.c_double(0.0)
        _capi.check(lib().fvs_compute_stable_dt_host(
            self._h, C.byref(fm.method), fm.equation.rank, self._np(states), _as_box(cell_box),
            float(dx), int(dir), int(window_rule), C.byref(out)))
        return out.value

    def UpdateConservatively(self, next, next_box, prev, prev_box, fluxes, face_box, ncomp, dt,
                             dx, dir) -> None:
        _capi.check(lib().fvs_update_conservatively_host(
            self._h, self._np(next), _as_box(next_box), self._np(prev), _as_box(prev_box),
            self._np(fluxes), _as_box(face_box), int(ncomp), float(dt), float(dx), int(dir)))

    def CompleteFromCons(self, equation: PerfectGas, complete, complete_box, cons, cons_box,
                         region) -> None:
        _capi.check(lib().fvs_complete_from_cons_host(
            self._h, equation.rank, equation.gamma, self._np(complete), _as_box(complete_box),
            self._np(cons), _as_box(cons_box), _as_box(region)))


class Solver:
    """A uniform single-level grid advanced by the reference's split step
    sequence, with the time step kept on the device."""

    def __init__(self, n, dx, bc="periodic", method: Method | None = None, dt_rule=0):
        rank = len(n)
        g = GridDesc()
        g.rank = rank
        bcs = [bc] * rank if isinstance(bc, (str, int)) else list(bc)
        for d in range(3):
            g.n[d] = int(n[d]) if d < rank else 1
            b = bcs[d] if d < rank else 0
            g.bc[d] = BCS[b] if isinstance(b, str) else int(b)
            g.dx[d] = float(dx[d] if not isinstance(dx, (int, float)) else dx) if d < rank else 1.0
        g.dt_rule = dt_rule
        self.rank = rank
        self.n = [int(x) for x in n]
        self.method = method if method is not None else make_method()
        self._h = C.c_void_p()
        _capi.check(lib().fvs_solver_create(C.byref(g), C.byref(self.method),
                                            C.byref(self._h)))

    def close(self):
        if self._h:
            lib().fvs_solver_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def shape(self):
        return (self.rank + 2,) + tuple(reversed(self.n + [1] * (3 - self.rank)))

    def upload(self, cons_host) -> None:
        import numpy as np
        a = np.ascontiguousarray(cons_host, dtype=np.float64)
        assert a.size == int(np.prod(self.shape()))
        _capi.check(lib().fvs_solver_upload(self._h, a.ctypes.data))

    def download(self):
        import numpy as np
        a = np.empty(self.shape(), dtype=np.float64)
        _capi.check(lib().fvs_solver_download(self._h, a.ctypes.data))
        return a

    def write_plotfile(self, directory) -> None:
        """AMReX plotfile of the current state (fub::amrex::PlotfileOutput)."""
        _capi.check(lib().fvs_solver_write_plotfile(self._h, str(directory).encode()))

    def state_device_ptr(self) -> int:
        p = C.c_void_p()
        _capi.check(lib().fvs_solver_state_device(self._h, C.byref(p)))
        return int(p.value or 0)

    def stream_handle(self) -> int:
        p = C.c_void_p()
        _capi.check(lib().fvs_solver_stream(self._h, C.byref(p)))
        return int(p.value or 0)

    def set_tiling(self, seg_len: int) -> None:
        _capi.check(lib().fvs_solver_set_tiling(self._h, int(seg_len)))

    def set_launch(self, dir, seg_len=0, variant=0) -> None:
        """Force direction dir's segment length and launch variant."""
        _capi.check(lib().fvs_solver_set_launch(self._h, int(dir), int(seg_len), int(variant)))

    def set_embedded_circles(self, circles, x0=0.0, y0=0.0) -> None:
        """Union of circles (rows cx, cy, r; the body is their inside) as an
        embedded boundary: the solver switches to the KBN cut-cell update."""
        import numpy as np
        c = np.ascontiguousarray(circles, dtype=np.float64).reshape(-1, 3)
        self._circles = c
        _capi.check(lib().fvs_solver_set_embedded_circles(self._h, c.ctypes.data, len(c),
                                                          float(x0), float(y0)))

    def set_embedded_geometry(self, shapes, x0=0.0, y0=0.0) -> None:
        """Union of shapes as the embedded body (the KBN cut-cell update):
        dicts {"kind": "circle", "p": (cx, cy, r)}, {"kind": "halfspace",
        "p": (nx, ny, offset)} (inside n . x - offset > 0), {"kind":
        "polygon", "xy": [(x, y), ...]} (closed), each with an optional
        "inverted": True (the body is the shape's outside)."""
        import numpy as np
        kinds = {"circle": 0, "halfspace": 1, "polygon": 2}
        arr = (_capi.Shape * len(shapes))()
        keep = []
        for k, sh in enumerate(shapes):
            arr[k].kind = kinds[sh["kind"]]
            arr[k].inverted = 1 if sh.get("inverted") else 0
            if sh["kind"] == "polygon":
                xy = np.ascontiguousarray(sh["xy"], dtype=np.float64).reshape(-1, 2)
                keep.append(xy)
                arr[k].nvertices = len(xy)
                arr[k].xy = xy.ctypes.data_as(C.POINTER(C.c_double))
            else:
                for i in range(3):
                    arr[k].p[i] = float(sh["p"][i])
        self._shapes = (arr, keep)
        _capi.check(lib().fvs_solver_set_embedded_geometry(self._h, arr, len(shapes), float(x0),
                                                           float(y0)))

    def cutcell_geometry(self):
        import numpy as np
        G = lib().fvs_cutcell_ghost_layers()
        nx, ny = self.n[0], self.n[1]
        NX, NY = nx + 2 * G, ny + 2 * G
        out = {"alpha": np.zeros((NY, NX)), "betax": np.zeros((NY, NX + 1)),
               "betay": np.zeros((NY + 1, NX)), "normal": np.zeros((2, NY, NX)),
               "center": np.zeros((2, NY, NX)), "cut": np.zeros((NY, NX), dtype=np.int8)}
        _capi.check(lib().fvs_solver_cutcell_geometry(
            self._h, *[out[k].ctypes.data for k in ("alpha", "betax", "betay", "normal", "center",
                                                   "cut")]))
        out["ghost"] = G
        return out

    def cutcell_shielded(self, dir: int):
        """[us, sL, sR, us_rel, sL_rel, sR_rel] of direction `dir` over the
        face array of the grown grid (the order of the oracle's
        CutCellGeometry.shielded)."""
        import numpy as np
        G = lib().fvs_cutcell_ghost_layers()
        NX, NY = self.n[0] + 2 * G, self.n[1] + 2 * G
        shape = (NY, NX + 1) if dir == 0 else (NY + 1, NX)
        outs = [np.zeros(shape) for _ in range(6)]
        _capi.check(lib().fvs_solver_cutcell_shielded(self._h, int(dir),
                                                       *[o.ctypes.data for o in outs]))
        return outs

    def autotune(self):
        segs = (C.c_int * 3)()
        _capi.check(lib().fvs_solver_autotune(self._h, segs))
        return list(segs)[: self.rank]

    def tuning(self):
        """(segment cells, occupancy variant) per direction after autotune()."""
        import numpy as np
        seg = np.zeros(3, dtype=np.int32)
        occ = np.zeros(3, dtype=np.int32)
        _capi.check(lib().fvs_solver_tuning(self._h, seg.ctypes.data, occ.ctypes.data))
        return seg[: self.rank].tolist(), occ[: self.rank].tolist()

    def set_cycle(self, cycle: int) -> None:
        _capi.check(lib().fvs_solver_set_cycle(self._h, int(cycle)))

    def set_time(self, t: float) -> None:
        _capi.check(lib().fvs_solver_set_time(self._h, float(t)))

    def ComputeStableDt(self, dir: int = -1) -> float:
        out = C.c_double(0.0)
        _capi.check(lib().fvs_solver_stable_dt(self._h, int(dir), C.byref(out)))
        return out.value

    def newton_stats(self, reset: bool = False, fallbacks: bool = False):
        """(Newton iterations, non-converged faces[, rejected learned starts])
        of the Godunov sweeps since the last reset."""
        it = C.c_uint64(0)
        fl = C.c_uint64(0)
        fb = C.c_uint64(0)
        _capi.check(lib().fvs_solver_newton_stats(self._h, C.byref(it), C.byref(fl),
                                                  C.byref(fb), int(reset)))
        return (it.value, fl.value, fb.value) if fallbacks else (it.value, fl.value)

    def sweep(self, dir: int, dt: float) -> float:
        out = C.c_double(0.0)
        _capi.check(lib().fvs_solver_sweep(self._h, int(dir), float(dt), C.byref(out)))
        return out.value

    def step(self, dt: float, cycle: int) -> None:
        _capi.check(lib().fvs_solver_step(self._h, float(dt), int(cycle)))

    def step_host(self, cons_host, cfl=0.8, t_end=1e300):
        """One split step of a host-resident state, in place (fvs_solver_step_host):
        cons_host is a C-contiguous float64 array or tensor in host memory
        (page-locked for overlapped copies) holding the conservative state."""
        import numpy as np
        if hasattr(cons_host, "data_ptr"):
            if getattr(cons_host, "is_cuda", False):
                raise ValueError("cons_host must live in host memory")
            assert cons_host.numel() == int(np.prod(self.shape()))
            ptr = cons_host.data_ptr()
        else:
            assert cons_host.flags["C_CONTIGUOUS"] and cons_host.dtype == np.float64
            assert cons_host.size == int(np.prod(self.shape()))
            ptr = cons_host.ctypes.data
        st = RunStats()
        _capi.check(lib().fvs_solver_step_host(self._h, C.c_void_p(ptr), float(cfl),
                                               float(t_end), C.byref(st)))
        return st

    def run(self, cfl=0.8, t_end=1.0, max_steps=-1, log_len=0):
        import numpy as np
        log = np.zeros(max(log_len, 1))
        st = RunStats()
        code = lib().fvs_solver_run(self._h, float(cfl), float(t_end), int(max_steps),
                                    log.ctypes.data_as(C.POINTER(C.c_double)), int(log_len),
                                    C.byref(st))
        _capi.check(code)
        return st, log[:min(log_len, st.steps)].copy()


def riemann_features(gamma, rhoL, uL, pL, rhoR, uR, pR, features, pstar=None, labels=None,
                     stream=None) -> None:
    """Features (float32 [n, 5]) and, given p*, the labels log(p*/max(pL, pR))
    of the learned start value for n Riemann problems (device arrays)."""
    n = int(rhoL.numel()) if hasattr(rhoL, "numel") else int(len(rhoL))
    _capi.check(lib().fvs_riemann_features(
        n, float(gamma), _ptr(rhoL), _ptr(uL), _ptr(pL), _ptr(rhoR), _ptr(uR), _ptr(pR),
        _ptr(pstar), _ptr(features), _ptr(labels), _stream(stream)))


def tc_gemm_bf16(A, B, C_out, M, N, K, lda=None, ldb=None, ldc=None, splits=1,
                 accumulate=False, stream=None) -> None:
    """C[M, N] (+)= A[M, K] . B[N, K]^T on the tcgen05 tensor cores (bf16
    operands, fp32 result; device arrays)."""
    _capi.check(lib().fvs_tc_gemm_bf16(
        _ptr(A), int(lda or K), _ptr(B), int(ldb or K), _ptr(C_out), int(ldc or N), int(M),
        int(N), int(K), int(splits), int(bool(accumulate)), _stream(stream)))


class LearnedGuess:
    """The learned Newton start value of the exact Riemann solver (no
    counterpart in the reference): a 5-64-64-1 GELU perceptron trained and
    evaluated with BF16 operands on the tcgen05 tensor cores."""

    def __init__(self, seed: int = 0):
        self._h = C.c_void_p()
        _capi.check(lib().fvs_mlp_create(int(seed), C.byref(self._h)))

    @staticmethod
    def param_count() -> int:
        return int(lib().fvs_mlp_param_count())

    def close(self):
        if self._h:
            lib().fvs_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_normalization(self, features) -> None:
        n = int(features.numel()) // 5 if hasattr(features, "numel") else len(features)
        _capi.check(lib().fvs_mlp_set_normalization(self._h, _ptr(features), n))

    def train(self, features, labels, steps, batch=8192, lr=1e-3, seed=1) -> float:
        n = int(labels.numel()) if hasattr(labels, "numel") else len(labels)
        loss = C.c_float(0.0)
        _capi.check(lib().fvs_mlp_train(self._h, _ptr(features), _ptr(labels), n, int(steps),
                                        int(batch), float(lr), int(seed), C.byref(loss)))
        return loss.value

    def gradients(self, features, labels, batch):
        import numpy as np
        g = np.zeros(self.param_count(), dtype=np.float32)
        loss = C.c_float(0.0)
        _capi.check(lib().fvs_mlp_gradients(self._h, _ptr(features), _ptr(labels), int(batch),
                                            g.ctypes.data, C.byref(loss)))
        return g, loss.value

    def predict(self, features, out) -> None:
        n = int(out.numel()) if hasattr(out, "numel") else len(out)
        _capi.check(lib().fvs_mlp_predict(self._h, _ptr(features), n, _ptr(out)))

    def params_device_ptr(self) -> int:
        p = C.c_void_p()
        _capi.check(lib().fvs_mlp_params(self._h, C.byref(p)))
        return int(p.value or 0)

    def master(self):
        import numpy as np
        h = np.zeros(self.param_count(), dtype=np.float32)
        _capi.check(lib().fvs_mlp_get_master(self._h, h.ctypes.data))
        return h

    def set_master(self, params) -> None:
        import numpy as np
        h = np.ascontiguousarray(params, dtype=np.float32)
        assert h.size == self.param_count()
        _capi.check(lib().fvs_mlp_set_master(self._h, h.ctypes.data))


class AmrSolver:
    """A static 2-D AMR patch set (refinement ratio 2) advanced by
    SubcycleFineFirstSolver's coarse steps: one persistent launch per level
    and sweep over a device patch-row table, each coarse step one CUDA graph.
    `hier` has nlevels, n0, bc, dx0, levels [npatch] and boxes [npatch, 4]
    (lo_x, lo_y, hi_x, hi_y), e.g. workloads.AmrHierarchy."""

    def __init__(self, hier, method: Method | None = None):
        import numpy as np
        d = AmrDesc()
        d.rank = 2
        d.nlevels = int(hier.nlevels)
        for k in range(3):
            d.n0[k] = int(hier.n0[k]) if k < 2 else 1
            d.bc[k] = int(hier.bc[k]) if k < 2 else 0
        d.dx0 = float(hier.dx0)
        npatch = len(hier.levels)
        d.npatches = npatch
        self._levels = np.ascontiguousarray(hier.levels, dtype=np.int32)
        self._boxes = (Box * npatch)()
        for p, (x0, y0, x1, y1) in enumerate(np.asarray(hier.boxes).reshape(-1, 4)):
            self._boxes[p].lo[:] = [int(x0), int(y0), 0]
            self._boxes[p].hi[:] = [int(x1), int(y1), 1]
        d.patch_level = self._levels.ctypes.data_as(C.POINTER(C.c_int32))
        d.patch_box = self._boxes
        self.hier = hier
        self.method = method if method is not None else make_method()
        self._h = C.c_void_p()
        _capi.check(lib().fvs_amr_create(C.byref(d), C.byref(self.method), C.byref(self._h)))
        self.size = int(sum(4 * (int(b[2]) - int(b[0])) * (int(b[3]) - int(b[1]))
                            for b in np.asarray(hier.boxes).reshape(-1, 4)))

    def close(self):
        if self._h:
            lib().fvs_amr_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, cons) -> None:
        import numpy as np
        a = np.ascontiguousarray(cons, dtype=np.float64)
        assert a.size == self.size
        _capi.check(lib().fvs_amr_upload(self._h, a.ctypes.data))

    def download(self):
        import numpy as np
        a = np.empty(self.size, dtype=np.float64)
        _capi.check(lib().fvs_amr_download(self._h, a.ctypes.data))
        return a

    def write_plotfile(self, directory) -> None:
        """AMReX plotfile of every level (fub::amrex::PlotfileOutput)."""
        _capi.check(lib().fvs_amr_write_plotfile(self._h, str(directory).encode()))

    def info(self):
        import numpy as np
        nl = int(self.hier.nlevels)
        cells = np.zeros(nl, dtype=np.int64)
        storage = np.zeros(nl, dtype=np.int64)
        ns = C.c_int32(0)
        _capi.check(lib().fvs_amr_info(self._h, cells.ctypes.data, storage.ctypes.data,
                                       C.byref(ns)))
        return {"cells": cells, "storage": storage, "slots": ns.value}

    def stream_handle(self) -> int:
        p = C.c_void_p()
        _capi.check(lib().fvs_amr_stream(self._h, C.byref(p)))
        return int(p.value or 0)

    def stable_dt(self) -> float:
        out = C.c_double(0.0)
        _capi.check(lib().fvs_amr_stable_dt(self._h, C.byref(out)))
        return out.value

    def run(self, cfl=0.8, t_end=1.0, max_steps=-1, log_len=0):
        import numpy as np
        log = np.zeros(max(log_len, 1))
        st = RunStats()
        _capi.check(lib().fvs_amr_run(self._h, float(cfl), float(t_end), int(max_steps),
                                      log.ctypes.data_as(C.POINTER(C.c_double)), int(log_len),
                                      C.byref(st)))
        return st, log[:min(log_len, st.steps)].copy()

    def set_launch(self, level, dir, block, grid, threads_per_row=1) -> None:
        """Launch shape of a level's sweeps in direction dir: threads per
        block, blocks, threads per patch row (1, 2, 4, 8; 32 for the mixed x
        sweep with the lanes of a warp along x)."""
        _capi.check(lib().fvs_amr_set_launch(self._h, int(level), int(dir), int(block),
                                             int(grid), int(threads_per_row)))

    def autotune(self):
        """Tuned [level][direction][block, grid, threads per row]."""
        import numpy as np
        cfg = np.zeros((int(self.hier.nlevels), 2, 3), dtype=np.int32)
        _capi.check(lib().fvs_amr_autotune(self._h, cfg.ctypes.data))
        return cfg
