"""ctypes declarations of libfvs_gb300.so (include/fvs_gpu.h).

The library is built in-tree by finitevolumesolver_gb300.build; loading
fails loudly when it is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "libfvs_gb300.so"
HEADER = PKG_DIR.parent / "include" / "fvs_gpu.h"

FVS_OK = 0
FVS_ERR_INVALID = 1
FVS_ERR_CUDA = 2
FVS_ERR_DT_TOO_LARGE = 3
FVS_ERR_UNSUPPORTED = 4
FVS_ERR_NO_DEVICE = 5
FVS_ERR_STATE = 6
FVS_ERR_IO = 7

STATUS_NAMES = {0: "OK", 1: "INVALID", 2: "CUDA", 3: "DT_TOO_LARGE", 4: "UNSUPPORTED",
                5: "NO_DEVICE", 6: "STATE"}


class Shape(C.Structure):
    _fields_ = [("kind", C.c_int32), ("inverted", C.c_int32), ("p", C.c_double * 3),
                ("nvertices", C.c_int32), ("reserved", C.c_int32),
                ("xy", C.POINTER(C.c_double))]


class Box(C.Structure):
    _fields_ = [("lo", C.c_int32 * 3), ("hi", C.c_int32 * 3)]


class Method(C.Structure):
    _fields_ = [("flux_method", C.c_int32), ("limiter", C.c_int32), ("precision", C.c_int32),
                ("guess", C.c_int32), ("max_iterations", C.c_int32), ("reserved", C.c_int32),
                ("tolerance", C.c_double), ("gamma", C.c_double), ("mlp_params", C.c_void_p)]


class GridDesc(C.Structure):
    _fields_ = [("rank", C.c_int32), ("n", C.c_int32 * 3), ("bc", C.c_int32 * 3),
                ("dt_rule", C.c_int32), ("dx", C.c_double * 3)]


class RunStats(C.Structure):
    _fields_ = [("time", C.c_double), ("steps", C.c_int32), ("restarts", C.c_int32),
                ("status", C.c_int32), ("reserved", C.c_int32), ("last_dt", C.c_double)]


class AmrDesc(C.Structure):
    _fields_ = [("rank", C.c_int32), ("nlevels", C.c_int32), ("n0", C.c_int32 * 3),
                ("bc", C.c_int32 * 3), ("dx0", C.c_double), ("npatches", C.c_int32),
                ("reserved", C.c_int32), ("patch_level", C.POINTER(C.c_int32)),
                ("patch_box", C.POINTER(Box))]


class FvsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"fvs error {STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


_lib = None
_VP = C.c_void_p
_DP = C.POINTER(C.c_double)


def header_symbols() -> list[str]:
    """Function names declared in include/fvs_gpu.h."""
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w[\w\s\*]*?\b(fvs_\w+)\s*\(", text,
                                 re.M)))


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build it with finitevolumesolver_gb300.build.build() "
            "(the package has no CPU fallback)")
    L = C.CDLL(str(LIB_PATH))
    P = C.POINTER
    L.fvs_method_default.argtypes = [P(Method)]
    L.fvs_method_default.restype = None
    L.fvs_last_error.restype = C.c_char_p
    L.fvs_abi_version.restype = C.c_int
    L.fvs_device_count.restype = C.c_int
    L.fvs_compute_numeric_fluxes.argtypes = [P(Method), C.c_int, _VP, Box, _VP, Box, C.c_double,
                                             C.c_double, C.c_int, _VP]
    L.fvs_compute_stable_dt.argtypes = [P(Method), C.c_int, _VP, Box, C.c_double, C.c_int,
                                        C.c_int, _DP, _VP]
    L.fvs_compute_max_speed.argtypes = [P(Method), C.c_int, _VP, Box, C.c_int, C.c_int, _VP,
                                         _VP]
    L.fvs_compute_stable_dt_noalloc.argtypes = [P(Method), C.c_int, _VP, Box, C.c_double,
                                                C.c_int, C.c_int, _DP, _VP]
    L.fvs_update_conservatively.argtypes = [_VP, Box, _VP, Box, _VP, Box, C.c_int, C.c_double,
                                            C.c_double, C.c_int, _VP]
    L.fvs_update_conservatively_region.argtypes = [_VP, Box, Box, _VP, Box, _VP, Box, C.c_int,
                                                   C.c_double, C.c_double, C.c_int, _VP]
    L.fvs_complete_from_cons.argtypes = [C.c_int, C.c_double, _VP, Box, _VP, Box, Box, _VP]
    L.fvs_patch_ctx_create.argtypes = [P(_VP)]
    L.fvs_patch_ctx_destroy.argtypes = [_VP]
    L.fvs_compute_numeric_fluxes_host.argtypes = [_VP, P(Method), C.c_int, _VP, Box, _VP, Box,
                                                  C.c_double, C.c_double, C.c_int]
    L.fvs_compute_stable_dt_host.argtypes = [_VP, P(Method), C.c_int, _VP, Box, C.c_double,
                                             C.c_int, C.c_int, P(C.c_double)]
    L.fvs_update_conservatively_host.argtypes = [_VP, _VP, Box, _VP, Box, _VP, Box, C.c_int,
                                                 C.c_double, C.c_double, C.c_int]
    L.fvs_complete_from_cons_host.argtypes = [_VP, C.c_int, C.c_double, _VP, Box, _VP, Box, Box]
    L.fvs_solver_create.argtypes = [P(GridDesc), P(Method), P(_VP)]
    L.fvs_solver_destroy.argtypes = [_VP]
    L.fvs_solver_upload.argtypes = [_VP, _VP]
    L.fvs_solver_step_host.argtypes = [_VP, _VP, C.c_double, C.c_double, P(RunStats)]
    L.fvs_solver_download.argtypes = [_VP, _VP]
    L.fvs_solver_write_plotfile.argtypes = [_VP, C.c_char_p]
    L.fvs_solver_state_device.argtypes = [_VP, P(_VP)]
    L.fvs_solver_set_tiling.argtypes = [_VP, C.c_int]
    L.fvs_solver_set_launch.argtypes = [_VP, C.c_int, C.c_int, C.c_int]
    L.fvs_solver_autotune.argtypes = [_VP, P(C.c_int)]
    L.fvs_solver_tuning.argtypes = [_VP, _VP, _VP]
    L.fvs_solver_stable_dt.argtypes = [_VP, C.c_int, _DP]
    L.fvs_solver_sweep.argtypes = [_VP, C.c_int, C.c_double, _DP]
    L.fvs_solver_step.argtypes = [_VP, C.c_double, C.c_int]
    L.fvs_solver_run.argtypes = [_VP, C.c_double, C.c_double, C.c_int, _DP, C.c_int,
                                 P(RunStats)]
    L.fvs_solver_stream.argtypes = [_VP, P(_VP)]
    L.fvs_solver_newton_stats.argtypes = [_VP, P(C.c_uint64), P(C.c_uint64), P(C.c_uint64),
                                          C.c_int]
    L.fvs_exact_riemann_star.argtypes = [P(Method), C.c_int64, _VP, _VP, _VP, _VP, _VP, _VP, _VP,
                                         _VP, _VP, _VP, _VP]
    L.fvs_cutcell_ghost_layers.restype = C.c_int
    L.fvs_solver_set_embedded_circles.argtypes = [_VP, _VP, C.c_int, C.c_double, C.c_double]
    L.fvs_solver_cutcell_geometry.argtypes = [_VP, _VP, _VP, _VP, _VP, _VP, _VP]
    L.fvs_solver_set_embedded_geometry.argtypes = [_VP, P(Shape), C.c_int, C.c_double,
                                                   C.c_double]
    L.fvs_solver_cutcell_shielded.argtypes = [_VP, C.c_int, _VP, _VP, _VP, _VP, _VP, _VP]
    L.fvs_solver_set_cycle.argtypes = [_VP, C.c_int64]
    L.fvs_solver_set_time.argtypes = [_VP, C.c_double]
    L.fvs_amr_create.argtypes = [P(AmrDesc), P(Method), P(_VP)]
    L.fvs_amr_destroy.argtypes = [_VP]
    L.fvs_amr_upload.argtypes = [_VP, _VP]
    L.fvs_amr_download.argtypes = [_VP, _VP]
    L.fvs_amr_write_plotfile.argtypes = [_VP, C.c_char_p]
    L.fvs_amr_info.argtypes = [_VP, _VP, _VP, _VP]
    L.fvs_amr_stream.argtypes = [_VP, P(_VP)]
    L.fvs_amr_stable_dt.argtypes = [_VP, _DP]
    L.fvs_amr_run.argtypes = [_VP, C.c_double, C.c_double, C.c_int, _DP, C.c_int, P(RunStats)]
    L.fvs_amr_set_launch.argtypes = [_VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
    L.fvs_amr_autotune.argtypes = [_VP, _VP]
    L.fvs_mlp_param_count.restype = C.c_int
    L.fvs_mlp_create.argtypes = [C.c_uint64, P(_VP)]
    L.fvs_mlp_destroy.argtypes = [_VP]
    L.fvs_riemann_features.argtypes = [C.c_int64, C.c_double] + [_VP] * 10
    L.fvs_mlp_set_normalization.argtypes = [_VP, _VP, C.c_int64]
    L.fvs_mlp_train.argtypes = [_VP, _VP, _VP, C.c_int64, C.c_int, C.c_int, C.c_float,
                                C.c_uint64, P(C.c_float)]
    L.fvs_mlp_gradients.argtypes = [_VP, _VP, _VP, C.c_int, _VP, P(C.c_float)]
    L.fvs_mlp_predict.argtypes = [_VP, _VP, C.c_int64, _VP]
    L.fvs_mlp_params.argtypes = [_VP, P(_VP)]
    L.fvs_mlp_get_master.argtypes = [_VP, _VP]
    L.fvs_mlp_set_master.argtypes = [_VP, _VP]
    L.fvs_tc_gemm_bf16.argtypes = [_VP, C.c_int, _VP, C.c_int, _VP, C.c_int, C.c_int, C.c_int,
                                   C.c_int, C.c_int, C.c_int, _VP]
    _lib = L
    return L


def check(code: int) -> None:
    if code != FVS_OK:
        msg = load().fvs_last_error()
        raise FvsError(code, msg.decode() if msg else "")
