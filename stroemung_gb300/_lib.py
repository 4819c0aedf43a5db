"""ctypes binding of the C ABI declared in include/stroemung_gpu.h.

Loads the in-tree ``_build/libstroemung_gb300.so`` (building it when absent).
There is no fallback: if the library cannot be built or loaded, or the
device is not an sm_103 GPU, calls raise.
"""
from __future__ import annotations

import ctypes
import math
from pathlib import Path

HERE = Path(__file__).resolve().parent

STRM_OK = 0
STRM_ERR_THIN_WALL = 1
STRM_ERR_BAD_BOUNDARY = 2
STRM_ERR_NONFINITE = 3
STRM_ERR_TIMEOUT = 4
STRM_ERR_CUDA = 5
STRM_ERR_INVALID = 6
STRM_ERR_NO_DEVICE = 7

FIELD_U, FIELD_V, FIELD_P, FIELD_F, FIELD_G, FIELD_RHS = range(6)
SOR_RED_BLACK, SOR_LEXICOGRAPHIC = 0, 1
ARITH_EXACT, ARITH_FAST = 0, 1
PREC_FP64, PREC_MIXED = 0, 1
EXEC_GRAPH, EXEC_EAGER = 0, 1
BATCH_GRAPH_LOOP, BATCH_PERSISTENT = 0, 1
NORM_ALL_INTERIOR, NORM_FLUID, NORM_FLUID_MEAN_FREE = 0, 1, 2
SWEEPS_DEFAULT, SWEEPS_PER_COLOUR, SWEEPS_COUNT = 0, 1, 8
STOP_REFERENCE, STOP_STRICT, STOP_RELATIVE = 0, 1, 2


class Params(ctypes.Structure):
    _fields_ = [
        ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("delt", ctypes.c_double),
        ("gamma", ctypes.c_double), ("reynolds", ctypes.c_double), ("eps", ctypes.c_double),
        ("omega", ctypes.c_double), ("max_iterations", ctypes.c_uint32),
        ("iterations", ctypes.c_uint32), ("time", ctypes.c_double),
        ("initial_norm_squared", ctypes.c_double), ("tau", ctypes.c_double),
    ]


class Mode(ctypes.Structure):
    _fields_ = [("sor_order", ctypes.c_int), ("arithmetic", ctypes.c_int),
                ("precision", ctypes.c_int), ("strict_eps", ctypes.c_int),
                ("inner_sweeps", ctypes.c_int), ("execution", ctypes.c_int),
                ("norm_cells", ctypes.c_int), ("sweep_schedule", ctypes.c_int)]


class State(ctypes.Structure):
    _fields_ = [
        ("time", ctypes.c_double), ("iterations", ctypes.c_uint64), ("delt", ctypes.c_double),
        ("initial_norm_squared", ctypes.c_double), ("fluid_cells", ctypes.c_double),
        ("pressure_range", ctypes.c_double * 2), ("speed_range", ctypes.c_double * 2),
        ("last_sor_iterations", ctypes.c_uint32), ("last_norm_squared", ctypes.c_double),
        ("last_converged", ctypes.c_uint32),
    ]


class StepStats(ctypes.Structure):
    _fields_ = [("sor_iterations", ctypes.c_uint32), ("converged", ctypes.c_uint32),
                ("norm_squared", ctypes.c_double), ("delt", ctypes.c_double)]


class DeviceView(ctypes.Structure):
    _fields_ = [("u", ctypes.c_void_p), ("v", ctypes.c_void_p), ("p", ctypes.c_void_p),
                ("f", ctypes.c_void_p), ("g", ctypes.c_void_p), ("rhs", ctypes.c_void_p),
                ("flags", ctypes.c_void_p), ("nx", ctypes.c_int), ("ny", ctypes.c_int),
                ("pitch", ctypes.c_int), ("stream", ctypes.c_void_p)]


# Every function include/stroemung_gpu.h declares, with its ctypes signature.
_vp = ctypes.c_void_p
_dp = ctypes.POINTER(ctypes.c_double)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_u8d = ctypes.c_void_p
_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)
_fp = ctypes.c_void_p  # device float pointers are passed as plain addresses
_i = ctypes.c_int
SIGNATURES = {
    "strm_create": [ctypes.POINTER(Params), ctypes.c_int, ctypes.c_int, _u8p, _dp, _dp, _dp, _dp,
                    ctypes.POINTER(_vp), _i64p],
    "strm_destroy": [_vp],
    "strm_set_mode": [_vp, ctypes.POINTER(Mode)],
    "strm_tick": [_vp, ctypes.POINTER(ctypes.c_uint32), _dp],
    "strm_step_n": [_vp, ctypes.c_int, ctypes.POINTER(StepStats)],
    "strm_download": [_vp, ctypes.c_int, _dp],
    "strm_upload": [_vp, ctypes.c_int, _dp],
    "strm_download_cells": [_vp, _u8p, _u8p],
    "strm_edit_cells": [_vp, ctypes.c_int, _i32p, _i32p, _u8p, _dp, _i64p],
    "strm_get_state": [_vp, ctypes.POINTER(State)],
    "strm_set_boundary_u_and_v": [_vp],
    "strm_calculate_f_g_rhs": [_vp],
    "strm_copy_pressure_to_boundaries": [_vp],
    "strm_calculate_norm_squared": [_vp, _dp],
    "strm_set_u_and_v": [_vp],
    "strm_calculate_pressure_range": [_vp],
    "strm_calculate_speed_range": [_vp],
    "strm_device_view_get": [_vp, ctypes.POINTER(DeviceView)],
    "strm_sor_sweeps": [_vp, ctypes.c_int, _dp],
    "strm_tick_prepare": [_vp],
    "strm_tick_solve": [_vp, ctypes.POINTER(ctypes.c_uint32), _dp],
    "strm_export_planes": [_vp, _vp, _vp, _vp],
    "strm_autotune_sweeps": [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int), _dp],
    "strm_set_programmatic_launch": [ctypes.c_int],
    "strm_residual_history": [_vp, _dp, ctypes.c_int, ctypes.POINTER(ctypes.c_int)],
    "strm_batch_create": [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int,
                          ctypes.POINTER(ctypes.c_void_p)],
    "strm_batch_destroy": [_vp],
    "strm_batch_step": [_vp, ctypes.c_int, _vp],
    "strm_batch_prepare": [_vp],
    "strm_batch_solve": [_vp, _vp],
    "strm_batch_set_schedule": [_vp, ctypes.c_int],
    "strm_batch_set_solver": [_vp, ctypes.c_int, ctypes.c_uint64],
    "strm_batch_autotune": [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int), _dp],
    "strm_apply_correction": [_vp, _vp, ctypes.c_double],
    "strm_copy_field_device": [_vp, ctypes.c_int, _vp, ctypes.c_int],
    "strm_judge_correction": [_vp, _vp, ctypes.c_double, ctypes.c_int, _dp, _dp,
                              ctypes.POINTER(ctypes.c_int)],
    "strm_render_rgba": [_vp, ctypes.c_int, _u8p],
    "strm_synchronize": [_vp],
    "strm_norm_squared_noalloc": [_dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_double, ctypes.c_double, ctypes.c_double, _dp, _vp],
    "strm_host_classify": [ctypes.c_int, ctypes.c_int, _u8p, _u8p, _dp, _i64p],
    "strm_host_boundary_pass": [ctypes.c_int, ctypes.c_int, _u8p, _dp, _dp, _dp, _dp, _dp],
    "strm_last_error": [ctypes.c_char_p, ctypes.c_size_t],
    # include/stroemung_nn.h
    "strm_nn_set_sync": [_i],
    "strm_nn_set_conv_tma": [_i],
    "strm_nn_tune_conv_tma": [_i, _i, _i, _i],
    "strm_nn_status": [_vp],
    "strm_nn_gemm_bf16": [_vp, _vp, _fp, _i, _i, _i, _vp],
    "strm_nn_conv3x3": [_vp, _i, _i, _vp, _i, _fp, _vp, _fp, _i, _i, _i, _i, _i, _i, _vp],
    "strm_nn_conv3x3_head": [_vp, _i, _i, _vp, _i, _fp, _vp, _i, _i, _i, _i, _i, _fp, _fp, _fp,
                             _vp],
    "strm_nn_conv3x3_wgrad": [_vp, _i, _i, _i, _vp, _i, _vp, _i, _fp, _i, _i, _i, _i, _vp],
    "strm_nn_avgpool": [_vp, _i, _vp, _i, _i, _i, _i, _i, _vp],
    "strm_nn_avgpool_bwd": [_vp, _i, _vp, _i, _i, _i, _i, _i, _i, _vp],
    "strm_nn_upsample": [_vp, _i, _vp, _i, _i, _i, _i, _i, _vp],
    "strm_nn_upsample_bwd": [_vp, _i, _vp, _i, _i, _i, _i, _i, _vp],
    "strm_nn_relu_mask": [_vp, _i, _vp, _i, _vp, _i, ctypes.c_longlong, _i, _vp],
    "strm_nn_bias_grad": [_vp, _i, _vp, _i, _fp, ctypes.c_longlong, _i, _vp],
    "strm_nn_flip_weights": [_vp, _i, _i, _i, _vp, _i, _i, _vp],
    "strm_nn_head": [_vp, _i, _i, _fp, _fp, _fp, ctypes.c_longlong, _vp],
    "strm_nn_zero": [_vp, ctypes.c_longlong, _vp],
    "strm_nn_error_loss": [_fp, _fp, _fp, _u8d, _fp, ctypes.c_float, _fp, _fp, _fp, _i, _i, _i,
                           _vp],
    "strm_nn_head_bwd": [_vp, _i, _i, _fp, _fp, _vp, _i, _fp, _fp, ctypes.c_longlong, _vp],
    "strm_nn_prepare_input": [_fp, _u8d, _fp, _fp, _fp, _fp, ctypes.c_float, _vp, _i, _i, _i,
                              _vp],
    "strm_nn_residual_loss": [_fp, _fp, _u8d, _fp, _fp, ctypes.c_float, ctypes.c_float,
                              ctypes.c_float, _fp, _fp, _fp, _fp, _i, _i, _i, _vp],
    "strm_nn_residual_loss_grad": [_fp, _u8d, _fp, _fp, ctypes.c_float, ctypes.c_float,
                                   ctypes.c_float, _fp, _fp, _i, _i, _i, _vp],
    "strm_nn_adam": [_fp, _fp, _fp, _fp, ctypes.c_longlong, ctypes.c_float, ctypes.c_float,
                     ctypes.c_float, ctypes.c_float, _i, _vp, _vp],
    "strm_abi_version": [],
}

_lib = None


def library_path() -> Path:
    from . import build as _build
    return _build.LIB


def load(build_if_missing: bool = True):
    """Loads (building first when needed) the in-tree C-ABI library."""
    global _lib
    if _lib is not None:
        return _lib
    from . import build as _build
    path = _build.LIB
    if build_if_missing:
        _build.build()
    if not path.exists():
        raise RuntimeError(f"stroemung_gb300 native library missing at {path}")
    L = ctypes.CDLL(str(path))
    for name, args in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    _lib = L
    return L


class StroemungError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class BoundaryTooThinError(StroemungError):
    """Mirror of SimulationGridError::BoundaryTooThinError (src/grid/mod.rs:57-58)."""


class NonFiniteError(StroemungError):
    pass


def last_error() -> str:
    buf = ctypes.create_string_buffer(1024)
    load().strm_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(code: int) -> None:
    if code == STRM_OK:
        return
    msg = last_error()
    if code == STRM_ERR_THIN_WALL:
        raise BoundaryTooThinError(code, msg)
    if code == STRM_ERR_NONFINITE:
        raise NonFiniteError(code, msg)
    raise StroemungError(code, msg)


NAN = math.nan
