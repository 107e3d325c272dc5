"""ctypes binding of ``lib/libmi_inverse.so`` (the C ABI in include/mi_inverse.h).

Loading fails loudly when the library has not been built: there is no
CPU or framework fallback behind this module.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

MI_OK = 0
MI_ERR_INVALID_VALUE = -1
MI_ERR_NULL_POINTER = -2
MI_ERR_MISALIGNED = -3
MI_ERR_CUDA = -4
MI_ERR_SCRATCH_LIMIT = -5
MI_NOALLOC_MAX_COUNT = 262144
MI_LANES_ALT_MIN_BATCH = 131072      # contiguous batches from this size follow the tuned lanes per matrix

# flags of mi_device_error
MI_DEVERR_COPY_TIMEOUT, MI_DEVERR_MMA_TIMEOUT = 1, 2

# kernel forms reported by mi_query_launch
MI_FORM_THREAD, MI_FORM_LANES, MI_FORM_ROWS = 1, 2, 3
FORM_NAMES = {MI_FORM_THREAD: "thread", MI_FORM_LANES: "lanes", MI_FORM_ROWS: "rows"}

PIVOT_MODES = {"none": 0, "reference": 1, "reference_serial": 2, "partial": 3}

_lib = None


class MatrixInversionError(RuntimeError):
    """A non-zero status from the C ABI."""

    def __init__(self, status: int, message: str):
        super().__init__(f"mi status {status}: {message}")
        self.status = status


def load(path: str | None = None):
    """Load (once) and type the shared library."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(
            f"CUDA library {path} is not built; run matrixinversion_gb300.build.build() "
            "(or __graft_entry__.build()) first"
        )
    L = ctypes.CDLL(path)
    vp, i32, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64
    L.mi_inverse_f32.argtypes = [vp, vp, vp, i64, i32, i32, vp]
    L.mi_inverse_f32.restype = i32
    L.mi_inverse_cfg_f32.argtypes = [vp, vp, vp, i64, i32, i32, i32, i32, vp]
    L.mi_inverse_cfg_f32.restype = i32
    ip = ctypes.POINTER(ctypes.c_int)
    L.mi_query_config.argtypes = [i32, ip, ip, ip, ip]
    L.mi_query_config.restype = i32
    L.mi_query_launch.argtypes = [i32, i32, i64, i32, ip, ip, ip, ip]
    L.mi_query_launch.restype = i32
    L.mi_device_error.argtypes = [ip, i32]
    L.mi_device_error.restype = i32
    L.mi_set_wait_test.argtypes = [i64, i32]
    L.mi_set_wait_test.restype = i32
    L.mi_serve_scratch_bytes.argtypes = [i64]
    L.mi_serve_scratch_bytes.restype = ctypes.c_size_t
    L.mi_serve_run.argtypes = [i64, vp, vp, vp, vp, vp, vp, vp, vp, i64, vp, ctypes.c_size_t, i64, i32, i32, vp, vp,
                               vp]
    L.mi_serve_run.restype = i32
    L.mi_error_string.argtypes = [i32]
    L.mi_error_string.restype = ctypes.c_char_p
    L.mi_last_cuda_error.argtypes = []
    L.mi_last_cuda_error.restype = ctypes.c_char_p
    L.mi_abi_version.argtypes = []
    L.mi_abi_version.restype = i32
    L.mi_inverse_descr_f32.argtypes = [vp, i64, vp, vp, vp, vp, vp, i64, ctypes.c_uint32, ctypes.c_uint32, vp,
                                       ctypes.c_size_t, vp]
    L.mi_inverse_descr_f32.restype = i32
    L.mi_inverse_descr_noalloc_f32.argtypes = [vp, i64, vp, vp, vp, vp, vp, i64, ctypes.c_uint32, ctypes.c_uint32,
                                               vp]
    L.mi_inverse_descr_noalloc_f32.restype = i32
    L.mi_newton_schulz_f32.argtypes = [vp, vp, i64, i32, i32, vp]
    L.mi_newton_schulz_f32.restype = i32
    L.mi_refine_fp64_f32.argtypes = [vp, vp, vp, i64, i64, i32, vp]
    L.mi_refine_fp64_f32.restype = i32
    L.mi_refine_df_f32.argtypes = [vp, vp, vp, i64, i64, i32, vp]
    L.mi_refine_df_f32.restype = i32
    L.mi_refine_df_next_f32.argtypes = [vp, vp, vp, i64, i64, i32, ctypes.c_float, vp, vp]
    L.mi_refine_df_next_f32.restype = i32
    L.mi_refine_tc_f32.argtypes = [vp, vp, vp, i64, i64, i32, vp]
    L.mi_refine_tc_f32.restype = i32
    L.mi_refine_tc_next_f32.argtypes = [vp, vp, vp, i64, i64, i32, ctypes.c_float, vp, vp]
    L.mi_refine_tc_next_f32.restype = i32
    L.mi_refine_tc_flagged_f32.argtypes = [vp, vp, i64, i32, ctypes.c_float, ctypes.c_float, vp, vp]
    L.mi_refine_tc_flagged_f32.restype = i32
    L.mi_flag_condition_f32.argtypes = [vp, vp, i64, i32, ctypes.c_float, vp, vp]
    L.mi_flag_condition_f32.restype = i32
    L.mi_descr_workspace_bytes.argtypes = [i64]
    L.mi_descr_workspace_bytes.restype = ctypes.c_size_t
    L.mi_set_launch_config.argtypes = [i32, i32, i32]
    L.mi_set_launch_config.restype = i32
    L.mi_get_launch_config.argtypes = [i32, i32, ip]
    L.mi_get_launch_config.restype = i32
    L.mi_set_launch_lanes.argtypes = [i32, i32, i32]
    L.mi_set_launch_lanes.restype = i32
    L.mi_get_launch_lanes.argtypes = [i32, i32, ip, ip]
    L.mi_get_launch_lanes.restype = i32
    L.mi_set_descr_chunk.argtypes = [i32]
    L.mi_set_descr_chunk.restype = i32
    L.mi_get_descr_chunk.argtypes = []
    L.mi_get_descr_chunk.restype = i32
    _lib = L
    return L


def check(status: int) -> None:
    if status != MI_OK:
        L = load()
        msg = L.mi_error_string(status).decode()
        if status == MI_ERR_CUDA:
            msg += ": " + L.mi_last_cuda_error().decode()
        raise MatrixInversionError(status, msg)


def exported_symbols() -> list[str]:
    """Entry points declared in include/mi_inverse.h (the C ABI surface)."""
    return [
        "mi_inverse_f32",
        "mi_inverse_cfg_f32",
        "mi_query_config",
        "mi_error_string",
        "mi_last_cuda_error",
        "mi_abi_version",
        "mi_inverse_descr_f32",
        "mi_descr_workspace_bytes",
        "mi_inverse_descr_noalloc_f32",
        "mi_newton_schulz_f32",
        "mi_refine_fp64_f32",
        "mi_refine_df_f32",
        "mi_refine_df_next_f32",
        "mi_refine_tc_f32",
        "mi_refine_tc_next_f32",
        "mi_refine_tc_flagged_f32",
        "mi_flag_condition_f32",
        "mi_set_launch_config",
        "mi_get_launch_config",
        "mi_set_launch_lanes",
        "mi_get_launch_lanes",
        "mi_set_descr_chunk",
        "mi_get_descr_chunk",
        "mi_set_wait_test",
        "mi_serve_scratch_bytes",
        "mi_serve_run",
    ]
