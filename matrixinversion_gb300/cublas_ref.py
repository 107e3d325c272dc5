"""cuBLAS getrfBatched + getriBatched on a device batch (the comparison point
of the measurements; not the product path)."""
from __future__ import annotations

import ctypes

from . import build as _build

_lib = None


def _load():
    global _lib
    if _lib is None:
        _build.build_comparator()
        L = ctypes.CDLL(_build.LIB_CUBLAS)
        vp = ctypes.c_void_p
        L.mi_cublas_inverse_f32.argtypes = [vp, vp, vp, vp, ctypes.c_int64, ctypes.c_int, vp,
                                            ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
        L.mi_cublas_inverse_f32.restype = ctypes.c_int
        L.mi_cublas_last_error.restype = ctypes.c_char_p
        _lib = L
    return _lib


def inverse(A, timed: bool = False):
    """Invert a CUDA float32 batch [batch, n, n] with cuBLAS (A is copied).

    Returns (Ainv, piv, info) and, with timed=True, (getrf_ms, getri_ms).
    """
    import torch

    L = _load()
    W = A.contiguous().clone()
    C = torch.empty_like(W)
    b, n = W.shape[0], W.shape[-1]
    piv = torch.empty((b, n), dtype=torch.int32, device=W.device)
    info = torch.empty((b,), dtype=torch.int32, device=W.device)
    t1, t2 = ctypes.c_float(), ctypes.c_float()
    rc = L.mi_cublas_inverse_f32(W.data_ptr(), C.data_ptr(), piv.data_ptr(), info.data_ptr(), b, n,
                                 torch.cuda.current_stream().cuda_stream,
                                 ctypes.byref(t1) if timed else None, ctypes.byref(t2) if timed else None)
    if rc != 0:
        raise RuntimeError("cuBLAS inverse failed: " + L.mi_cublas_last_error().decode())
    if timed:
        return (C, piv, info), (t1.value, t2.value)
    return C, piv, info


def inverse_into(W, C, piv, info, stream=None):
    """In-place form for timing loops: W is overwritten by the LU factors."""
    import torch

    L = _load()
    st = (stream or torch.cuda.current_stream()).cuda_stream
    rc = L.mi_cublas_inverse_f32(W.data_ptr(), C.data_ptr(), piv.data_ptr(), info.data_ptr(), W.shape[0],
                                 W.shape[-1], st, None, None)
    if rc != 0:
        raise RuntimeError("cuBLAS inverse failed: " + L.mi_cublas_last_error().decode())
