"""GB300-native batched small-matrix inverter (n <= 32, FP32).

Python surface of the C ABI in ``include/mi_inverse.h``.  The hot path is the
hand-written sm_103a kernel in ``csrc/``; PyTorch only supplies device memory
and streams.  Nothing here falls back to a CPU or framework implementation:
a missing library or a host tensor is an error.

The reference (sumukhashridhar/matrixInversion) has no library API: its entry
is one templated kernel launch per process, batched_lu_subwarp<float, n, T,
mpb, N>(d_A), in place on row-major matrices (parallel_pivot/
luBatchedInplace.cu:127).  ``batched_inverse`` is that launch for any batch
and n, with the pivot choice of the reference's variants.
"""
from __future__ import annotations

import ctypes

from . import _lib
from ._lib import MatrixInversionError, PIVOT_MODES

__all__ = [
    "batched_inverse",
    "batched_inverse_",
    "query_config",
    "query_launch",
    "device_error",
    "MatrixInversionError",
    "PIVOT_MODES",
    "pivot_mode",
]


def pivot_mode(pivot) -> int:
    """Map the ``pivot`` argument to the C ABI mode.

    True / "reference"  -> parallel_pivot's argmax rule (bit-exact pivots)
    "reference_serial"  -> serial_pivot's sequential argmax
    "partial"           -> textbook partial pivoting (getrf)
    False / "none"      -> no pivoting (templated/ kernel)
    """
    if pivot is True:
        return PIVOT_MODES["reference"]
    if pivot is False or pivot is None:
        return PIVOT_MODES["none"]
    if isinstance(pivot, str) and pivot in PIVOT_MODES:
        return PIVOT_MODES[pivot]
    if isinstance(pivot, int) and pivot in PIVOT_MODES.values():
        return int(pivot)
    raise ValueError(f"unknown pivot mode {pivot!r}; expected one of {sorted(PIVOT_MODES)} or a bool")


def _stream_handle(stream):
    import torch

    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


def batched_inverse_(A, pivot=True, *, perm=None, info=None, stream=None, threads_per_block: int = 0,
                     grid_blocks: int = 0):
    """Invert ``A`` ([batch, n, n] or [n, n], float32, CUDA, contiguous) in place.

    perm / info: optional preallocated int32 CUDA tensors [batch, n] / [batch].
    Returns (A, perm, info).
    """
    import torch

    if not isinstance(A, torch.Tensor) or not A.is_cuda:
        raise TypeError("batched_inverse needs a CUDA tensor (there is no host implementation)")
    if A.dtype != torch.float32:
        raise TypeError(f"batched_inverse computes in float32, got {A.dtype}")
    if A.dim() not in (2, 3) or A.shape[-1] != A.shape[-2]:
        raise ValueError(f"expected [batch, n, n] or [n, n], got {tuple(A.shape)}")
    if not A.is_contiguous():
        raise ValueError("A must be contiguous (row-major matrices at offset b*n*n)")
    n = A.shape[-1]
    batch = A.shape[0] if A.dim() == 3 else 1
    mode = pivot_mode(pivot)
    dev = A.device
    for name, t, shape in (("perm", perm, (batch, n)), ("info", info, (batch,))):
        if t is not None:
            if not (t.is_cuda and t.dtype == torch.int32 and t.is_contiguous() and t.device == dev):
                raise ValueError(f"{name} must be a contiguous int32 tensor on {dev}")
            if t.numel() != int(torch.Size(shape).numel()):
                raise ValueError(f"{name} must hold {shape} elements")
    L = _lib.load()
    with torch.cuda.device(dev):
        st = _stream_handle(stream)
        status = L.mi_inverse_cfg_f32(
            ctypes.c_void_p(A.data_ptr()),
            ctypes.c_void_p(perm.data_ptr() if perm is not None else 0),
            ctypes.c_void_p(info.data_ptr() if info is not None else 0),
            batch, n, mode, int(threads_per_block), int(grid_blocks), st,
        )
    _lib.check(status)
    return A, perm, info


def batched_inverse(A, pivot=True, *, return_perm: bool = True, return_info: bool = True, stream=None,
                    threads_per_block: int = 0):
    """Out-of-place batched inverse: returns (Ainv, perm, info).

    ``A`` is [batch, n, n] (or [n, n]) float32 on a CUDA device; ``pivot`` is a
    bool or one of "reference", "reference_serial", "partial", "none".
    perm[b][i] is the input row that ends at row i (the reference's pivots[]);
    info[b] is 0 or the 1-based step of the first exactly-zero pivot.
    """
    import torch

    if not isinstance(A, torch.Tensor) or not A.is_cuda:
        raise TypeError("batched_inverse needs a CUDA tensor (there is no host implementation)")
    X = A.contiguous().clone()
    n = X.shape[-1]
    batch = X.shape[0] if X.dim() == 3 else 1
    perm = torch.empty((batch, n), dtype=torch.int32, device=X.device) if return_perm else None
    info = torch.empty((batch,), dtype=torch.int32, device=X.device) if return_info else None
    batched_inverse_(X, pivot, perm=perm, info=info, stream=stream, threads_per_block=threads_per_block)
    if X.dim() == 2:
        perm = perm[0] if perm is not None else None
        info = info[0] if info is not None else None
    return X, perm, info


def query_config(n: int) -> dict:
    """Launch geometry for size n without pivoting or with the reference
    rules on large batches (lanes per matrix, matrices per warp, ...);
    :func:`query_launch` covers every pivot mode and batch size."""
    L = _lib.load()
    vals = [ctypes.c_int() for _ in range(4)]
    _lib.check(L.mi_query_config(int(n), *[ctypes.byref(v) for v in vals]))
    return {
        "lanes_per_matrix": vals[0].value,
        "matrices_per_warp": vals[1].value,
        "smem_bytes_per_warp": vals[2].value,
        "default_threads_per_block": vals[3].value,
    }


def query_launch(n: int, pivot=True, batch: int = 1_000_000, threads_per_block: int = 0) -> dict:
    """The kernel a contiguous ``batched_inverse_`` call of ``batch`` n x n
    matrices launches: its form ("thread": one thread per matrix; "lanes": a
    group of lanes per matrix; "rows": 16 lanes per matrix owning whole rows,
    partial pivoting), lanes per matrix, matrices per warp and threads per
    block.  ``knob`` says whether ``threads_per_block`` (the NUMTHREADS knob)
    reaches the launch -- the lane-group form only.  Needs no GPU."""
    L = _lib.load()
    vals = [ctypes.c_int() for _ in range(4)]
    _lib.check(L.mi_query_launch(int(n), pivot_mode(pivot), int(batch), int(threads_per_block),
                                 *[ctypes.byref(v) for v in vals]))
    form = vals[0].value
    return {
        "form": _lib.FORM_NAMES[form],
        "lanes_per_matrix": vals[1].value,
        "matrices_per_warp": vals[2].value,
        "threads_per_block": vals[3].value,
        "knob": form == _lib.MI_FORM_LANES,
    }


def device_error(clear: bool = True) -> int:
    """Flags of waits that ran out on the current device since the last clear
    (0 = none; MI_DEVERR_COPY_TIMEOUT = 1: a tile copy never arrived,
    MI_DEVERR_MMA_TIMEOUT = 2: a tensor-core product never completed).  The
    affected calls returned normally with some matrices left unwritten.
    Synchronise the streams that ran the work first."""
    L = _lib.load()
    v = ctypes.c_int(0)
    _lib.check(L.mi_device_error(ctypes.byref(v), 1 if clear else 0))
    return v.value
