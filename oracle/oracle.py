"""Python handle on the oracle (test infrastructure, never the product path).

Wraps ``_build/libmi_oracle.so`` (the C restatement in ``mi_oracle.c``) and,
where it was built, ``_ref/libref_emu.so`` (the reference's own kernel headers
run on host threads).  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmi_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref_emu.so")

PIVOT_NONE, PIVOT_REFERENCE, PIVOT_REFERENCE_SERIAL, PIVOT_PARTIAL = 0, 1, 2, 3
MODES = {"none": 0, "reference": 1, "reference_serial": 2, "partial": 3}

_lib = None
_ref = None

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64 = ctypes.c_int64


def build(quiet: bool = True, ref_root: str | None = None) -> None:
    """Compile the oracle library, and the reference emulation when the
    reference project's root is given (ref_root, else the MI_REF_ROOT
    environment variable) and holds its sources."""
    ref_root = ref_root or os.environ.get("MI_REF_ROOT", "")
    out = subprocess.run(["make", "-C", HERE, "all", f"REF_ROOT={ref_root}"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.mi_or_gen_uniform.argtypes = [ctypes.c_uint32, _i64, _f32p]
        L.mi_or_batch_pivots.argtypes = [_f32p, _i64, ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p]
        L.mi_or_batch_inverse_f64.argtypes = [_f32p, _i64, ctypes.c_int, ctypes.c_int, _f64p, _i32p, _i32p]
        L.mi_or_batch_ref_inverse_f32.argtypes = [_f32p, _i64, ctypes.c_int, ctypes.c_int, _i32p, _i32p]
        L.mi_or_batch_residual.argtypes = [_f32p, _f32p, _i64, ctypes.c_int, _f64p]
        L.mi_or_num_threads.restype = ctypes.c_int
        L.mi_or_set_num_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref_lib():
    """The reference kernels on host threads; None where they were not built."""
    global _ref
    if _ref is None and ref_available():
        R = ctypes.CDLL(REF_PATH)
        for name in ("ref_emu_parallel_pivot_run", "ref_emu_serial_pivot_run", "ref_emu_templated_run"):
            fn = getattr(R, name)
            fn.argtypes = [_f32p, ctypes.c_void_p, _i64, ctypes.c_int]
            fn.restype = ctypes.c_int
        _ref = R
    return _ref


# ----------------------------------------------------------------------------
def uniform(seed: int, batch: int, n: int) -> np.ndarray:
    """batch x n x n float32, uniform [-1, 1) from MT19937(seed)."""
    out = np.empty(batch * n * n, dtype=np.float32)
    lib().mi_or_gen_uniform(seed & 0xFFFFFFFF, out.size, out)
    return out.reshape(batch, n, n)


def uniform_numpy(seed: int, count: int) -> np.ndarray:
    """Same stream as :func:`uniform` through numpy's MT19937 (RandomState)."""
    u = np.random.RandomState(seed).randint(0, 2**32, size=count, dtype=np.uint32)
    return ((u >> 8).astype(np.int64) - (1 << 23)).astype(np.float32) * np.float32(2.0**-23)


def pivots(A: np.ndarray, mode: str = "reference", threads_per_matrix: int | None = None) -> np.ndarray:
    A = np.ascontiguousarray(A, dtype=np.float32)
    b, n, _ = A.shape
    T = n if threads_per_matrix is None else threads_per_matrix
    out = np.empty((b, n), dtype=np.int32)
    lib().mi_or_batch_pivots(A.reshape(-1), b, n, MODES[mode], T, out.reshape(-1))
    return out


def inverse_f64(A: np.ndarray, mode: str = "partial"):
    """FP64 LU-inverse; returns (X float64, perm int32, info int32)."""
    A = np.ascontiguousarray(A, dtype=np.float32)
    b, n, _ = A.shape
    X = np.empty((b, n, n), dtype=np.float64)
    perm = np.empty((b, n), dtype=np.int32)
    info = np.empty(b, dtype=np.int32)
    lib().mi_or_batch_inverse_f64(A.reshape(-1), b, n, MODES[mode], X.reshape(-1), perm.reshape(-1), info)
    return X, perm, info


def ref_inverse_f32(A: np.ndarray, mode: str = "reference"):
    """The reference algorithm in FP32 on the host; returns (X, perm, info)."""
    X = np.array(A, dtype=np.float32, copy=True, order="C")
    b, n, _ = X.shape
    perm = np.empty((b, n), dtype=np.int32)
    info = np.empty(b, dtype=np.int32)
    lib().mi_or_batch_ref_inverse_f32(X.reshape(-1), b, n, MODES[mode], perm.reshape(-1), info)
    return X, perm, info


def lu_growth_bound(A: np.ndarray, perm: np.ndarray, X64: np.ndarray | None = None) -> np.ndarray:
    """|| |L| |U| |X| ||_inf per matrix, with P A = L U factored in FP64 in the
    given pivot order (perm[b][k] = input row placed at step k, no further
    pivoting) and X the FP64 inverse.  n u times this is the componentwise
    residual bound of an LU-based inverse that used that pivot sequence: it
    grows with the sequence's own element growth, so it measures a kernel
    against what its pivot rule allows rather than against one rounding order.
    """
    A = np.asarray(A, dtype=np.float64)
    b, n, _ = A.shape
    Uf = np.take_along_axis(A, np.asarray(perm, dtype=np.int64)[:, :, None], axis=1).copy()
    L = np.zeros_like(Uf)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        for k in range(n):
            L[:, k, k] = 1.0
            m = Uf[:, k + 1:, k] / Uf[:, k:k + 1, k]
            L[:, k + 1:, k] = m
            Uf[:, k + 1:, :] -= m[:, :, None] * Uf[:, k:k + 1, :]
            Uf[:, k + 1:, k] = 0.0
        if X64 is None:
            X64 = np.linalg.inv(A)
        return (np.abs(L) @ np.abs(Uf) @ np.abs(X64)).sum(2).max(1)


def residual(A: np.ndarray, X: np.ndarray) -> np.ndarray:
    """Per matrix [||AX - I||_inf, max|AX - I|] in FP64."""
    A = np.ascontiguousarray(A, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.float32)
    b, n, _ = A.shape
    res = np.empty((b, 2), dtype=np.float64)
    lib().mi_or_batch_residual(A.reshape(-1), X.reshape(-1), b, n, res.reshape(-1))
    return res


def set_threads(t: int) -> None:
    lib().mi_or_set_num_threads(int(t))


def num_threads() -> int:
    return int(lib().mi_or_num_threads())


def ref_kernel_run(variant: str, A: np.ndarray):
    """Run a reference kernel ('parallel_pivot', 'serial_pivot', 'templated') on
    host threads.  Returns (output, pivots or None).  Pivots are exact; the
    pivoted variants' outputs are not (their comp_inv stores columns while other
    threads still read them, which only a lockstep warp tolerates)."""
    R = ref_lib()
    if R is None:
        raise RuntimeError("reference emulation not built (reference sources absent)")
    X = np.array(A, dtype=np.float32, copy=True, order="C")
    b, n, _ = X.shape
    piv = None if variant == "templated" else np.zeros((b, n), dtype=np.int32)
    fn = getattr(R, f"ref_emu_{variant}_run")
    rc = fn(X.reshape(-1), None if piv is None else piv.ctypes.data, b, n)
    if rc != 0:
        raise RuntimeError(f"reference emulation failed ({rc})")
    return X, piv
