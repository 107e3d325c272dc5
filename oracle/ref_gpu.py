"""Test and measurement infrastructure (never the product): the reference's
own GPU kernels, batched_lu_subwarp of parallel_pivot (luBatchedInplace.cuh:
127-198, the parallel-argmax rule), serial_pivot (:104-170, the serial rule)
and templated (:78-121, no pivoting), run on this GPU beside this project's
kernels.

The kernels are compiled unchanged from the reference tree into
oracle/_ref/ref_<variant>_sm103a.cubin by `make -C oracle REF_ROOT=... ref`
(instantiations in oracle/ref_gpu/ref_gpu_inst.cu); this module loads a cubin
through the CUDA driver API (ctypes on libcuda) into the context PyTorch uses
and launches the kernel exactly as the variant's driver does
(luBatchedInplace.cu:4-11 and its launch line): one block per NUMTHREADS / n
matrices, n threads per matrix, the variant's dynamic shared memory per
matrix (n^2 + 3n floats with the parallel argmax, n^2 + n with the serial
one, n^2 without pivoting), the batch inverted in place.

    python -m oracle.ref_gpu --n 4,8,16,24,31,32 --modes reference,reference_serial,none

times each reference kernel and mi.batched_inverse_(A, mode) on the same
seeded batches of 1,000,000 matrices (+n on the diagonal without pivoting)
and compares their residuals.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# this project's pivot mode -> (reference variant, shared floats per matrix beyond n^2, as a multiple of n)
VARIANTS = {"reference": ("parallel_pivot", 3), "reference_serial": ("serial_pivot", 1), "none": ("templated", 0)}


def cubin(mode: str = "reference") -> str:
    return os.path.join(HERE, "_ref", f"ref_{VARIANTS[mode][0]}_sm103a.cubin")


CUBIN = cubin("reference")

# (n, numMatrices) -> matrices per block, as instantiated in ref_gpu_inst.cu
CONFIGS = {(4, 1000000): 8, (8, 1000000): 4, (16, 1000000): 2, (24, 1000000): 1, (31, 1000000): 1,
           (32, 1000000): 1, (8, 4096): 4, (16, 4096): 2, (32, 4096): 1, (32, 1000): 1}


def available(mode: str = "reference") -> bool:
    return os.path.exists(cubin(mode))


def kernel_name(n: int, count: int) -> bytes:
    mpb = CONFIGS[(n, count)]
    return f"_Z18batched_lu_subwarpIfLi{n}ELi{n}ELi{mpb}ELi{count}EEvPT_".encode()


class RefKernels:
    """The cubin of one reference variant (by this project's name of its
    pivot mode) loaded into the current device's primary context."""

    def __init__(self, mode: str = "reference"):
        import torch

        self.mode = mode
        self.path = cubin(mode)
        if not os.path.exists(self.path):
            raise FileNotFoundError(f"{self.path} missing: build it with make -C oracle REF_ROOT=<reference root> ref")
        torch.cuda.init()
        torch.cuda.current_device()
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.cu.cuGetErrorString.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
        ctx = ctypes.c_void_p()
        self._check(self.cu.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            dev, pctx = ctypes.c_int(), ctypes.c_void_p()
            self._check(self.cu.cuDeviceGet(ctypes.byref(dev), torch.cuda.current_device()), "cuDeviceGet")
            self._check(self.cu.cuDevicePrimaryCtxRetain(ctypes.byref(pctx), dev), "cuDevicePrimaryCtxRetain")
            self._check(self.cu.cuCtxSetCurrent(pctx), "cuCtxSetCurrent")
        self.mod = ctypes.c_void_p()
        self._check(self.cu.cuModuleLoad(ctypes.byref(self.mod), self.path.encode()), "cuModuleLoad")
        self.fns = {}

    def _check(self, rc, what):
        if rc != 0:
            s = ctypes.c_char_p()
            self.cu.cuGetErrorString(rc, ctypes.byref(s))
            raise RuntimeError(f"{what}: CUDA driver error {rc} ({(s.value or b'').decode()})")

    def _fn(self, n, count):
        key = (n, count)
        if key not in self.fns:
            f = ctypes.c_void_p()
            self._check(self.cu.cuModuleGetFunction(ctypes.byref(f), self.mod, kernel_name(n, count)),
                        "cuModuleGetFunction")
            self.fns[key] = f
        return self.fns[key]

    def invert_(self, A, stream=None) -> None:
        """In-place inverse of A ([count, n, n] float32, contiguous, CUDA) by
        the reference kernel instantiated for exactly this (n, count)."""
        import torch

        count, n = int(A.shape[0]), int(A.shape[-1])
        if (n, count) not in CONFIGS:
            raise ValueError(f"no reference instantiation for n={n}, count={count}: {sorted(CONFIGS)}")
        if not (A.is_cuda and A.dtype == torch.float32 and A.is_contiguous() and A.numel() == count * n * n):
            raise ValueError("A must be a contiguous CUDA float32 tensor of count x n x n")
        mpb = CONFIGS[(n, count)]
        assert count % mpb == 0, "whole blocks only"
        grid, block = count // mpb, mpb * n
        smem = mpb * (n * n + VARIANTS[self.mode][1] * n) * 4
        ptr = ctypes.c_uint64(A.data_ptr())
        params = (ctypes.c_void_p * 1)(ctypes.cast(ctypes.pointer(ptr), ctypes.c_void_p))
        st = (stream or torch.cuda.current_stream()).cuda_stream
        self._check(self.cu.cuLaunchKernel(self._fn(n, count), grid, 1, 1, block, 1, 1, smem, ctypes.c_void_p(st),
                                           params, None), "cuLaunchKernel")


def residuals(A, X, sample: int = 2048):
    """||A X - I||_inf per matrix (FP64) on the first `sample` matrices."""
    import torch

    a, x = A[:sample].double(), X[:sample].double()
    eye = torch.eye(a.shape[-1], dtype=torch.float64, device=a.device)
    return (a @ x - eye).abs().sum(-1).amax(-1)


def compare(ns=(4, 8, 16, 24, 31, 32), count: int = 1000000, runs: int = 5, seed: int = 0, mode: str = "reference"):
    """Same-GPU timing of a reference kernel and this project's kernel in the
    same pivot mode on the same seeded uniform [-1, 1) batches (+n on the
    diagonal without pivoting); CUDA events around each launch only, each
    launch on a fresh copy."""
    import numpy as np
    import torch

    import matrixinversion_gb300 as mi

    ref = RefKernels(mode)
    out = []
    for n in ns:
        g = torch.Generator(device="cuda").manual_seed(seed + n)
        src = torch.rand(count, n, n, generator=g, device="cuda") * 2 - 1
        if mode == "none":
            src += n * torch.eye(n, device="cuda")

        def timed(fn):
            ts = []
            for i in range(runs + 2):
                A = src.clone()
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                fn(A)
                e1.record()
                torch.cuda.synchronize()
                if i >= 2:
                    ts.append(e0.elapsed_time(e1))
            return float(np.median(ts)), A

        t_ref, X_ref = timed(ref.invert_)
        t_mi, X_mi = timed(lambda A: mi.batched_inverse_(A, mode))
        r_ref, r_mi = residuals(src, X_ref), residuals(src, X_mi)
        rel = ((X_ref[:2048] - X_mi[:2048]).abs().amax((1, 2)) / X_ref[:2048].abs().amax((1, 2))).cpu().numpy()
        bytes_alg = count * (8 * n * n + 4 * n + 4)
        row = {"mode": mode, "n": n, "count": count, "reference_kernel_ms": t_ref, "mi_ms": t_mi, "speedup": t_ref / t_mi,
               "reference_GBs": bytes_alg / t_ref / 1e6, "mi_GBs": bytes_alg / t_mi / 1e6,
               "resid_median_reference": float(r_ref.median()), "resid_median_mi": float(r_mi.median()),
               "resid_p99_reference": float(r_ref.quantile(0.99)), "resid_p99_mi": float(r_mi.quantile(0.99)),
               "rel_diff_median": float(np.median(rel)), "rel_diff_max": float(rel.max())}
        out.append(row)
        del src, X_ref, X_mi
        torch.cuda.empty_cache()
    return out


def main(argv=None):
    import argparse
    import json

    p = argparse.ArgumentParser()
    p.add_argument("--n", default="4,8,16,24,31,32")
    p.add_argument("--modes", default="reference")
    p.add_argument("--count", type=int, default=1000000)
    p.add_argument("--runs", type=int, default=5)
    a = p.parse_args(argv)
    for mode in a.modes.split(","):
        for row in compare(tuple(int(x) for x in a.n.split(",")), count=a.count, runs=a.runs, mode=mode):
            print(json.dumps(row), flush=True)


if __name__ == "__main__":
    import sys

    main(sys.argv[1:])
