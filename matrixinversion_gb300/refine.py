"""Precision study: FP32 inverses of conditioned 32 x 32 matrices, plain and
refined by Newton-Schulz steps on the tensor cores.

Matrices are A = Q1 diag(s) Q2^T with Q1, Q2 from QR of seeded Gaussian
matrices and singular values log-spaced from 1 down to 1/kappa, in buckets of
kappa (default 1e1, 1e3, 1e5, 1e6).  The reference inverse is FP64 (batched
LU in FP64 on the device, of the FP32 matrix as stored).  Error of one matrix
= max |X - X64| / max |X64|.

    python -m matrixinversion_gb300.refine --per-bucket 65536
"""
from __future__ import annotations

import argparse
import ctypes
import json
import sys

import numpy as np

from . import _lib

KAPPAS = (1e1, 1e3, 1e5, 1e6)
# The refined form's defaults.  An FP32 inverse of a 32 x 32 matrix can miss
# 1e-6 relative error already at condition numbers of a few (max-norm error
# about u * ||A||_1 ||X||_1), so every matrix whose estimate reaches 8 gets
# one float-float step; a second step follows where the first leaves an
# estimated error above 3e-7.
REFINE_FLAG = 8.0
REFINE_TOL = 3e-7


def _check_pair(A, X, max_n: int = 32):
    """A and X: contiguous CUDA float32 [batch, n, n] of one shape on one
    device (the kernels index both by the same batch position)."""
    import torch

    for name, t in (("A", A), ("X", X)):
        if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()):
            raise TypeError(f"{name} must be a contiguous CUDA float32 tensor")
    if A.shape != X.shape or A.device != X.device or A.dim() != 3 or A.shape[-1] != A.shape[-2] \
            or not 1 <= A.shape[-1] <= max_n:
        raise ValueError(f"A and X must both be [batch, n, n] with n <= {max_n}, on one device")


def _check_list(name, t, device, numel=None):
    import torch

    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.int32 and t.is_contiguous()
            and t.device == device and (numel is None or t.numel() == numel)):
        what = f" of {numel} entries" if numel is not None else ""
        raise TypeError(f"{name} must be a contiguous CUDA int32 tensor{what} on {device}")


def newton_schulz_(A, X, steps: int = 1, stream=None):
    """Refine X (in place) toward A^-1: X <- X + X (I - A X), `steps` times.
    A, X: contiguous CUDA float32 [batch, 32, 32]."""
    import torch

    for name, t in (("A", A), ("X", X)):
        if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()):
            raise TypeError(f"{name} must be a contiguous CUDA float32 tensor")
    if A.shape != X.shape or A.dim() != 3 or A.shape[-1] != 32 or A.shape[-2] != 32:
        raise ValueError("A and X must both be [batch, 32, 32]")
    st = (stream or torch.cuda.current_stream(A.device)).cuda_stream
    with torch.cuda.device(A.device):
        status = _lib.load().mi_newton_schulz_f32(ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(X.data_ptr()),
                                                  A.shape[0], 32, int(steps), ctypes.c_void_p(st))
    _lib.check(status)
    return X


def refine_fp64_(A, X, index, stream=None):
    """One FP64-residual refinement step for the matrices X[index] (in place).
    index: CUDA int32 tensor of batch indices."""
    import torch

    _check_pair(A, X)
    _check_list("index", index, A.device)
    n = A.shape[-1]
    st = (stream or torch.cuda.current_stream(A.device)).cuda_stream
    with torch.cuda.device(A.device):
        status = _lib.load().mi_refine_fp64_f32(ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(X.data_ptr()),
                                                ctypes.c_void_p(index.data_ptr()), index.numel(), A.shape[0], n,
                                                ctypes.c_void_p(st))
    _lib.check(status)
    return X


def _refine_step(prefix, A, X, index, stream, next_tol, next_out, max_n=32):
    import torch

    _check_pair(A, X)
    _check_list("index", index, A.device)
    n = A.shape[-1]
    if n > max_n:
        raise ValueError(f"{prefix} refinement takes n <= {max_n}")
    st = (stream or torch.cuda.current_stream(A.device)).cuda_stream
    lib = _lib.load()
    step = getattr(lib, f"mi_refine_{prefix}_f32")
    step_next = getattr(lib, f"mi_refine_{prefix}_next_f32")
    with torch.cuda.device(A.device):
        if next_tol is None:
            status = step(ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(X.data_ptr()),
                          ctypes.c_void_p(index.data_ptr()), index.numel(), A.shape[0], n, ctypes.c_void_p(st))
            _lib.check(status)
            return X
        if next_out is None:
            next_out = torch.empty_like(index)
        _check_list("next_out", next_out, A.device, index.numel())
        status = step_next(ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(X.data_ptr()),
                           ctypes.c_void_p(index.data_ptr()), index.numel(), A.shape[0], n, float(next_tol),
                           ctypes.c_void_p(next_out.data_ptr()), ctypes.c_void_p(st))
    _lib.check(status)
    return next_out


def refine_df_(A, X, index, stream=None, next_tol=None, next_out=None):
    """One refinement step with a float-float residual for the matrices
    X[index] (in place): the accuracy of the FP64 step at FP32-pipe speed.

    With next_tol set, also returns the list for a second step: entry t is
    index[t] where the error left after this step, estimated on the device as
    max|X R^2| / max|X| (X, R = I - A X before the step), exceeds next_tol,
    else -1.  next_out (CUDA int32, index.numel() entries) receives it and may
    be `index` itself."""
    return _refine_step("df", A, X, index, stream, next_tol, next_out)


def refine_tc_(A, X, index, stream=None, next_tol=None, next_out=None):
    """As refine_df_ for 32 x 32 matrices, with the residual formed exactly on
    the tensor cores (base-256 digits in bf16, exact FP32 group sums, float-
    float combination) and the correction X R from two-term bf16 splits; the
    second-step estimate is max|C R| / max|X| with C = X R the correction."""
    return _refine_step("tc", A, X, index, stream, next_tol, next_out)


def refine_tc_flagged_(A, X, flag_threshold: float = REFINE_FLAG, next_tol: float = REFINE_TOL, next_out=None,
                       stream=None):
    """The flag and the first tensor-core step in one pass (32 x 32 only):
    every matrix whose condition estimate ||A||_1 ||X||_1 is at least
    flag_threshold (or not finite) gets one refine_tc_ step, in place.
    Returns the full-length CUDA int32 list for a second step: b where the
    step leaves an estimated error above next_tol, else -1."""
    import torch

    _check_pair(A, X)
    batch, n = A.shape[0], A.shape[-1]
    if n != 32:
        raise ValueError("the fused flag-and-step pass takes n = 32")
    if next_out is None:
        next_out = torch.empty(batch, dtype=torch.int32, device=A.device)
    _check_list("next_out", next_out, A.device, batch)
    st = (stream or torch.cuda.current_stream(A.device)).cuda_stream
    with torch.cuda.device(A.device):
        status = _lib.load().mi_refine_tc_flagged_f32(ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(X.data_ptr()),
                                                      batch, n, float(flag_threshold), float(next_tol),
                                                      ctypes.c_void_p(next_out.data_ptr()), ctypes.c_void_p(st))
    _lib.check(status)
    return next_out


def flag_ill_conditioned(A, X, threshold: float = 1e4):
    """Indices (CUDA int32) of matrices whose estimate ||A||_1 ||X||_1 of the
    condition number is at least `threshold`: there an FP32 residual is no
    better than the FP32 inverse, and a higher-precision step is worth its
    cost."""
    import torch

    est = A.abs().sum(-2).amax(-1) * X.abs().sum(-2).amax(-1)
    est = torch.where(torch.isfinite(est), est, torch.full_like(est, float("inf")))
    return torch.nonzero(est >= threshold).squeeze(1).to(torch.int32).contiguous()


def flag_list(A, X, threshold: float = 1e4, out=None):
    """Full-length CUDA int32 list: b where ||A_b||_1 ||X_b||_1 >= threshold
    (or is not finite), else -1 -- computed on the device, no host round trip;
    refine_df_ / refine_fp64_ take it as it is."""
    import torch

    _check_pair(A, X)
    batch, n = A.shape[0], A.shape[-1]
    if out is None:
        out = torch.empty(batch, dtype=torch.int32, device=A.device)
    _check_list("out", out, A.device, batch)
    st = torch.cuda.current_stream(A.device).cuda_stream
    with torch.cuda.device(A.device):
        status = _lib.load().mi_flag_condition_f32(ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(X.data_ptr()),
                                                   batch, n, float(threshold), ctypes.c_void_p(out.data_ptr()),
                                                   ctypes.c_void_p(st))
    _lib.check(status)
    return out


def refined_inverse(A, flag_threshold: float = REFINE_FLAG, tol: float = REFINE_TOL, lists: bool = False,
                    step: str = "auto"):
    """The refined form of batched_inverse(A, "partial"): the FP32
    partial-pivoting inverse, one refinement step with a residual accurate
    beyond FP32 for every matrix whose condition estimate ||A||_1 ||X||_1 is
    at least flag_threshold, and a second step only where the first leaves an
    estimated error above tol.  step: "tc" (residual on the tensor cores,
    n = 32 only), "df" (float-float on the FP32 pipes, any n), or "auto" ("tc"
    at n = 32, else "df").  Flags and lists stay on the device (no host round
    trip).  Returns (X, perm, info), plus the first and second step lists if
    `lists`."""
    import matrixinversion_gb300 as mi

    if step == "auto":
        step = "tc" if A.shape[-1] == 32 else "df"
    if step not in ("tc", "df"):
        raise ValueError(f"unknown refinement step {step!r}")
    X, perm, info = mi.batched_inverse(A, "partial")
    first = flag_list(A, X, threshold=flag_threshold) if (lists or step == "df") else None
    if step == "tc":
        # flag and first step fused: one pass over A and X fewer
        ix = refine_tc_flagged_(A, X, flag_threshold, tol)
        refine_tc_(A, X, ix)
    else:
        ix = first.clone() if lists else first
        refine_df_(A, X, ix, next_tol=tol, next_out=ix)
        refine_df_(A, X, ix)
    return (X, perm, info, first, ix) if lists else (X, perm, info)


def conditioned(batch: int, kappa: float, n: int = 32, seed: int = 0, device="cuda"):
    """FP32 [batch, n, n] with 2-norm condition number ~kappa (as FP64)."""
    import torch

    g = torch.Generator(device=device).manual_seed(seed)
    G1 = torch.randn(batch, n, n, generator=g, device=device, dtype=torch.float64)
    G2 = torch.randn(batch, n, n, generator=g, device=device, dtype=torch.float64)
    Q1, _ = torch.linalg.qr(G1)
    Q2, _ = torch.linalg.qr(G2)
    s = torch.logspace(0.0, -float(np.log10(kappa)), n, device=device, dtype=torch.float64)
    A = (Q1 * s) @ Q2.transpose(1, 2)
    return A.float().contiguous()


def rel_error(X, X64):
    """Per matrix: max |X - X64| / max |X64|."""
    d = (X.double() - X64).abs().amax((-1, -2))
    return d / X64.abs().amax((-1, -2))


def study(per_bucket: int = 65536, kappas=KAPPAS, steps=(1, 2), seed: int = 0, timing_iters: int = 5):
    import torch

    import matrixinversion_gb300 as mi

    out = []
    for bi, kappa in enumerate(kappas):
        A = conditioned(per_bucket, kappa, seed=seed + bi)
        X64 = torch.linalg.inv(A.double())
        X0, _, info = mi.batched_inverse(A, "partial")
        row = {"kappa": kappa, "matrices": per_bucket}
        e0 = rel_error(X0, X64)
        row["plain"] = {"median": float(e0.median()), "max": float(e0.max())}
        for k in steps:
            X = X0.clone()
            newton_schulz_(A, X, steps=k)
            e = rel_error(X, X64)
            row[f"ns{k}"] = {"median": float(e.median()), "max": float(e.max())}
        # NS step, then the FP64 step for the flagged matrices only
        X = X0.clone()
        newton_schulz_(A, X, steps=1)
        idx = flag_ill_conditioned(A, X)
        refine_fp64_(A, X, idx)
        e = rel_error(X, X64)
        row["ns1_fp64_flagged"] = {"median": float(e.median()), "max": float(e.max()), "flagged": int(idx.numel())}
        # float-float and tensor-core residual steps on the flagged matrices,
        # from the plain inverse
        for name, fn in (("df", refine_df_), ("tc", refine_tc_)):
            for nsteps in (1, 2):
                X = X0.clone()
                idx = flag_ill_conditioned(A, X)
                for _ in range(nsteps):
                    fn(A, X, idx)
                e = rel_error(X, X64)
                row[f"{name}{nsteps}_flagged"] = {"median": float(e.median()), "max": float(e.max()),
                                                  "flagged": int(idx.numel())}
        # the refined form (refined_inverse) with either step, timed end to end
        for label, step in (("refined", "tc"), ("refined_df", "df")):
            _, _, _, first, second = refined_inverse(A, lists=True, step=step)
            torch.cuda.synchronize()
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            ev[0].record()
            Xref, _, _ = refined_inverse(A, step=step)
            ev[1].record()
            torch.cuda.synchronize()
            ms = ev[0].elapsed_time(ev[1])
            e = rel_error(Xref, X64)
            row[label] = {"median": float(e.median()), "max": float(e.max()), "flagged": int((first >= 0).sum()),
                          "second_step": int((second >= 0).sum()), "ms": ms,
                          "matrices_per_s": per_bucket / ms * 1e3}
        # the reference pivot rule's inverse, plain and after one NS step
        Xr, _, _ = mi.batched_inverse(A, "reference")
        e = rel_error(Xr, X64)
        row["reference_plain"] = {"median": float(e.median()), "max": float(e.max())}
        newton_schulz_(A, Xr, steps=1)
        e = rel_error(Xr, X64)
        row["reference_ns1"] = {"median": float(e.median()), "max": float(e.max())}
        out.append(row)
    # throughput on one bucket's batch (kernel time, CUDA events, in place on a copy)
    A = conditioned(per_bucket, kappas[0], seed=seed)
    X0, _, _ = mi.batched_inverse(A, "partial")
    all_idx = torch.arange(per_bucket, dtype=torch.int32, device=A.device)
    timing = {}
    for label, fn in (("inverse_partial", lambda X: mi.batched_inverse_(X, "partial")),
                      ("inverse_reference", lambda X: mi.batched_inverse_(X, "reference")),
                      ("ns1", lambda X: newton_schulz_(A, X, 1)), ("ns2", lambda X: newton_schulz_(A, X, 2)),
                      ("fp64_all", lambda X: refine_fp64_(A, X, all_idx)),
                      ("df_all", lambda X: refine_df_(A, X, all_idx)),
                      ("df_all_with_estimate", lambda X: refine_df_(A, X, all_idx, next_tol=REFINE_TOL)),
                      ("tc_all", lambda X: refine_tc_(A, X, all_idx)),
                      ("tc_all_with_estimate", lambda X: refine_tc_(A, X, all_idx, next_tol=REFINE_TOL))):
        bufs = [(A if label.startswith("inverse") else X0).clone() for _ in range(timing_iters + 2)]
        for b in bufs[:2]:
            fn(b)
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record()
        for b in bufs[2:]:
            fn(b)
        ev[1].record()
        torch.cuda.synchronize()
        ms = ev[0].elapsed_time(ev[1]) / timing_iters
        timing[label] = {"ms": ms, "matrices_per_s": per_bucket / ms * 1e3}
    out.append({"timing": timing, "matrices": per_bucket})
    return out


def bench_ns(count: int = 262144, steps: int = 1, iters: int = 5, seed: int = 0):
    """Kernel time of `steps` Newton-Schulz steps on `count` matrices (no
    library linear algebra involved: uniform inputs with +32 on the diagonal,
    the starting inverse from the no-pivot kernel).  For profiling."""
    import torch

    import matrixinversion_gb300 as mi

    g = torch.Generator(device="cuda").manual_seed(seed)
    A = torch.rand(count, 32, 32, generator=g, device="cuda") * 2 - 1 + 32 * torch.eye(32, device="cuda")
    X0, _, _ = mi.batched_inverse(A, "none")
    bufs = [X0.clone() for _ in range(iters + 2)]
    for b in bufs[:2]:
        newton_schulz_(A, b, steps)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    torch.cuda._sleep(200_000)
    ev[0].record()
    for b in bufs[2:]:
        newton_schulz_(A, b, steps)
    ev[1].record()
    torch.cuda.synchronize()
    ms = ev[0].elapsed_time(ev[1]) / iters
    return {"count": count, "steps": steps, "ms": ms, "matrices_per_s": count / ms * 1e3,
            "GBs": count * 12288 * steps / ms / 1e6}


def bench_refined(count: int = 262144, iters: int = 5, seed: int = 0):
    """Throughput of the plain partial-pivoting inverse and of the refined
    form with either step on `count` uniform [-1, 1) 32 x 32 matrices (every
    one flagged: their condition estimates are far above 8), CUDA events on
    the current stream, fresh inputs per iteration (each batch 4 MB x count /
    1024, above L2 at the default size)."""
    import torch

    import matrixinversion_gb300 as mi

    g = torch.Generator(device="cuda").manual_seed(seed)
    As = [torch.rand(count, 32, 32, generator=g, device="cuda") * 2 - 1 for _ in range(2)]
    out = {"count": count}
    for label, fn in (("plain_partial", lambda A: mi.batched_inverse(A, "partial")),
                      ("refined_tc", lambda A: refined_inverse(A, step="tc")),
                      ("refined_df", lambda A: refined_inverse(A, step="df"))):
        for i in range(2):
            fn(As[i % 2])
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record()
        for i in range(iters):
            fn(As[i % 2])
        ev[1].record()
        torch.cuda.synchronize()
        ms = ev[0].elapsed_time(ev[1]) / iters
        out[label] = {"ms": ms, "matrices_per_s": count / ms * 1e3}
    _, _, _, first, second = refined_inverse(As[0], lists=True)
    out["flagged"] = int((first >= 0).sum())
    out["second_step"] = int((second >= 0).sum())
    out["tc_vs_plain"] = out["plain_partial"]["ms"] / out["refined_tc"]["ms"]
    out["df_vs_plain"] = out["plain_partial"]["ms"] / out["refined_df"]["ms"]
    return out


def config4(per_bucket: int = 65536, kappas=KAPPAS, seed: int = 0, iters: int = 5):
    """The precision configuration as one batch: the kappa buckets
    (per_bucket matrices each, 262,144 in all by default) concatenated into a
    single [batch, 32, 32] tensor, inverted plain (partial pivoting) and in the
    refined form with either step, each as one call over the whole batch.
    Per bucket: median and max relative error against the FP64 inverse; for
    the batch: kernel-path time (CUDA events, mean of `iters` calls after one
    warm-up) and matrices/s, and the refined form's rate as a fraction of the
    plain kernel's at the same batch."""
    import torch

    import matrixinversion_gb300 as mi

    A = torch.cat([conditioned(per_bucket, k, seed=seed + i) for i, k in enumerate(kappas)])
    X64 = torch.cat([torch.linalg.inv(A[i * per_bucket:(i + 1) * per_bucket].double())
                     for i in range(len(kappas))])
    batch = A.shape[0]
    out = {"batch": batch, "per_bucket": per_bucket, "buckets": []}
    runs = {"plain_partial": lambda: mi.batched_inverse(A, "partial")[0],
            "refined_tc": lambda: refined_inverse(A, step="tc")[0],
            "refined_df": lambda: refined_inverse(A, step="df")[0]}
    errs, timing = {}, {}
    for label, fn in runs.items():
        X = fn()
        torch.cuda.synchronize()
        errs[label] = rel_error(X, X64)
        del X
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record()
        for _ in range(iters):
            fn()
        ev[1].record()
        torch.cuda.synchronize()
        ms = ev[0].elapsed_time(ev[1]) / iters
        timing[label] = {"ms": ms, "matrices_per_s": batch / ms * 1e3}
    _, _, _, first, second = refined_inverse(A, lists=True)
    for i, k in enumerate(kappas):
        sl = slice(i * per_bucket, (i + 1) * per_bucket)
        row = {"kappa": k}
        for label, e in errs.items():
            row[label] = {"median": float(e[sl].median()), "max": float(e[sl].max())}
        row["flagged"] = int((first[sl] >= 0).sum())
        row["second_step"] = int((second[sl] >= 0).sum())
        out["buckets"].append(row)
    out["timing"] = timing
    out["refined_tc_vs_plain"] = timing["plain_partial"]["ms"] / timing["refined_tc"]["ms"]
    out["refined_df_vs_plain"] = timing["plain_partial"]["ms"] / timing["refined_df"]["ms"]
    return out


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--per-bucket", type=int, default=65536)
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--out", default=None)
    p.add_argument("--ns-only", type=int, default=0, help="only time the Newton-Schulz kernel on this many matrices")
    p.add_argument("--refined-only", type=int, default=0,
                   help="only time the refined form against the plain inverse on this many matrices")
    p.add_argument("--config4", action="store_true",
                   help="the kappa buckets as one batch: errors per bucket and the refined form's rate")
    a = p.parse_args(argv)
    if a.config4:
        r = config4(a.per_bucket, seed=a.seed)
        print(json.dumps(r), flush=True)
        if a.out:
            with open(a.out, "w") as f:
                json.dump(r, f, indent=1)
        return
    if a.refined_only:
        print(json.dumps(bench_refined(a.refined_only, seed=a.seed)), flush=True)
        return
    if a.ns_only:
        for k in (1, 2):
            print(json.dumps(bench_ns(a.ns_only, k, seed=a.seed)), flush=True)
        return
    rows = study(a.per_bucket, seed=a.seed)
    for r in rows:
        print(json.dumps(r), flush=True)
    if a.out:
        with open(a.out, "w") as f:
            json.dump(rows, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1:])
