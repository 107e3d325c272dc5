"""Size sweep in the shape of the reference's run.py (parallel_pivot/run.py:169-251).

For every matrix size n and batch size N it times the kernel over `runs`
launches (each on a fresh copy of the seeded batch), records runtimes, mean,
variance and standard deviation under the key ``m{n}_n{N}_t{T}`` like the
reference, and adds what the reference does not report: matrices/s, the
fraction of the measured HBM roofline, cuBLAS getrfBatched + getriBatched on
the same data, and ||AX - I||_inf statistics (FP64, on a sample) for both.

The reference's knobs are honoured as environment variables:
MATRIXSIZE (one n), NUMMATRICES (one batch size), NUMTHREADS (threads per
block; 0 = default).

    python -m matrixinversion_gb300.sweep --n 2-32 --batch 1000000 --pivot reference --cublas
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np


def parse_range(text: str) -> list[int]:
    out: list[int] = []
    for part in text.split(","):
        if "-" in part:
            a, b = part.split("-")
            out.extend(range(int(a), int(b) + 1))
        elif part:
            out.append(int(part))
    return out


def hbm_peak_gbs() -> float:
    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    try:
        with open(os.path.join(here, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except Exception:
        return 6800.0


def residual_stats(A, X, sample: int, seed: int = 1):
    """||A X - I||_inf (max row sum) in FP64 on a random sample of matrices."""
    import torch

    b = A.shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    idx = torch.randperm(b, generator=g)[: min(sample, b)].to(A.device)
    a = A[idx].double()
    x = X[idx].double()
    eye = torch.eye(A.shape[-1], dtype=torch.float64, device=A.device)
    r = (a @ x - eye).abs().sum(-1).amax(-1)
    r = torch.where(torch.isfinite(r), r, torch.full_like(r, float("inf")))
    q = torch.quantile(r.float().cpu(), torch.tensor([0.5, 0.99])).tolist()
    return {"median": q[0], "p99": q[1], "max": float(r.max().item()),
            "fail_1e-3": float(((a @ x - eye).abs().amax((-1, -2)) >= 1e-3).float().mean().item())}


_HOST: dict = {}


def run_case(n: int, batch: int, pivot: str, runs: int, threads: int, with_cublas: bool, sample: int, seed: int):
    import torch

    import matrixinversion_gb300 as mi
    from matrixinversion_gb300 import data

    dev = torch.device("cuda")
    key = (seed, batch, n)
    if key not in _HOST:
        _HOST.clear()
        _HOST[key] = data.uniform(seed, batch, n)
    host = _HOST[key].copy() if pivot == "none" else _HOST[key]
    if pivot == "none":
        host += np.float32(n) * np.eye(n, dtype=np.float32)
    src = torch.from_numpy(host).to(dev)
    perm = torch.empty((batch, n), dtype=torch.int32, device=dev)
    info = torch.empty((batch,), dtype=torch.int32, device=dev)
    times = []
    X = None
    for r in range(runs + 1):
        w = src.clone()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        # keep the device busy while the host issues the launch, so the event
        # pair brackets device time only (the reference times from C++)
        torch.cuda._sleep(200_000)
        e0.record()
        mi.batched_inverse_(w, pivot, perm=perm, info=info, threads_per_block=threads)
        e1.record()
        torch.cuda.synchronize()
        if r > 0:                      # the first launch is a warm-up
            times.append(e0.elapsed_time(e1))
        X = w
    avg = float(np.mean(times))
    bytes_per = 8 * n * n + 4 * n + 4
    res = {
        "matrix_size": n, "num_matrices": batch, "num_threads": threads, "pivot": pivot,
        "runtimes": times, "runtime_avg": avg, "variance": float(np.var(times)), "std_dev": float(np.std(times)),
        "matrices_per_s": batch / (avg / 1e3),
        "hbm_roofline_frac": batch * bytes_per / (avg / 1e3) / 1e9 / hbm_peak_gbs(),
        "residual": residual_stats(src, X, sample),
        "singular": int((info != 0).sum().item()),
        # the kernel form that ran; NUMTHREADS reaches only the lane-group form
        "launch": mi.query_launch(n, pivot, batch, threads),
    }
    del X, w
    if with_cublas:
        from matrixinversion_gb300 import cublas_ref

        C = torch.empty_like(src)
        ctimes, split = [], None
        for r in range(min(runs, 3) + 1):
            W = src.clone()
            torch.cuda.synchronize()
            (Ci, _, _), (t1, t2) = cublas_ref.inverse(W, timed=True)
            if r > 0:
                ctimes.append(t1 + t2)
                split = (t1, t2)
            C = Ci
        cavg = float(np.mean(ctimes))
        res["cublas"] = {"runtime_avg": cavg, "getrf_ms": split[0], "getri_ms": split[1],
                         "matrices_per_s": batch / (cavg / 1e3), "speedup": cavg / avg,
                         "residual": residual_stats(src, C, sample)}
        del C
    torch.cuda.empty_cache()
    return res


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--n", default=os.environ.get("MATRIXSIZE", "2-32"))
    p.add_argument("--batch", default=os.environ.get("NUMMATRICES", "1000000"))
    p.add_argument("--threads", type=int, default=int(os.environ.get("NUMTHREADS", "0")))
    p.add_argument("--pivot", default="reference")
    p.add_argument("--runs", type=int, default=10)
    p.add_argument("--cublas", action="store_true")
    p.add_argument("--sample", type=int, default=4096)
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--out", default=None)
    args = p.parse_args(argv)

    results = {}
    for batch in parse_range(args.batch):
        for n in parse_range(args.n):
            for pivot in args.pivot.split(","):
                key = f"m{n}_n{batch}_t{args.threads}" + ("" if pivot == "reference" else f"_{pivot}")
                results[key] = run_case(n, batch, pivot, args.runs, args.threads, args.cublas, args.sample,
                                        args.seed)
                r = results[key]
                line = {"key": key, "ms": round(r["runtime_avg"], 4), "mps": r["matrices_per_s"],
                        "roofline": round(r["hbm_roofline_frac"], 4), "res_med": r["residual"]["median"],
                        "res_p99": r["residual"]["p99"]}
                if "cublas" in r:
                    line.update({"cublas_ms": round(r["cublas"]["runtime_avg"], 4),
                                 "speedup": round(r["cublas"]["speedup"], 2),
                                 "cublas_res_med": r["cublas"]["residual"]["median"]})
                print(json.dumps(line), flush=True)
                if args.out:
                    with open(args.out, "w") as f:
                        json.dump(results, f, indent=1)
    return results


if __name__ == "__main__":
    main(sys.argv[1:])
