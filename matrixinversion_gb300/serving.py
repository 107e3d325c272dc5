"""Serving loop: a stream of inversion requests, coalesced into device batches.

A request holds k matrices of one size n (partial pivoting by default).
Requests arrive (Poisson, in real time) into a pinned host ring in arrival
order -- the way a network receive buffer fills.  The loop itself is native
code (`mi_serve_run` in the C ABI, csrc/mi_serve.cu); this module builds the
trace and the buffers and reads the results:

* the device pool is the HBM budget, carved once at start-up (no allocation
  on the serving path); an arrived request is admitted, first come first
  served, as soon as a free extent of the pool holds it (first fit, extents
  merged on release), and its host-to-device copy goes out at once;
* while fewer than two batches compute, every admitted request not yet
  computed goes into one launch: one descriptor call over the pool (GPU
  bucketing by size, one persistent launch per size present), or one
  contiguous call for a batch of a single request;
* each request's results return to the output ring with an event of its own;
  when the loop sees it, the request has completed and its extent is free.

With `resident=True` the requests' matrices already sit in HBM (produced by
an upstream device stage, in a device ring that counts against the budget):
batches are inverted in place, with no copies, a request completes with its
batch's kernels, and `offline()` gives the plain batched kernel's rate on the
same matrices for comparison.

The baseline ("per_request") runs the same loop with one request per launch.
Both paths run the same kernels on the same data, so results are equal bit
for bit (tested).

    python -m matrixinversion_gb300.serving --rates 2000,8000,32000 --requests 2000
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import sys
import time
from dataclasses import dataclass, field

import numpy as np

SIZES = (4, 8, 12, 16, 20, 24, 28, 32)
PIVOT_PARTIAL = 3


def nvtx_ranges():
    """(push, pop) of NVTX host ranges, so a timeline profiler shows each
    serving run; no-ops where torch was built without NVTX."""
    try:
        import torch.cuda.nvtx as nv

        nv.range_push("mi_serving")
        nv.range_pop()
        return nv.range_push, nv.range_pop
    except Exception:
        return (lambda msg: None), (lambda: None)


@dataclass
class Trace:
    """Requests in arrival order: arrival time (s), matrices k, size n, and
    the request's first float in the ring (16-byte aligned)."""

    arrival: np.ndarray
    k: np.ndarray
    n: np.ndarray
    offset: np.ndarray = field(default=None)

    @property
    def floats(self) -> np.ndarray:
        return self.k.astype(np.int64) * self.n.astype(np.int64) ** 2

    @property
    def total_floats(self) -> int:
        return int(self.offset[-1] + self.floats[-1]) if len(self.k) else 0


def make_trace(num_requests: int, rate: float, seed: int = 0, sizes=SIZES, kmax: int = 4096) -> Trace:
    """Poisson arrivals at `rate` requests/s; k log-uniform in [1, kmax];
    n uniform over `sizes`."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=num_requests)
    arrival = np.cumsum(gaps) - gaps[0]
    k = np.floor(np.exp(rng.uniform(0.0, math.log(kmax + 1), size=num_requests))).astype(np.int64)
    k = np.clip(k, 1, kmax)
    n = np.asarray(sizes, dtype=np.int64)[rng.integers(0, len(sizes), size=num_requests)]
    t = Trace(arrival=arrival, k=k, n=n)
    fl = t.floats
    sizes4 = (fl + 3) // 4 * 4
    t.offset = np.concatenate([[0], np.cumsum(sizes4)[:-1]]).astype(np.int64)
    return t


def retime(trace: Trace, rate: float, seed: int = 0) -> Trace:
    """The same requests (and ring layout) with Poisson arrivals at `rate`."""
    rng = np.random.default_rng(seed + 7)
    gaps = rng.exponential(1.0 / rate, size=len(trace.k))
    return Trace(arrival=np.cumsum(gaps) - gaps[0], k=trace.k, n=trace.n, offset=trace.offset)


class CudaServer:
    """The device side: pinned rings, the pool (or the resident device ring),
    the scratch of the native loop, and the descriptor tables of the trace for
    the offline comparison."""

    def __init__(self, trace: Trace, hbm_budget_bytes: int = 16 << 30, device=None, pivot: int = PIVOT_PARTIAL,
                 seed: int = 0, resident: bool = False, max_batch: int | None = None):
        import torch

        from . import _lib

        self.torch = torch
        self.L = _lib.load()
        self.check = _lib.check
        self.dev = torch.device(device or "cuda")
        self.trace = trace
        self.pivot = pivot
        total = trace.total_floats
        largest = int(((trace.floats + 3) // 4 * 4).max()) if len(trace.k) else 0
        self.resident = resident
        if resident:
            # the upstream stage's device ring holds the requests: it is the
            # server's memory for them and must fit the budget
            if 4 * total > hbm_budget_bytes:
                raise ValueError("the resident request ring does not fit the HBM budget")
            self.pool_floats = 0
            self.pool = None
        else:
            # the pool: the budget, or less when the whole trace needs less
            self.pool_floats = int(min(hbm_budget_bytes // 4, (total + 3) // 4 * 4))
            if largest > self.pool_floats:
                raise ValueError("the largest request does not fit the HBM budget")
            self.pool = torch.empty(self.pool_floats, dtype=torch.float32, device=self.dev)
        # host rings (pinned): requests in arrival order, uniform [-1, 1)
        g = torch.Generator(device=self.dev).manual_seed(seed)
        src = torch.empty(total, dtype=torch.float32, device=self.dev)
        chunk = 1 << 28
        for a in range(0, total, chunk):
            b = min(total, a + chunk)
            src[a:b] = torch.rand(b - a, generator=g, device=self.dev) * 2 - 1
        self.ring_in = torch.empty(total, dtype=torch.float32, pin_memory=True)
        self.ring_in.copy_(src)
        self.ring_out = torch.empty(total, dtype=torch.float32, pin_memory=True)
        if resident:
            self.ring_dev = src                       # inverted in place, restored before each run
            self.pristine = src.clone()
        del src
        # most matrices in one coalesced launch: with host copies a batch waits
        # for all its inputs, so moderate batches keep latency down; resident
        # batches have no copies to wait for and amortise better when large
        if max_batch is None:
            max_batch = (1 << 20) if resident else (1 << 16)
        self.max_batch = int(max(int(trace.k.max()) if len(trace.k) else 1, min(int(trace.k.sum()), max_batch)))
        self.scratch = torch.empty(int(self.L.mi_serve_scratch_bytes(self.max_batch)), dtype=torch.uint8,
                                   device=self.dev)
        # descriptor tables of every matrix of the trace, in ring order (offline comparison)
        k, n, off = trace.k, trace.n, trace.offset
        req_of = np.repeat(np.arange(len(k)), k)
        first = np.concatenate([[0], np.cumsum(k)[:-1]])
        local = np.arange(int(k.sum())) - np.repeat(first, k)
        mat_off = off[req_of] + local * (n[req_of] ** 2)
        self.d_off = torch.from_numpy(mat_off.astype(np.int64)).to(self.dev)
        self.d_n = torch.from_numpy(n[req_of].astype(np.int32)).to(self.dev)
        self.d_flag = torch.full((int(k.sum()),), pivot, dtype=torch.int32, device=self.dev)
        self.d_info = torch.zeros(int(k.sum()), dtype=torch.int32, device=self.dev)
        self.ws = torch.empty(max(int(self.L.mi_descr_workspace_bytes(int(k.sum()))), 256), dtype=torch.uint8,
                              device=self.dev)
        self.s_cmp = torch.cuda.Stream(self.dev)
        self.n_mask = 0
        for v in np.unique(n):
            self.n_mask |= 1 << (int(v) - 1)
        self.last_stats = None

    def run(self, trace: Trace | None = None, coalesce: bool = True):
        """Serve `trace` in real time through the native loop; returns
        per-request latencies (s) and the wall time from the first arrival to
        the last completion."""
        torch = self.torch
        t = trace or self.trace
        assert np.array_equal(t.offset, self.trace.offset)
        nreq = len(t.k)
        arrival = np.ascontiguousarray(t.arrival, dtype=np.float64)
        kk = np.ascontiguousarray(t.k, dtype=np.int64)
        nn = np.ascontiguousarray(t.n, dtype=np.int32)
        off = np.ascontiguousarray(t.offset, dtype=np.int64)
        lat = np.empty(nreq, dtype=np.float64)
        wall = ctypes.c_double(0.0)
        stats = np.zeros(2, dtype=np.int64)
        if self.resident:
            self.ring_dev.copy_(self.pristine)
        torch.cuda.synchronize(self.dev)
        push, pop = nvtx_ranges()
        push(f"mi_serve_run {nreq} requests")
        p = lambda a: ctypes.c_void_p(a.ctypes.data)
        with torch.cuda.device(self.dev):
            status = self.L.mi_serve_run(
                nreq, p(arrival), p(kk), p(nn), p(off), ctypes.c_void_p(self.ring_in.data_ptr()),
                ctypes.c_void_p(self.ring_out.data_ptr()),
                ctypes.c_void_p(self.ring_dev.data_ptr() if self.resident else 0),
                ctypes.c_void_p(self.pool.data_ptr() if self.pool is not None else 0), self.pool_floats,
                ctypes.c_void_p(self.scratch.data_ptr()), self.scratch.numel(), self.max_batch, self.pivot,
                1 if coalesce else 0, p(lat), ctypes.byref(wall), p(stats))
        pop()
        self.check(status)
        self.last_stats = {"batches": int(stats[0]), "peak_pool_bytes": int(stats[1]) * 4}
        return lat, float(wall.value)

    def results(self, r: int):
        """Output matrices of request r (host copy of the output ring)."""
        t = self.trace
        o, kk, nn = int(t.offset[r]), int(t.k[r]), int(t.n[r])
        if self.resident:
            return self.ring_dev[o: o + kk * nn * nn].cpu().numpy().reshape(kk, nn, nn)
        return self.ring_out[o: o + kk * nn * nn].numpy().reshape(kk, nn, nn)

    def offline(self, iters: int = 5) -> float:
        """matrices/s of one descriptor call over the whole trace, resident in
        HBM (the plain batched kernel on the same matrices, no serving)."""
        torch = self.torch
        t = self.trace
        m = int(t.k.sum())
        src = self.pristine if self.resident else None
        if src is None:
            src = torch.from_numpy(self.ring_in.numpy()).to(self.dev)
        work = torch.empty_like(src)
        st = ctypes.c_void_p(self.s_cmp.cuda_stream)
        ts = []
        for it in range(iters + 1):
            work.copy_(src)
            torch.cuda.synchronize(self.dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(self.s_cmp):
                torch.cuda._sleep(200_000)
                e0.record()
                self.check(self.L.mi_inverse_descr_f32(
                    ctypes.c_void_p(work.data_ptr()), work.numel(), ctypes.c_void_p(self.d_off.data_ptr()),
                    ctypes.c_void_p(self.d_n.data_ptr()), ctypes.c_void_p(self.d_flag.data_ptr()), None,
                    ctypes.c_void_p(self.d_info.data_ptr()), m, self.n_mask, 1 << self.pivot,
                    ctypes.c_void_p(self.ws.data_ptr()), self.ws.numel(), st))
                e1.record()
            torch.cuda.synchronize(self.dev)
            if it > 0:
                ts.append(e0.elapsed_time(e1))
        return m / (float(np.median(ts)) / 1e3)

    def inputs(self, r: int):
        t = self.trace
        o, kk, nn = int(t.offset[r]), int(t.k[r]), int(t.n[r])
        return self.ring_in[o: o + kk * nn * nn].numpy().reshape(kk, nn, nn)


def residual_max(A: np.ndarray, X: np.ndarray) -> float:
    """max over the matrices of ||AX - I||_inf (FP64)."""
    n = A.shape[-1]
    R = np.einsum("bij,bjk->bik", A.astype(np.float64), X.astype(np.float64)) - np.eye(n)
    return float(np.abs(R).sum(-1).max())


def sweep(rates, num_requests: int, budget_gb: float = 16.0, seed: int = 0, modes=("coalesced", "per_request"),
          resident: bool = False, max_batch: int | None = None):
    base = make_trace(num_requests, rates[0], seed=seed)
    srv = CudaServer(base, hbm_budget_bytes=int(budget_gb * (1 << 30)), seed=seed, resident=resident,
                     max_batch=max_batch)
    out = []
    matrices = int(base.k.sum())
    srv.run(retime(base, rates[0], seed), coalesce=True)        # warm-up: module load, occupancy caches
    plain = srv.offline()
    print(json.dumps({"resident": resident, "offline_matrices_per_s": plain}), flush=True)
    sample = np.random.default_rng(seed).choice(num_requests, size=min(16, num_requests), replace=False)
    for rate in rates:
        tr = retime(base, rate, seed)
        row = {"rate_rps": rate, "requests": num_requests, "matrices": matrices, "resident": resident,
               "offline_matrices_per_s": plain, "max_batch": srv.max_batch}
        outs = {}
        for mode in modes:
            lat, wall = srv.run(tr, coalesce=(mode == "coalesced"))
            res = max(residual_max(srv.inputs(r), srv.results(r)) for r in sample)
            outs[mode] = {int(r): srv.results(r).copy() for r in sample[:4]}
            row[mode] = {"p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
                         "matrices_per_s": matrices / wall, "requests_per_s": num_requests / wall,
                         "max_residual_sample": res, **srv.last_stats}
        if len(modes) == 2:
            row["equal_bits"] = all(np.array_equal(outs[modes[0]][r], outs[modes[1]][r]) for r in outs[modes[0]])
        out.append(row)
        print(json.dumps(row), flush=True)
    return out


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--rates", default="1000,4000,16000,64000")
    p.add_argument("--requests", type=int, default=2000)
    p.add_argument("--budget-gb", type=float, default=16.0)
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--out", default=None)
    p.add_argument("--resident", action="store_true", help="requests already in HBM: no host copies")
    p.add_argument("--max-batch", type=int, default=None,
                   help="most matrices in one coalesced launch (default 2^20 resident, 2^16 with copies)")
    a = p.parse_args(argv)
    rows = sweep([float(x) for x in a.rates.split(",")], a.requests, a.budget_gb, a.seed, resident=a.resident,
                 max_batch=a.max_batch)
    if a.out:
        with open(a.out, "w") as f:
            json.dump(rows, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1:])
