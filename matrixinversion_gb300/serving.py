"""Serving loop: a stream of inversion requests, coalesced into device batches.

A request holds k matrices of one size n (partial pivoting by default).
Requests arrive (Poisson, in real time) into a pinned host ring in arrival
order -- the way a network receive buffer fills -- and the server admits
them first come, first served into a device pool with a fixed HBM budget:

* the pool is two arena halves carved once at start-up (no allocation on the
  serving path); a batch takes every arrived request that fits in a free
  half, so a half is the largest batch and the budget bounds what is resident;
* one batch = one host-to-device copy of its contiguous span of the ring, one
  descriptor call (GPU bucketing by size, one persistent launch per size
  present; a batch of one size stored back to back takes a single contiguous
  launch instead) and one device-to-host copy into the output ring, on
  separate copy and compute streams so that consecutive batches overlap;
* a request completes when the host sees its batch's last copy finish.

With `resident=True` the requests' matrices already sit in HBM (produced by
an upstream device stage): batches are inverted in place in the device ring,
with no copies, and `offline()` gives the plain batched kernel's rate on the
same matrices for comparison.

The baseline ("per_request") runs the same loop with one request per batch
and a plain contiguous launch per request.  Both paths run the same kernels
on the same data, so results are equal bit for bit (tested).

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
    batch's admission and issue; no-ops where torch was built without NVTX."""
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


class Batcher:
    """First come, first served admission under a per-batch float budget.

    next_batch(i, now) returns the end j of the batch [i, j): every request
    that has arrived by `now`, in order, while the span of the ring it covers
    fits in `half_floats` (the first request always fits: it is rejected at
    start-up if it alone exceeds the budget), at most `max_requests` of them.
    """

    def __init__(self, trace: Trace, half_floats: int, max_requests: int | None = None):
        self.t = trace
        self.half = int(half_floats)
        self.max_requests = max_requests
        ends = trace.offset + trace.floats
        if len(trace.k) and int((trace.floats).max()) > self.half:
            raise ValueError("a request is larger than one pool half; raise the HBM budget")
        self.ends = ends

    def next_batch(self, i: int, now: float) -> int:
        t = self.t
        nreq = len(t.k)
        if i >= nreq or t.arrival[i] > now:
            return i
        arrived = int(np.searchsorted(t.arrival, now, side="right"))
        limit = t.offset[i] + self.half
        fit = int(np.searchsorted(self.ends, limit, side="right"))
        j = min(arrived, fit)
        if self.max_requests is not None:
            j = min(j, i + self.max_requests)
        return max(j, i + 1)


class CudaServer:
    """The device side: pinned rings, the two arena halves, streams and the
    descriptor tables of the trace (built once on the device)."""

    def __init__(self, trace: Trace, hbm_budget_bytes: int = 16 << 30, device=None, pivot: int = PIVOT_PARTIAL,
                 seed: int = 0, resident: bool = False):
        import torch

        from . import _lib

        self.torch = torch
        self.L = _lib.load()
        self.check = _lib.check
        self.dev = torch.device(device or "cuda")
        self.trace = trace
        self.pivot = pivot
        total = trace.total_floats
        # the pool: two halves, each at most half the budget and no larger than the whole trace
        half = min(hbm_budget_bytes // 8, (total + 3) // 4 * 4)
        half = max(half, int(trace.floats.max()) + 4)
        if 8 * half > hbm_budget_bytes:
            raise ValueError("the largest request does not fit the HBM budget")
        self.half_floats = int(half)
        # resident: the requests' matrices already sit in HBM (an upstream
        # device stage produced them) and are inverted in place, no copies
        self.resident = resident
        self.arena = None if resident else torch.empty(2 * self.half_floats, dtype=torch.float32, device=self.dev)
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
        # descriptor tables of every matrix of the trace, in ring order, on the device
        k, n, off = trace.k, trace.n, trace.offset
        req_of = np.repeat(np.arange(len(k)), k)
        first = np.concatenate([[0], np.cumsum(k)[:-1]])
        local = np.arange(int(k.sum())) - np.repeat(first, k)
        mat_off = off[req_of] + local * (n[req_of] ** 2)
        self.mat_first = first.astype(np.int64)
        self.d_off = torch.from_numpy(mat_off.astype(np.int64)).to(self.dev)
        self.d_n = torch.from_numpy(n[req_of].astype(np.int32)).to(self.dev)
        self.d_flag = torch.full((int(k.sum()),), pivot, dtype=torch.int32, device=self.dev)
        self.d_rel = torch.empty_like(self.d_off)          # batch-relative offsets, written per batch
        self.d_info = torch.zeros(int(k.sum()), dtype=torch.int32, device=self.dev)
        self.ws = torch.empty(max(int(self.L.mi_descr_workspace_bytes(int(k.sum()))), 256), dtype=torch.uint8,
                              device=self.dev)
        self.s_h2d = torch.cuda.Stream(self.dev)
        self.s_cmp = torch.cuda.Stream(self.dev)
        self.s_d2h = torch.cuda.Stream(self.dev)
        self.n_mask = 0
        for v in np.unique(n):
            self.n_mask |= 1 << (int(v) - 1)

    def _launch_batch(self, i: int, j: int, half: int, coalesce: bool):
        torch = self.torch
        t = self.trace
        base = int(t.offset[i])
        end = int(t.offset[j - 1] + t.floats[j - 1])
        span = end - base
        if self.resident:
            dst = self.ring_dev[base:end]
        else:
            dst = self.arena[half * self.half_floats: half * self.half_floats + span]
            ev_in = torch.cuda.Event()
            with torch.cuda.stream(self.s_h2d):
                dst.copy_(self.ring_in[base:end], non_blocking=True)
                ev_in.record(self.s_h2d)
            self.s_cmp.wait_event(ev_in)
        st = ctypes.c_void_p(self.s_cmp.cuda_stream)
        m0 = int(self.mat_first[i])
        m1 = int(self.mat_first[j - 1] + t.k[j - 1])
        with torch.cuda.stream(self.s_cmp):
            nb = t.n[i:j]
            packed = bool(np.all(t.offset[i + 1:j] == t.offset[i:j - 1] + t.floats[i:j - 1]))
            if coalesce and nb.min() == nb.max() and packed:
                # one size, back to back in the ring: a single contiguous launch
                status = self.L.mi_inverse_f32(ctypes.c_void_p(dst.data_ptr()), None,
                                               ctypes.c_void_p(self.d_info[m0:m1].data_ptr()), m1 - m0, int(nb[0]),
                                               self.pivot, st)
                self.check(status)
            elif coalesce:
                offs = torch.sub(self.d_off[m0:m1], base, out=self.d_rel[m0:m1])
                status = self.L.mi_inverse_descr_f32(
                    ctypes.c_void_p(dst.data_ptr()), dst.numel(), ctypes.c_void_p(offs.data_ptr()),
                    ctypes.c_void_p(self.d_n[m0:m1].data_ptr()), ctypes.c_void_p(self.d_flag[m0:m1].data_ptr()),
                    None, ctypes.c_void_p(self.d_info[m0:m1].data_ptr()), m1 - m0, self.n_mask, 1 << self.pivot,
                    ctypes.c_void_p(self.ws.data_ptr()), self.ws.numel(), st)
                self.check(status)
            else:
                for r in range(i, j):
                    o = int(t.offset[r]) - base
                    nr = int(t.n[r])
                    mr = int(self.mat_first[r])
                    status = self.L.mi_inverse_f32(ctypes.c_void_p(dst.data_ptr() + 4 * o), None,
                                                   ctypes.c_void_p(self.d_info[mr:mr + int(t.k[r])].data_ptr()),
                                                   int(t.k[r]), nr, self.pivot, st)
                    self.check(status)
            ev_cmp = torch.cuda.Event()
            ev_cmp.record(self.s_cmp)
        if self.resident:
            return ev_cmp
        self.s_d2h.wait_event(ev_cmp)
        ev_out = torch.cuda.Event()
        with torch.cuda.stream(self.s_d2h):
            self.ring_out[base:end].copy_(dst, non_blocking=True)
            ev_out.record(self.s_d2h)
        return ev_out

    def run(self, trace: Trace | None = None, coalesce: bool = True, max_requests: int | None = None):
        """Serve `trace` in real time; returns per-request latencies (s) and the
        wall time from the first arrival to the last completion."""
        t = trace or self.trace
        assert np.array_equal(t.offset, self.trace.offset)
        batcher = Batcher(t, self.half_floats, max_requests=(max_requests if coalesce else 1))
        nreq = len(t.k)
        done = np.full(nreq, np.nan)
        inflight: list[tuple[int, int, int, object]] = []   # (i, j, half, event)
        free = [0, 1]
        i = 0
        completed = 0
        push, pop = nvtx_ranges()
        if self.resident:
            self.ring_dev.copy_(self.pristine)
        self.torch.cuda.synchronize(self.dev)
        t0 = time.perf_counter()
        while completed < nreq:
            now = time.perf_counter() - t0
            while inflight and inflight[0][3].query():
                a, b, h, _ = inflight.pop(0)
                done[a:b] = now
                completed += b - a
                free.append(h)
            if free and i < nreq and t.arrival[i] <= now:
                j = batcher.next_batch(i, now)
                h = free.pop(0)
                push(f"batch requests {i}-{j - 1}")
                inflight.append((i, j, h, self._launch_batch(i, j, h, coalesce)))
                pop()
                i = j
        lat = done - t.arrival
        wall = float(np.nanmax(done))
        return lat, wall

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
          resident: bool = False):
    base = make_trace(num_requests, rates[0], seed=seed)
    srv = CudaServer(base, hbm_budget_bytes=int(budget_gb * (1 << 30)), seed=seed, resident=resident)
    out = []
    matrices = int(base.k.sum())
    srv.run(retime(base, rates[0], seed), coalesce=True)        # warm-up: module load, occupancy caches
    plain = srv.offline()
    print(json.dumps({"resident": resident, "offline_matrices_per_s": plain}), flush=True)
    sample = np.random.default_rng(seed).choice(num_requests, size=min(16, num_requests), replace=False)
    for rate in rates:
        tr = retime(base, rate, seed)
        row = {"rate_rps": rate, "requests": num_requests, "matrices": matrices, "resident": resident,
               "offline_matrices_per_s": plain}
        outs = {}
        for mode in modes:
            lat, wall = srv.run(tr, coalesce=(mode == "coalesced"))
            res = max(residual_max(srv.inputs(r), srv.results(r)) for r in sample)
            outs[mode] = {int(r): srv.results(r).copy() for r in sample[:4]}
            row[mode] = {"p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
                         "matrices_per_s": matrices / wall, "requests_per_s": num_requests / wall,
                         "max_residual_sample": res}
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
    a = p.parse_args(argv)
    rows = sweep([float(x) for x in a.rates.split(",")], a.requests, a.budget_gb, a.seed, resident=a.resident)
    if a.out:
        with open(a.out, "w") as f:
            json.dump(rows, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1:])
