"""Batched inverse of matrices held in host memory.

The reference's driver copies the whole batch to the device, launches once
and copies it back (parallel_pivot/luBatchedInplace.cu:113-135).  Here the
batch streams through in chunks: one stream copies chunks in, one inverts
them, one copies them out, and `slots` device buffers rotate between them
(events order each chunk's three stages and keep a buffer from being refilled
before its results have left), so the copy-in of one chunk, the kernel on
another and the copy-out of a third overlap, and the two copy directions never
share a stream.  The kernel is the same C-ABI entry point (mi_inverse_cfg_f32);
there is no host computation.
"""
from __future__ import annotations

import time

import torch

from . import batched_inverse_


class HostPipeline:
    """Reusable device buffers and streams for host-memory batches of one n."""

    def __init__(self, n: int, chunk: int = 65536, streams: int = 4, device: int | str | None = None):
        self.n = int(n)
        self.chunk = int(chunk)
        self.slots = max(2, int(streams))
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.s_in, self.s_cmp, self.s_out = (torch.cuda.Stream(device=self.device) for _ in range(3))
        self.buf = [torch.empty((self.chunk, n, n), dtype=torch.float32, device=self.device) for _ in range(self.slots)]
        self.pbuf = [torch.empty((self.chunk, n), dtype=torch.int32, device=self.device) for _ in range(self.slots)]
        self.ibuf = [torch.empty((self.chunk,), dtype=torch.int32, device=self.device) for _ in range(self.slots)]
        self.free = [torch.cuda.Event() for _ in range(self.slots)]

    def run(self, A: torch.Tensor, pivot=True, out: torch.Tensor | None = None, perm: torch.Tensor | None = None,
            info: torch.Tensor | None = None):
        """Invert host tensor A [batch, n, n] (pinned for overlap) into `out`.

        Returns (out, perm, info), all host tensors; allocated pinned when not
        given.  Synchronises before returning.
        """
        if A.is_cuda or A.dtype != torch.float32 or A.dim() != 3 or A.shape[1:] != (self.n, self.n):
            raise ValueError(f"expected a host float32 tensor [batch, {self.n}, {self.n}]")
        batch = A.shape[0]
        pin = A.is_pinned()
        if out is None:
            out = torch.empty_like(A, pin_memory=pin)
        if perm is None:
            perm = torch.empty((batch, self.n), dtype=torch.int32, pin_memory=pin)
        if info is None:
            info = torch.empty((batch,), dtype=torch.int32, pin_memory=pin)
        cur = torch.cuda.current_stream(self.device)
        for s in (self.s_in, self.s_cmp, self.s_out):
            s.wait_stream(cur)
        for c, lo in enumerate(range(0, batch, self.chunk)):
            hi = min(batch, lo + self.chunk)
            k = c % self.slots
            d, dp, di = self.buf[k][: hi - lo], self.pbuf[k][: hi - lo], self.ibuf[k][: hi - lo]
            loaded, done = torch.cuda.Event(), torch.cuda.Event()
            with torch.cuda.stream(self.s_in):
                if c >= self.slots:
                    self.s_in.wait_event(self.free[k])      # this buffer's previous results have left
                d.copy_(A[lo:hi], non_blocking=True)
                loaded.record(self.s_in)
            with torch.cuda.stream(self.s_cmp):
                self.s_cmp.wait_event(loaded)
                batched_inverse_(d, pivot, perm=dp, info=di, stream=self.s_cmp)
                done.record(self.s_cmp)
            with torch.cuda.stream(self.s_out):
                self.s_out.wait_event(done)
                out[lo:hi].copy_(d, non_blocking=True)
                perm[lo:hi].copy_(dp, non_blocking=True)
                info[lo:hi].copy_(di, non_blocking=True)
                self.free[k].record(self.s_out)
        self.s_out.synchronize()
        return out, perm, info

    def launches_per_call(self, batch: int) -> int:
        return (batch + self.chunk - 1) // self.chunk


def link_bandwidth(device=None, nbytes: int = 1 << 30, reps: int = 3) -> dict:
    """Pinned host <-> device copy rates (GB/s): each direction alone, and each
    way while both run at once (the ceiling of an overlapped pipeline).  Best
    of `reps` after one warm-up copy."""
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    n = nbytes // 4
    h_in = torch.ones(n, dtype=torch.float32).pin_memory()
    h_out = torch.empty(n, dtype=torch.float32).pin_memory()
    d_a = torch.empty(n, dtype=torch.float32, device=dev)
    d_b = torch.zeros(n, dtype=torch.float32, device=dev)
    s1, s2 = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)
    res = {}
    for name in ("h2d_gbs", "d2h_gbs", "both_each_way_gbs"):
        best = None
        for _ in range(reps + 1):
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            if name != "d2h_gbs":
                with torch.cuda.stream(s1):
                    d_a.copy_(h_in, non_blocking=True)
            if name != "h2d_gbs":
                with torch.cuda.stream(s2):
                    h_out.copy_(d_b, non_blocking=True)
            torch.cuda.synchronize(dev)
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        res[name] = nbytes / best / 1e9
    del h_in, h_out, d_a, d_b
    return res


def batched_inverse_host(A: torch.Tensor, pivot=True, *, chunk: int = 65536, streams: int = 4):
    """One-shot convenience wrapper around HostPipeline.run."""
    return HostPipeline(A.shape[-1], chunk=chunk, streams=streams).run(A, pivot)
