"""Batched inverse of matrices held in host memory.

The reference's driver copies the whole batch to the device, launches once
and copies it back (parallel_pivot/luBatchedInplace.cu:113-135).  Here the
batch streams through in chunks on several CUDA streams, so the host-to-
device copy of one chunk, the kernel on another and the device-to-host copy
of a third overlap.  The kernel is the same C-ABI entry point
(mi_inverse_cfg_f32); there is no host computation.
"""
from __future__ import annotations

import torch

from . import batched_inverse_


class HostPipeline:
    """Reusable device buffers and streams for host-memory batches of one n."""

    def __init__(self, n: int, chunk: int = 65536, streams: int = 3, device: int | str | None = None):
        self.n = int(n)
        self.chunk = int(chunk)
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(streams)]
        self.buf = [torch.empty((self.chunk, n, n), dtype=torch.float32, device=self.device) for _ in range(streams)]
        self.pbuf = [torch.empty((self.chunk, n), dtype=torch.int32, device=self.device) for _ in range(streams)]
        self.ibuf = [torch.empty((self.chunk,), dtype=torch.int32, device=self.device) for _ in range(streams)]

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
        for s in self.streams:
            s.wait_stream(cur)
        for c, lo in enumerate(range(0, batch, self.chunk)):
            hi = min(batch, lo + self.chunk)
            k = c % len(self.streams)
            s, d, dp, di = self.streams[k], self.buf[k][: hi - lo], self.pbuf[k][: hi - lo], self.ibuf[k][: hi - lo]
            with torch.cuda.stream(s):
                d.copy_(A[lo:hi], non_blocking=True)
                batched_inverse_(d, pivot, perm=dp, info=di, stream=s)
                out[lo:hi].copy_(d, non_blocking=True)
                perm[lo:hi].copy_(dp, non_blocking=True)
                info[lo:hi].copy_(di, non_blocking=True)
        for s in self.streams:
            s.synchronize()
        return out, perm, info

    def launches_per_call(self, batch: int) -> int:
        return (batch + self.chunk - 1) // self.chunk


def batched_inverse_host(A: torch.Tensor, pivot=True, *, chunk: int = 65536, streams: int = 3):
    """One-shot convenience wrapper around HostPipeline.run."""
    return HostPipeline(A.shape[-1], chunk=chunk, streams=streams).run(A, pivot)
