"""Mixed-size batches through an (offset, n, pivot flag) descriptor table.

Matrix i of a packed float32 buffer starts at offsets[i] (floats) and is
n_i x n_i, row-major; flags[i] is its pivot mode (0 none, 1 reference,
2 reference_serial, 3 partial).  One call buckets the table by (n, flag) on
the GPU and runs one persistent launch per bucket present (the default) or,
after set_chunk(c > 0), ONE persistent launch whose warps take chunks of
groups of every bucket from a device counter, largest n first -- all
stream-ordered, so the call can be captured into a CUDA graph (DescrGraph).
Either way every matrix gets the bits of the contiguous call.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib, pivot_mode


def pack(matrices, align: int = 4):
    """Pack host matrices (a list of square float32 arrays) back to back.

    Each matrix starts on a multiple of `align` floats (4 = 16 bytes, which
    lets the copies use the bulk copy engine; 1 = densely packed).  Returns
    (packed float32[total], offsets int64[count], ns int32[count]).
    """
    ns = np.array([m.shape[0] for m in matrices], dtype=np.int32)
    offsets = np.zeros(len(matrices), dtype=np.int64)
    pos = 0
    for i, m in enumerate(matrices):
        pos = (pos + align - 1) // align * align
        offsets[i] = pos
        pos += m.shape[0] * m.shape[0]
    packed = np.zeros(max(pos, 1), dtype=np.float32)
    for i, m in enumerate(matrices):
        k = m.shape[0]
        packed[offsets[i]: offsets[i] + k * k] = np.asarray(m, dtype=np.float32).reshape(-1)
    return packed, offsets, ns


def unpack(packed, offsets, ns):
    return [np.asarray(packed[o: o + n * n]).reshape(n, n) for o, n in zip(offsets, ns)]


def set_chunk(chunk_floats: int) -> None:
    """Form of the descriptor call: 0 (the default) = one launch per (n, mode)
    bucket; c > 0 = the single persistent launch with chunks of about c input
    floats (1 to 8 groups).  Process-wide."""
    _lib.check(_lib.load().mi_set_descr_chunk(int(chunk_floats)))


def get_chunk() -> int:
    return int(_lib.load().mi_get_descr_chunk())


def workspace_bytes(count: int) -> int:
    return int(_lib.load().mi_descr_workspace_bytes(int(count)))


def masks(ns, flags) -> tuple[int, int]:
    """(n_mask, mode_mask) covering the sizes and modes present."""
    ns = np.asarray(ns)
    flags = np.asarray(flags)
    n_mask = 0
    for n in np.unique(ns):
        if 1 <= n <= 32:
            n_mask |= 1 << (int(n) - 1)
    mode_mask = 0
    for f in np.unique(flags):
        if 0 <= f <= 3:
            mode_mask |= 1 << int(f)
    return n_mask, mode_mask


def batched_inverse_descr_(packed, offsets, ns, flags, *, perm=None, info=None, workspace=None, n_mask: int = 0,
                           mode_mask: int = 0, stream=None):
    """In-place inverse of every described matrix (CUDA tensors).

    packed float32 [total]; offsets int64 [count]; ns, flags int32 [count];
    perm int32 [count, 32] and info int32 [count] optional; workspace uint8
    [workspace_bytes(count)] (allocated when None).  Returns (perm, info).
    """
    import torch

    for name, t, dt in (("packed", packed, torch.float32), ("offsets", offsets, torch.int64),
                        ("ns", ns, torch.int32), ("flags", flags, torch.int32)):
        if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == dt and t.is_contiguous()):
            raise TypeError(f"{name} must be a contiguous CUDA {dt} tensor")
    count = offsets.numel()
    if ns.numel() != count or flags.numel() != count:
        raise ValueError("offsets, ns and flags must have the same length")
    dev = packed.device
    for name, t in (("offsets", offsets), ("ns", ns), ("flags", flags)):
        if t.device != dev:
            raise ValueError(f"{name} must be on {dev}, with packed")
    # the kernels write perm[i * 32 ..] and info[i] for every listed matrix
    for name, t, numel in (("perm", perm, count * 32), ("info", info, count)):
        if t is not None and not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.int32
                                  and t.is_contiguous() and t.device == dev and t.numel() == numel):
            raise ValueError(f"{name} must be a contiguous int32 tensor of {numel} elements on {dev}")
    if workspace is not None and not (isinstance(workspace, torch.Tensor) and workspace.device == dev
                                      and workspace.is_contiguous()):
        raise ValueError(f"workspace must be a contiguous tensor on {dev}")
    if workspace is None:
        workspace = torch.empty(max(workspace_bytes(count), 256), dtype=torch.uint8, device=dev)
    L = _lib.load()
    st = (stream or torch.cuda.current_stream(dev)).cuda_stream
    with torch.cuda.device(dev):
        status = L.mi_inverse_descr_f32(
            ctypes.c_void_p(packed.data_ptr()), packed.numel(), ctypes.c_void_p(offsets.data_ptr()),
            ctypes.c_void_p(ns.data_ptr()),
            ctypes.c_void_p(flags.data_ptr()), ctypes.c_void_p(perm.data_ptr() if perm is not None else 0),
            ctypes.c_void_p(info.data_ptr() if info is not None else 0), count, n_mask & 0xFFFFFFFF,
            mode_mask & 0xF, ctypes.c_void_p(workspace.data_ptr()), workspace.numel() * workspace.element_size(),
            ctypes.c_void_p(st))
    _lib.check(status)
    return perm, info


class DescrGraph:
    """One descriptor call captured into a CUDA graph over fixed buffers.

    Refill `packed` (and the descriptor tensors) in place, then `replay()`:
    every bucket launch goes out as a single graph launch.
    """

    def __init__(self, packed, offsets, ns, flags, perm=None, info=None, n_mask: int = 0, mode_mask: int = 0):
        import torch

        self.args = (packed, offsets, ns, flags)
        self.perm, self.info = perm, info
        self.workspace = torch.empty(max(workspace_bytes(offsets.numel()), 256), dtype=torch.uint8,
                                     device=packed.device)
        self.masks = (n_mask, mode_mask)
        self.stream = torch.cuda.Stream(device=packed.device)
        # the first call sets kernel attributes and occupancy caches outside capture
        scratch = packed.clone()
        with torch.cuda.stream(self.stream):
            batched_inverse_descr_(scratch, offsets, ns, flags, perm=perm, info=info, workspace=self.workspace,
                                   n_mask=n_mask, mode_mask=mode_mask, stream=self.stream)
        self.stream.synchronize()
        del scratch
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=self.stream):
            batched_inverse_descr_(packed, offsets, ns, flags, perm=perm, info=info, workspace=self.workspace,
                                   n_mask=n_mask, mode_mask=mode_mask, stream=self.stream)

    def replay(self):
        self.graph.replay()


def uneven_batch(count: int, align: int = 4, seed: int = 0, pivot_flag: int = 1, device="cuda"):
    """The uneven workload: n ~ U{2..32} (seeded), a 50/50 flag between no
    pivoting and `pivot_flag`, entries uniform [-1, 1), +n on the diagonal of
    the no-pivot matrices; packed with `align`-float alignment.  Returns device
    tensors (packed, offsets, ns, flags)."""
    import torch

    g = torch.Generator(device="cpu").manual_seed(seed)
    ns = torch.randint(2, 33, (count,), generator=g, dtype=torch.int32)
    flags = torch.where(torch.rand(count, generator=g) < 0.5, 0, pivot_flag).to(torch.int32)
    sz = (ns.long() * ns.long() + align - 1) // align * align
    offsets = torch.cumsum(sz, 0) - sz
    total = int(sz.sum())
    gd = torch.Generator(device=device).manual_seed(seed + 1)
    packed = torch.rand(total, generator=gd, device=device) * 2 - 1
    offsets, ns, flags = offsets.to(device), ns.to(device), flags.to(device)
    sel = (flags == 0).nonzero().squeeze(1)
    nn_ = ns[sel].long()
    rep = torch.repeat_interleave(sel, nn_)
    k = torch.arange(rep.numel(), device=device) - torch.repeat_interleave(torch.cumsum(nn_, 0) - nn_, nn_)
    packed[offsets[rep] + k * (ns[rep].long() + 1)] += ns[rep].float()
    return packed, offsets, ns, flags


def bench_uneven(count: int = 1_000_000, align: int = 4, iters: int = 10, seed: int = 0, pivot_flag: int = 1,
                 chunks=(16384,)):
    """Descriptor call (eager and graph-captured; the single persistent launch
    at each chunk size of `chunks`, and one launch per bucket) vs one
    contiguous launch per (n, flag) bucket over the same matrices pre-sorted;
    kernel time by CUDA events, each run on a fresh copy of the inputs."""
    import torch

    import matrixinversion_gb300 as mi

    packed, offsets, ns, flags = uneven_batch(count, align, seed, pivot_flag)
    src = packed.clone()
    ws = torch.empty(max(workspace_bytes(count), 256), dtype=torch.uint8, device=packed.device)
    info = torch.empty(count, dtype=torch.int32, device=packed.device)
    n_mask, mode_mask = masks(ns.cpu().numpy(), flags.cpu().numpy())

    def timed(fn, reset):
        for _ in range(3):
            reset()
            fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(iters):
            reset()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    reset = lambda: packed.copy_(src)
    eager = lambda: batched_inverse_descr_(packed, offsets, ns, flags, info=info, workspace=ws, n_mask=n_mask,
                                           mode_mask=mode_mask)
    saved = get_chunk()
    forms = {}
    try:
        for c in [*chunks, 0]:
            set_chunk(c)
            t_e = timed(eager, reset)
            graph = DescrGraph(packed, offsets, ns, flags, info=info, n_mask=n_mask, mode_mask=mode_mask)
            forms[c] = (t_e, timed(graph.replay, reset))
    finally:
        set_chunk(saved)
    t_eager, t_graph = forms[chunks[0]]
    # per-bucket baseline: the same matrices sorted into contiguous buckets
    host = src.cpu().numpy()
    nh, fh, oh = ns.cpu().numpy(), flags.cpu().numpy(), offsets.cpu().numpy()
    buckets = []
    for n in range(2, 33):
        for f in np.unique(fh):
            sel = np.nonzero((nh == n) & (fh == f))[0]
            if len(sel):
                idx = (oh[sel][:, None] + np.arange(n * n)[None]).reshape(-1)
                B = torch.from_numpy(host[idx].reshape(len(sel), n, n)).to(packed.device)
                buckets.append((int(f), B, B.clone()))
    names = {0: "none", 1: "reference", 2: "reference_serial", 3: "partial"}

    def per_bucket():
        for f, B, _ in buckets:
            mi.batched_inverse_(B, names[f])

    def breset():
        for _, B, S in buckets:
            B.copy_(S)

    t_bucket = timed(per_bucket, breset)
    bytes_alg = float((8 * ns.double() ** 2 + 4 * ns.double() + 4).sum() + 16 * count)
    return {"count": count, "align": align, "chunk_floats": chunks[0], "eager_ms": t_eager, "graph_ms": t_graph,
            "launch_per_bucket": {"eager_ms": forms[0][0], "graph_ms": forms[0][1]},
            "chunk_sweep": {str(c): {"eager_ms": e, "graph_ms": g} for c, (e, g) in forms.items() if c},
            "per_bucket_ms": t_bucket,
            "buckets": len(buckets), "matrices_per_s_graph": count / t_graph * 1e3,
            "bytes_per_launch": bytes_alg, "GBs_graph": bytes_alg / t_graph / 1e6,
            "singular": int((info != 0).sum().item())}


def bench_single_size(ns=(2, 8, 14, 16, 24, 31, 32), count: int = 131072, flag: int = 1, iters: int = 8,
                      chunks=(1, 16384)):
    """Descriptor calls over one size at a time (masks naming that size and
    mode only): one launch per bucket against the single persistent launch
    at each chunk size; kernel time by CUDA events (median after two
    warm-ups), each run on a fresh copy of the inputs."""
    import torch

    saved = get_chunk()
    rows = []
    try:
        for n in ns:
            g = torch.Generator(device="cuda").manual_seed(n)
            src = (torch.rand(count, n, n, generator=g, device="cuda") * 2 - 1).reshape(-1)
            if flag == 0:
                src.view(count, n, n).add_(n * torch.eye(n, device="cuda"))
            d = src.clone()
            offsets = torch.arange(count, dtype=torch.int64, device="cuda") * (n * n)
            nsd = torch.full((count,), n, dtype=torch.int32, device="cuda")
            fl = torch.full((count,), flag, dtype=torch.int32, device="cuda")
            ws = torch.empty(workspace_bytes(count), dtype=torch.uint8, device="cuda")
            info = torch.empty(count, dtype=torch.int32, device="cuda")
            row = {"n": n, "flag": flag, "count": count}
            for c in (0, *chunks):
                set_chunk(c)
                ts = []
                for it in range(iters + 2):
                    d.copy_(src)
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record()
                    batched_inverse_descr_(d, offsets, nsd, fl, info=info, workspace=ws, n_mask=1 << (n - 1),
                                           mode_mask=1 << flag)
                    e1.record()
                    torch.cuda.synchronize()
                    if it >= 2:
                        ts.append(e0.elapsed_time(e1))
                row["per_bucket_ms" if c == 0 else f"persistent_{c}_ms"] = float(np.median(ts))
            rows.append(row)
    finally:
        set_chunk(saved)
    return rows


def main(argv=None):
    import argparse
    import json

    p = argparse.ArgumentParser()
    p.add_argument("--count", type=int, default=1_000_000)
    p.add_argument("--align", default="4,1")
    p.add_argument("--tune", action="store_true", help="autotune threads per block first")
    p.add_argument("--iters", type=int, default=10)
    p.add_argument("--chunks", default="16384", help="persistent-launch chunk sizes (floats), the first reported")
    p.add_argument("--single-size", default="", help="sizes to time one at a time (both forms) instead")
    a = p.parse_args(argv)
    if a.single_size:
        chunks = tuple(int(c) for c in a.chunks.split(","))
        for flag in (1, 0):
            for row in bench_single_size(tuple(int(x) for x in a.single_size.split(",")), a.count, flag,
                                         chunks=chunks):
                print(json.dumps(row), flush=True)
        return
    if a.tune:
        from . import autotune

        autotune.tune(range(2, 33), ("none", "reference"), batch=131072, iters=3)
    for al in a.align.split(","):
        chunks = tuple(int(c) for c in a.chunks.split(","))
        print(json.dumps({"tuned": a.tune, **bench_uneven(a.count, int(al), a.iters, chunks=chunks)}), flush=True)


__all__ = ["pack", "unpack", "set_chunk", "get_chunk", "workspace_bytes", "masks", "batched_inverse_descr_", "DescrGraph", "pivot_mode",
           "uneven_batch", "bench_uneven", "bench_single_size"]

if __name__ == "__main__":
    import sys

    main(sys.argv[1:])
