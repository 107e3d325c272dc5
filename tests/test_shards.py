"""Batch shards and the max-over-ranks timing, with two gloo ranks on CPU."""
import os
import socket

import pytest
import torch
import torch.multiprocessing as mp

from matrixinversion_gb300 import shards


def test_shard_ranges_cover_the_batch():
    for total in (0, 1, 7, 1000, 1_000_003):
        for world in (1, 2, 3, 8):
            ranges = [shards.shard_range(total, r, world) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == total
            assert all(ranges[i][1] == ranges[i + 1][0] for i in range(world - 1))
            sizes = [hi - lo for lo, hi in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shards.shard_range(10, 2, 2)
    assert shards.shard_seed(5, 0) != shards.shard_seed(5, 1)
    assert shards.aggregate_rate(1000, 0.5, 4) == 8000.0


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # each rank "times" its shard; the job time is the slowest rank's
        t = shards.max_over_ranks(0.25 + rank * 0.5)
        lo, hi = shards.shard_range(1001, rank, world)
        got = torch.tensor([lo, hi], dtype=torch.int64)
        gathered = [torch.zeros(2, dtype=torch.int64) for _ in range(world)]
        dist.all_gather(gathered, got)
        out[rank] = (t, [tuple(g.tolist()) for g in gathered])
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        t, ranges = res[r]
        assert t == 0.75                                   # max over ranks
        assert ranges == [(0, 501), (501, 1001)]           # disjoint, covering
