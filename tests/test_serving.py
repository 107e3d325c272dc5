"""Serving loop: host-side admission (CPU) and alone-vs-coalesced equality (GPU)."""
import numpy as np
import pytest

from matrixinversion_gb300 import serving


def test_trace_shape_and_ring_layout():
    t = serving.make_trace(500, 1000.0, seed=3)
    assert np.all(np.diff(t.arrival) >= 0) and t.arrival[0] == 0.0
    assert t.k.min() >= 1 and t.k.max() <= 4096
    assert set(np.unique(t.n)) <= set(serving.SIZES)
    assert np.all(t.offset % 4 == 0)                      # 16-byte aligned requests
    assert np.all(t.offset[1:] >= t.offset[:-1] + t.floats[:-1])
    # log-uniform k: about as many requests below 64 as above
    assert 0.35 < np.mean(t.k < 64) < 0.65
    r = serving.retime(t, 5000.0)
    assert np.array_equal(r.k, t.k) and np.array_equal(r.offset, t.offset)
    assert r.arrival[-1] < t.arrival[-1]


def test_batcher_is_fifo_within_budget():
    t = serving.make_trace(200, 1000.0, seed=5, kmax=64)
    half = int(t.floats.max()) * 10
    b = serving.Batcher(t, half)
    i, now = 0, 0.0
    seen = []
    while i < len(t.k):
        now = max(now, t.arrival[i])
        j = b.next_batch(i, now)
        assert j > i
        assert np.all(t.arrival[i:j] <= now)                         # only arrived requests
        assert t.offset[j - 1] + t.floats[j - 1] - t.offset[i] <= half   # the span fits one half
        if j < len(t.k) and t.arrival[j] <= now:                     # stopped by the budget
            assert t.offset[j] + t.floats[j] - t.offset[i] > half
        seen.extend(range(i, j))
        i = j
        now += 0.0005
    assert seen == list(range(len(t.k)))
    one = serving.Batcher(t, half, max_requests=1)
    assert one.next_batch(0, 10.0) == 1
    assert b.next_batch(5, t.arrival[5] - 1e-9) == 5                  # nothing has arrived yet
    with pytest.raises(ValueError):
        serving.Batcher(t, int(t.floats.max()) - 1)


@pytest.mark.gpu
def test_coalesced_equals_alone(mi_gpu):
    """Every request's inverse is the same, bit for bit, whether it is served
    in a coalesced mixed-size batch, alone, or by a direct call."""
    import torch

    t = serving.make_trace(60, 20000.0, seed=11, kmax=64)
    srv = serving.CudaServer(t, hbm_budget_bytes=1 << 28, seed=11)
    lat, wall = srv.run(coalesce=True)
    assert np.all(np.isfinite(lat)) and np.all(lat >= 0) and wall > 0
    mixed = [srv.results(r).copy() for r in range(60)]
    lat1, _ = srv.run(coalesce=False)
    assert np.all(np.isfinite(lat1))
    for r in range(60):
        assert np.array_equal(srv.results(r), mixed[r]), r
        A = srv.inputs(r)
        X, _, _ = mi_gpu.batched_inverse(torch.from_numpy(A.copy()).cuda(), "partial")
        assert np.array_equal(X.cpu().numpy(), mixed[r]), r
    assert serving.residual_max(srv.inputs(0), mixed[0]) < 1e-2


@pytest.mark.gpu
def test_resident_mode_equals_host_mode(mi_gpu):
    """Requests already in HBM, inverted in place: same bits as the host-ring path."""
    t = serving.make_trace(40, 20000.0, seed=13, kmax=64)
    host = serving.CudaServer(t, hbm_budget_bytes=1 << 28, seed=13)
    res = serving.CudaServer(t, hbm_budget_bytes=1 << 28, seed=13, resident=True)
    host.run(coalesce=True)
    for _ in range(2):                         # the ring is restored before every run
        lat, wall = res.run(coalesce=True)
        assert np.all(np.isfinite(lat)) and wall > 0
        for r in range(40):
            assert np.array_equal(res.results(r), host.results(r)), r
    assert res.offline(iters=2) > 0


def test_nvtx_ranges_are_callable_without_a_profiler():
    push, pop = serving.nvtx_ranges()
    push("batch requests 0-3")
    pop()
