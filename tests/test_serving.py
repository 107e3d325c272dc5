"""Serving loop: the pool allocator and argument checks (CPU), alone-vs-coalesced
equality, admission under a tight budget and the resident mode (GPU)."""
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


EXTENT_TEST = r"""
#include <cstdio>
#include <vector>
#include "mi_extents.h"
int main() {
    mi::ExtentPool p(100);
    long a = p.alloc(30), b = p.alloc(30), c = p.alloc(30);
    if (a != 0 || b != 30 || c != 60 || p.alloc(20) != -1 || p.alloc(10) != 90) return 1;   // first fit
    p.release(30, 30);                                  // a hole in the middle
    if (p.alloc(40) != -1 || p.largest_free() != 30) return 2;
    if (p.alloc(25) != 30) return 3;                    // first fit takes the hole
    p.release(30, 25); p.release(0, 30); p.release(60, 30); p.release(90, 10);
    if (p.free_extents() != 1 || p.largest_free() != 100 || p.used() != 0) return 4;   // merged back
    if (p.peak() != 100) return 5;
    if (p.alloc(0) != -1 || p.alloc(101) != -1) return 6;
    // a long random sequence keeps the accounting exact and merges fully
    mi::ExtentPool q(1 << 20);
    std::vector<std::pair<long, long>> live;
    unsigned x = 12345;
    for (int i = 0; i < 20000; i++) {
        x = x * 1103515245u + 12345u;
        if ((x >> 16) % 3 != 0 || live.empty()) {
            long len = 1 + (long)((x >> 8) % 4096);
            long off = q.alloc(len);
            if (off >= 0) {
                for (auto& e : live) if (off < e.first + e.second && e.first < off + len) return 7;   // no overlap
                live.push_back({off, len});
            }
        } else {
            size_t k = (x >> 4) % live.size();
            q.release(live[k].first, live[k].second);
            live.erase(live.begin() + k);
        }
    }
    long used = 0;
    for (auto& e : live) used += e.second;
    if (used != q.used()) return 8;
    for (auto& e : live) q.release(e.first, e.second);
    if (q.free_extents() != 1 || q.used() != 0) return 9;
    std::puts("ok");
    return 0;
}
"""


def test_extent_pool_first_fit_and_merging(tmp_path):
    """The serving pool's allocator (csrc/mi_extents.h): first fit, holes
    reused, released extents merged back, no two live extents overlap."""
    import os
    import subprocess

    src = tmp_path / "t.cpp"
    src.write_text(EXTENT_TEST)
    exe = tmp_path / "t"
    csrc = os.path.join(os.path.dirname(serving.__file__), "csrc")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + csrc, str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.returncode


def test_serve_run_argument_checks_without_gpu():
    """mi_serve_run rejects malformed traces before any CUDA call."""
    import ctypes

    from matrixinversion_gb300 import _lib

    L = _lib.load()
    assert L.mi_serve_scratch_bytes(0) == 0
    assert L.mi_serve_scratch_bytes(1000) >= 2 * 16 * 1000 + L.mi_descr_workspace_bytes(1000)
    arr = np.zeros(2, dtype=np.float64)
    k = np.ones(2, dtype=np.int64)
    n = np.full(2, 4, dtype=np.int32)
    off = np.array([0, 16], dtype=np.int64)
    lat = np.zeros(2, dtype=np.float64)
    p = lambda a: ctypes.c_void_p(a.ctypes.data)
    fake = ctypes.c_void_p(0x100000)

    def call(nreq=2, arrival=arr, kk=k, nn=n, maxb=8, pivot=3, scratch=fake, sbytes=1 << 20, ring=None, pool=fake):
        return L.mi_serve_run(nreq, p(arrival), p(kk), p(nn), p(off), fake, fake, ring, pool, 1 << 20, scratch,
                              sbytes, maxb, pivot, 1, p(lat), None, None)

    assert call(nreq=0) == _lib.MI_OK
    assert call(nreq=-1) == _lib.MI_ERR_INVALID_VALUE
    assert call(pivot=4) == _lib.MI_ERR_INVALID_VALUE
    assert call(maxb=0) == _lib.MI_ERR_INVALID_VALUE
    assert call(scratch=None) == _lib.MI_ERR_NULL_POINTER
    assert call(sbytes=16) == _lib.MI_ERR_INVALID_VALUE
    assert call(scratch=ctypes.c_void_p(0x100010)) == _lib.MI_ERR_INVALID_VALUE
    assert call(nn=np.array([4, 33], dtype=np.int32)) == _lib.MI_ERR_INVALID_VALUE
    assert call(kk=np.array([1, 9], dtype=np.int64)) == _lib.MI_ERR_INVALID_VALUE    # above max_batch
    assert call(arrival=np.array([1.0, 0.5])) == _lib.MI_ERR_INVALID_VALUE           # not in arrival order
    assert call(pool=None) == _lib.MI_ERR_NULL_POINTER


@pytest.mark.gpu
def test_coalesced_equals_alone(mi_gpu):
    """Every request's inverse is the same, bit for bit, whether it is served
    in a coalesced mixed-size batch, alone, or by a direct call."""
    import torch

    t = serving.make_trace(60, 20000.0, seed=11, kmax=64)
    srv = serving.CudaServer(t, hbm_budget_bytes=1 << 28, seed=11)
    lat, wall = srv.run(coalesce=True)
    assert np.all(np.isfinite(lat)) and np.all(lat >= 0) and wall > 0
    assert srv.last_stats["batches"] >= 1 and srv.last_stats["peak_pool_bytes"] <= 1 << 28
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


@pytest.mark.gpu
def test_tight_budget_admits_as_extents_free(mi_gpu):
    """A pool that holds only a few requests at a time: requests wait for
    memory, are admitted as extents free, and every result is still the
    direct call's, bit for bit; the pool's peak stays inside the budget."""
    import torch

    t = serving.make_trace(80, 50000.0, seed=17, kmax=256)
    budget = int(((t.floats + 3) // 4 * 4).max()) * 4 * 3          # about three of the largest requests
    srv = serving.CudaServer(t, hbm_budget_bytes=budget, seed=17)
    lat, wall = srv.run(coalesce=True)
    assert np.all(np.isfinite(lat)) and wall > 0
    assert srv.last_stats["peak_pool_bytes"] <= budget
    for r in range(0, 80, 7):
        X, _, _ = mi_gpu.batched_inverse(torch.from_numpy(srv.inputs(r).copy()).cuda(), "partial")
        assert np.array_equal(X.cpu().numpy(), srv.results(r)), r


def test_resident_ring_must_fit_the_budget():
    t = serving.make_trace(50, 1000.0, seed=3, kmax=64)
    with pytest.raises(ValueError):
        serving.CudaServer(t, hbm_budget_bytes=4 * t.total_floats - 4, resident=True, device="cpu")
