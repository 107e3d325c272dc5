"""The no-allocation descriptor entry point, called through the C ABI.

mi_inverse_descr_noalloc_f32 runs the same bucketing and kernels as
mi_inverse_descr_f32 with its scratch in a fixed device array, so its
results must equal the workspace entry point's within a tolerance of zero
(same arithmetic on the same data), on two calls in a row with different
data -- the second call must not see the first call's bucket counters.
The file name sorts last, so in a full run this also checks the entry point
after every other GPU test has used the device in the same process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 0.0   # bit-identical: the two entry points share every kernel


def _case(oracle, count, seed):
    rng = np.random.RandomState(seed)
    ns = rng.randint(1, 33, size=count).astype(np.int32)
    flags = rng.randint(0, 4, size=count).astype(np.int32)
    mats = []
    for i, (n, f) in enumerate(zip(ns, flags)):
        A = oracle.uniform(seed * 100003 + i, 1, int(n))[0]
        if f == 0:
            A = A + np.float32(n) * np.eye(n, dtype=np.float32)
        mats.append(A)
    return mats, flags


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_matches_workspace_entry_point_twice(mi_gpu, oracle):
    import torch

    from matrixinversion_gb300 import _lib, descr

    L = _lib.load()
    stream = torch.cuda.current_stream()
    for call, seed in enumerate((5, 6)):
        mats, flags = _case(oracle, 1500 + 300 * call, seed)
        packed, offsets, ns = descr.pack(mats, align=1 + 3 * call)
        count = len(mats)
        d_off = torch.from_numpy(offsets).cuda()
        d_n = torch.from_numpy(ns).cuda()
        d_f = torch.from_numpy(flags).cuda()
        a = torch.from_numpy(packed).cuda()
        b = a.clone()
        perm_a = torch.full((count, 32), -9, dtype=torch.int32, device="cuda")
        perm_b = perm_a.clone()
        info_a = torch.full((count,), -9, dtype=torch.int32, device="cuda")
        info_b = info_a.clone()
        ws = torch.empty(descr.workspace_bytes(count), dtype=torch.uint8, device="cuda")
        st = L.mi_inverse_descr_f32(_ptr(a), a.numel(), _ptr(d_off), _ptr(d_n), _ptr(d_f), _ptr(perm_a),
                                    _ptr(info_a), count, 0, 0, _ptr(ws), ws.numel(),
                                    ctypes.c_void_p(stream.cuda_stream))
        assert st == 0, _lib.load().mi_error_string(st)
        st = L.mi_inverse_descr_noalloc_f32(_ptr(b), b.numel(), _ptr(d_off), _ptr(d_n), _ptr(d_f), _ptr(perm_b),
                                            _ptr(info_b), count, 0, 0, ctypes.c_void_p(stream.cuda_stream))
        assert st == 0, (st, L.mi_error_string(st), L.mi_last_cuda_error())
        torch.cuda.synchronize()
        a, b = a.cpu().numpy(), b.cpu().numpy()
        np.testing.assert_allclose(b, a, rtol=TOL, atol=TOL)
        assert np.array_equal(perm_b.cpu().numpy(), perm_a.cpu().numpy())
        assert np.array_equal(info_b.cpu().numpy(), info_a.cpu().numpy())
        # and the result is an inverse, not a copy of the input
        X = descr.unpack(b, offsets, ns)
        k = int(np.argmax(ns))
        r = np.abs(mats[k].astype(np.float64) @ X[k].astype(np.float64) - np.eye(ns[k])).max()
        assert r < 1e-2, r


def test_noalloc_rejects_count_above_limit(mi_gpu):
    import torch

    from matrixinversion_gb300 import _lib

    L = _lib.load()
    x = torch.zeros(16, dtype=torch.float32, device="cuda")
    o = torch.zeros(1, dtype=torch.int64, device="cuda")
    i = torch.ones(1, dtype=torch.int32, device="cuda")
    st = L.mi_inverse_descr_noalloc_f32(_ptr(x), x.numel(), _ptr(o), _ptr(i), _ptr(i), None, None,
                                        _lib.MI_NOALLOC_MAX_COUNT + 1, 0, 0, None)
    assert st == _lib.MI_ERR_SCRATCH_LIMIT
    assert b"MI_NOALLOC_MAX_COUNT" in L.mi_error_string(st)
    torch.cuda.synchronize()
    assert float(x.abs().sum()) == 0.0     # nothing launched
