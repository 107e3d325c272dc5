"""Descriptor batches (mixed n and pivot modes in one call) through the C ABI.

Every matrix must come back bit-for-bit equal to the contiguous kernel's
result for the same matrix (same arithmetic, different data movement), with
the same pivots; malformed descriptors are reported and left untouched; the
call replays correctly from a CUDA graph.  Each check runs in both forms of
the call: the single persistent launch (chunks of the default size) and one
launch per (n, mode) bucket.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MODES = ["none", "reference", "reference_serial", "partial"]


@pytest.fixture(params=["persistent", "per_bucket"])
def form(request):
    from matrixinversion_gb300 import descr

    saved = descr.get_chunk()
    descr.set_chunk(16384 if request.param == "persistent" else 0)
    yield request.param
    descr.set_chunk(saved)


def make_case(oracle, count, seed, nmin=1, nmax=32):
    rng = np.random.RandomState(seed)
    ns = rng.randint(nmin, nmax + 1, size=count)
    flags = rng.randint(0, 4, size=count)
    mats = []
    for i, (n, f) in enumerate(zip(ns, flags)):
        A = oracle.uniform(seed * 7919 + i, 1, int(n))[0]
        if f == 0:
            A = A + np.float32(n) * np.eye(n, dtype=np.float32)
        mats.append(A)
    return mats, ns.astype(np.int32), flags.astype(np.int32)


def contiguous_results(mi, mats, flags):
    import torch

    out, perms, infos = [], [], []
    for A, f in zip(mats, flags):
        X, p, i = mi.batched_inverse(torch.from_numpy(A[None]).cuda(), MODES[f])
        out.append(X[0].cpu().numpy())
        perms.append(p[0].cpu().numpy())
        infos.append(int(i[0].item()))
    return out, perms, infos


@pytest.mark.parametrize("align", [4, 1])
def test_descriptor_batch_matches_contiguous(mi_gpu, oracle, align, form):
    import torch

    from matrixinversion_gb300 import descr

    mats, ns, flags = make_case(oracle, 700, 3 + align)
    packed, offsets, ns_ = descr.pack(mats, align=align)
    d_packed = torch.from_numpy(packed).cuda()
    perm = torch.full((len(mats), 32), -7, dtype=torch.int32, device="cuda")
    info = torch.full((len(mats),), -7, dtype=torch.int32, device="cuda")
    descr.batched_inverse_descr_(d_packed, torch.from_numpy(offsets).cuda(), torch.from_numpy(ns_).cuda(),
                                 torch.from_numpy(flags).cuda(), perm=perm, info=info)
    got = descr.unpack(d_packed.cpu().numpy(), offsets, ns_)
    want, wperm, winfo = contiguous_results(mi_gpu, mats, flags)
    perm = perm.cpu().numpy()
    info = info.cpu().numpy()
    for i, n in enumerate(ns_):
        assert np.array_equal(got[i], want[i]), (i, n, flags[i])
        assert np.array_equal(perm[i, :n], wperm[i]), i
        assert info[i] == winfo[i]
    # pivots of the reference rules against the oracle replay
    for i, (A, f) in enumerate(zip(mats, flags)):
        if f in (1, 2):
            assert np.array_equal(perm[i, : A.shape[0]], oracle.pivots(A[None], MODES[f])[0])


def test_malformed_descriptors_and_masks(mi_gpu, oracle, form):
    import torch

    from matrixinversion_gb300 import descr

    mats, ns, flags = make_case(oracle, 40, 11, 2, 12)
    packed, offsets, ns_ = descr.pack(mats)
    bad_n = ns_.copy()
    bad_n[3] = 0
    bad_n[5] = 33
    bad_f = flags.copy()
    bad_f[7] = 9
    # matrices outside the packed buffer: a negative offset, and one that ends
    # a float past the end
    bad_off = offsets.copy()
    bad_off[9] = -4
    bad_off[11] = packed.size - int(ns_[11]) ** 2 + 1
    d_packed = torch.from_numpy(packed).cuda()
    info = torch.zeros(len(mats), dtype=torch.int32, device="cuda")
    descr.batched_inverse_descr_(d_packed, torch.from_numpy(bad_off).cuda(), torch.from_numpy(bad_n).cuda(),
                                 torch.from_numpy(bad_f).cuda(), info=info)
    info = info.cpu().numpy()
    out = d_packed.cpu().numpy()
    got = descr.unpack(out, offsets, ns_)
    for i in (3, 5, 7, 9, 11):
        assert info[i] == -1, i
        assert np.array_equal(got[i], mats[i]), i     # untouched
    want, _, _ = contiguous_results(mi_gpu, mats, flags)
    assert np.array_equal(got[0], want[0])
    # masks that exclude a present size leave those matrices untouched
    d_packed = torch.from_numpy(packed).cuda()
    n_mask, mode_mask = descr.masks(ns_, flags)
    n_mask &= ~(1 << (int(ns_[0]) - 1))
    descr.batched_inverse_descr_(d_packed, torch.from_numpy(offsets).cuda(), torch.from_numpy(ns_).cuda(),
                                 torch.from_numpy(flags).cuda(), n_mask=n_mask, mode_mask=mode_mask)
    got = descr.unpack(d_packed.cpu().numpy(), offsets, ns_)
    assert np.array_equal(got[0], mats[0])


def test_descriptor_graph_replay(mi_gpu, oracle, form):
    import torch

    from matrixinversion_gb300 import descr

    mats, ns, flags = make_case(oracle, 300, 21)
    packed, offsets, ns_ = descr.pack(mats)
    d_packed = torch.from_numpy(packed).cuda()
    n_mask, mode_mask = descr.masks(ns_, flags)
    g = descr.DescrGraph(d_packed, torch.from_numpy(offsets).cuda(), torch.from_numpy(ns_).cuda(),
                         torch.from_numpy(flags).cuda(), n_mask=n_mask, mode_mask=mode_mask)
    want, _, _ = contiguous_results(mi_gpu, mats, flags)
    for _ in range(2):
        d_packed.copy_(torch.from_numpy(packed))
        g.replay()
        torch.cuda.synchronize()
        got = descr.unpack(d_packed.cpu().numpy(), offsets, ns_)
        for i in range(len(mats)):
            assert np.array_equal(got[i], want[i]), i


@pytest.mark.parametrize("chunk", [1, 5000, 1 << 22])
def test_persistent_chunk_sizes(mi_gpu, oracle, chunk):
    """One group per chunk (the smallest chunk), mid-size chunks that split
    buckets between warps, and the largest (eight groups): the bits of the
    contiguous call every time, densely packed (4-byte aligned matrices)."""
    import torch

    from matrixinversion_gb300 import descr

    mats, ns, flags = make_case(oracle, 500, 31)
    packed, offsets, ns_ = descr.pack(mats, align=1)
    want, wperm, winfo = contiguous_results(mi_gpu, mats, flags)
    saved = descr.get_chunk()
    try:
        descr.set_chunk(chunk)
        d_packed = torch.from_numpy(packed).cuda()
        perm = torch.full((len(mats), 32), -7, dtype=torch.int32, device="cuda")
        info = torch.full((len(mats),), -7, dtype=torch.int32, device="cuda")
        descr.batched_inverse_descr_(d_packed, torch.from_numpy(offsets).cuda(), torch.from_numpy(ns_).cuda(),
                                     torch.from_numpy(flags).cuda(), perm=perm, info=info)
        torch.cuda.synchronize()
    finally:
        descr.set_chunk(saved)
    got = descr.unpack(d_packed.cpu().numpy(), offsets, ns_)
    perm, info = perm.cpu().numpy(), info.cpu().numpy()
    for i, n in enumerate(ns_):
        assert np.array_equal(got[i], want[i]), (i, n, flags[i])
        assert np.array_equal(perm[i, :n], wperm[i]), i
        assert info[i] == winfo[i]


def test_persistent_equals_per_bucket_large(mi_gpu):
    """60,000 matrices, every n = 1..32 and every pivot mode, some singular:
    the single persistent launch (many chunks per bucket, thousands of warps)
    and one launch per bucket give the same bits, pivots and info."""
    import torch

    from matrixinversion_gb300 import descr

    rng = np.random.RandomState(5)
    count = 60000
    ns = rng.randint(1, 33, size=count).astype(np.int32)
    flags = rng.randint(0, 4, size=count).astype(np.int32)
    offsets = np.zeros(count, dtype=np.int64)
    offsets[1:] = np.cumsum(ns.astype(np.int64) ** 2)[:-1]
    total = int(offsets[-1] + int(ns[-1]) ** 2)
    src = torch.from_numpy(rng.uniform(-1, 1, size=total).astype(np.float32)).cuda()
    for i in rng.choice(count, 50, replace=False):      # singular: a zero matrix
        src[int(offsets[i]): int(offsets[i]) + int(ns[i]) ** 2] = 0.0
    d_off, d_n, d_f = (torch.from_numpy(x).cuda() for x in (offsets, ns, flags))
    saved = descr.get_chunk()
    out = {}
    try:
        for c in (16384, 0):
            descr.set_chunk(c)
            d = src.clone()
            perm = torch.full((count, 32), -7, dtype=torch.int32, device="cuda")
            info = torch.full((count,), -7, dtype=torch.int32, device="cuda")
            descr.batched_inverse_descr_(d, d_off, d_n, d_f, perm=perm, info=info)
            torch.cuda.synchronize()
            out[c] = (d, perm, info)
    finally:
        descr.set_chunk(saved)
    assert torch.equal(out[16384][0].view(torch.int32), out[0][0].view(torch.int32))
    assert torch.equal(out[16384][1], out[0][1]) and torch.equal(out[16384][2], out[0][2])
    assert int((out[0][2] == -7).sum()) == 0 and int((out[0][2] != 0).sum()) >= 50
