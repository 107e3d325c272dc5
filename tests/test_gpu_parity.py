"""Parity of the sm_103a kernel (through the C ABI) with the oracle.

Tolerances, stated once:
  * pivots: bit-exact -- against the oracle's replay of the reference rules on
    every seeded input, and against the pivots the reference's own kernels
    produced (tests/golden).  The rules compare raw inputs only, so no
    floating-point slack is involved.
  * inverse, pivoted modes: per matrix
        ||AX - I||_inf <= max(8 n u || |L| |U| |X64| ||_inf, 2 r_port),
    where L U = P A is factored in FP64 in the kernel's own pivot order (the
    oracle's lu_growth_bound), X64 is the FP64 inverse and u = 2^-24 -- the
    componentwise residual bound of an LU-based inverse with that pivot
    sequence, which grows with the sequence's element growth (the reference
    rule is not stable) -- or, where even the reference algorithm breaks that
    bound (element growth so large that FP32 factors part from FP64 ones:
    about one matrix in 10^5), within 2x of r_port, the residual of the
    reference algorithm itself (FP32 Doolittle + comp_inv, the oracle's port)
    with the same pivots; and the batch median of ||AX - I||_inf within 2x of
    the port's median.  Over 1,000,000-matrix batches, two FP32 evaluation
    orders of one unstable pivot sequence differ by up to ~400x on single
    matrices, so no fixed multiple of r_port alone bounds them.
  * inverse, no pivoting (diagonally dominant inputs): ||AX - I||_inf <= 1e-5
    and max |X - X64| <= 1e-5 * max |X64| per matrix against the FP64 oracle.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

U = 2.0 ** -24


def gpu_inverse(mi, A, mode, **kw):
    import torch

    X, perm, info = mi.batched_inverse(torch.from_numpy(np.ascontiguousarray(A)).cuda(), mode, **kw)
    torch.cuda.synchronize()
    return X.cpu().numpy(), perm.cpu().numpy(), info.cpu().numpy()


def residual_bound(oracle, A, mode, perm=None):
    """Per-matrix tolerance on ||AX - I||_inf and the port's residuals."""
    n = A.shape[-1]
    Xp, pp, _ = oracle.ref_inverse_f32(A, mode)
    rp = oracle.residual(A, Xp)[:, 0]
    growth = oracle.lu_growth_bound(A, pp if perm is None else perm)
    return np.maximum(8.0 * n * U * growth, 2.0 * rp), rp


def check_pivoted_accuracy(oracle, A, X, mode):
    n = A.shape[-1]
    bound, rp = residual_bound(oracle, A, mode)
    rg = oracle.residual(A, X)[:, 0]
    bad = np.nonzero(~(rg <= bound))[0]
    assert bad.size == 0, f"{bad.size} matrices above tolerance, e.g. #{bad[:3]}: {rg[bad[:3]]} vs {bound[bad[:3]]}"
    assert np.median(rg) <= 2.0 * np.median(rp) + 8 * n * U


@pytest.mark.parametrize("n", range(1, 33))
@pytest.mark.parametrize("mode", ["reference", "reference_serial"])
def test_pivots_bit_exact_and_accuracy(mi_gpu, oracle, golden, n, mode):
    seed, count = golden[f"n{n}_uniform_seed"]
    A = oracle.uniform(int(seed), int(count), n)
    X, perm, info = gpu_inverse(mi_gpu, A, mode)
    key = "parallel" if mode == "reference" else "serial"
    assert np.array_equal(perm, golden[f"n{n}_uniform_piv_{key}"])
    # a larger seeded batch against the oracle replay
    B = oracle.uniform(1000 + n, 3000, n)
    Xb, pb, ib = gpu_inverse(mi_gpu, B, mode)
    assert np.array_equal(pb, oracle.pivots(B, mode))
    assert (ib == 0).all()
    check_pivoted_accuracy(oracle, B, Xb, mode)


@pytest.mark.parametrize("n", range(1, 33))
def test_ties_and_nan_golden(mi_gpu, oracle, golden, n):
    T = golden[f"n{n}_ties_A"].astype(np.float32)
    Z = golden[f"n{n}_nan_A"]
    for mode, key in (("reference", "parallel"), ("reference_serial", "serial")):
        _, pt, _ = gpu_inverse(mi_gpu, T, mode)
        assert np.array_equal(pt, golden[f"n{n}_ties_piv_{key}"]), mode
        _, pz, _ = gpu_inverse(mi_gpu, Z, mode)
        assert np.array_equal(pz, golden[f"n{n}_nan_piv_{key}"]), mode


def test_reference_fixtures(mi_gpu, golden):
    _, p, _ = gpu_inverse(mi_gpu, golden["literal4_A"], "reference")
    assert np.array_equal(p, golden["literal4_piv_parallel"])
    tmpl = golden["mtrand32_template"]
    for n in range(1, 33):
        M = tmpl[: n * n].reshape(1, n, n).copy()
        _, p, _ = gpu_inverse(mi_gpu, M, "reference")
        assert np.array_equal(p, golden[f"mtrand_n{n}_piv_parallel"]), n
        _, p, _ = gpu_inverse(mi_gpu, M, "reference_serial")
        assert np.array_equal(p, golden[f"mtrand_n{n}_piv_serial"]), n


@pytest.mark.parametrize("n", [3, 17, 32])
def test_subnormals_compare_as_zero(mi_gpu, oracle, n):
    # the reference is built with --use_fast_math: subnormal entries compare as 0
    A = oracle.uniform(4242, 64, n)
    A[:, :, 0] *= np.float32(1e-39)
    A[::2, 1:, 0] = np.float32(3e-39)
    _, p, _ = gpu_inverse(mi_gpu, A, "reference")
    assert np.array_equal(p, oracle.pivots(A, "reference"))


@pytest.mark.parametrize("n", [2, 5, 9, 12, 16, 20, 24, 28, 32])
def test_partial_pivoting(mi_gpu, oracle, n):
    A = oracle.uniform(300 + n, 2000, n)
    X, perm, info = gpu_inverse(mi_gpu, A, "partial")
    _, p64, _ = oracle.inverse_f64(A, "partial")
    agree = (perm == p64).all(1).mean()
    assert agree >= 0.99, agree   # differs only where FP32 rounding flips a near-tie
    for b in range(0, A.shape[0], 97):
        assert sorted(perm[b]) == list(range(n))
    rg = oracle.residual(A, X)[:, 0]
    bound, rp = residual_bound(oracle, A, "partial")
    assert np.all(rg <= bound)
    assert np.median(rg) <= 2.0 * np.median(rp) + 8 * n * U


def test_plain_small_config(mi_gpu, oracle, golden):
    # 1,000 FP32 32x32, uniform [-1, 1) from MT19937 seed 0, +32 on the diagonal
    A = oracle.uniform(0, 1000, 32) + np.float32(32.0) * np.eye(32, dtype=np.float32)
    X, perm, info = gpu_inverse(mi_gpu, A, "none")
    assert (info == 0).all()
    assert np.array_equal(perm, np.tile(np.arange(32, dtype=np.int32), (1000, 1)))
    X64, _, _ = oracle.inverse_f64(A, "none")
    res = oracle.residual(A, X)[:, 0]
    assert res.max() <= 1e-5
    err = np.abs(X - X64).max((1, 2)) / np.abs(X64).max((1, 2))
    assert err.max() <= 1e-5
    for n in (4, 17, 32):
        D, Xt = golden[f"n{n}_nopiv_A"], golden[f"n{n}_nopiv_X"]
        Xg, _, _ = gpu_inverse(mi_gpu, D, "none")
        assert np.abs(Xg - Xt).max() <= 1e-5 * max(1.0, np.abs(Xt).max())


@pytest.mark.parametrize("mode", ["reference", "partial", "none"])
def test_singular_info(mi_gpu, mode):
    n = 6
    A = np.zeros((3, n, n), dtype=np.float32)
    A[1] = np.eye(n)
    A[2] = np.eye(n)
    A[2, 4, 4] = 0.0           # zero row and column 4 -> fifth pivot is zero
    _, _, info = gpu_inverse(mi_gpu, A, mode)
    assert list(info) == [1, 0, 5]


@pytest.mark.parametrize("n", [1, 3, 8, 13, 32])
def test_ragged_and_tiny_batches(mi_gpu, oracle, n):
    import torch

    for batch in (1, 2, 3, 5, 7, 9, 33, 131):
        A = oracle.uniform(50 + batch, batch, n)
        X, perm, _ = gpu_inverse(mi_gpu, A, "reference")
        assert np.array_equal(perm, oracle.pivots(A, "reference"))
        Xs, _, _ = gpu_inverse(mi_gpu, A[batch // 2 : batch // 2 + 1], "reference")
        assert np.array_equal(Xs[0], X[batch // 2])     # alone == in the batch, bit for bit
    X, perm, info = mi_gpu.batched_inverse(torch.zeros((0, n, n), device="cuda"), "reference")
    assert X.shape == (0, n, n) and perm.shape == (0, n)
    M = torch.from_numpy(oracle.uniform(9, 1, n)[0]).cuda()
    X1, p1, i1 = mi_gpu.batched_inverse(M, "reference")
    assert X1.shape == (n, n) and p1.shape == (n,) and i1.shape == ()


def test_launch_knobs_do_not_change_results(mi_gpu, oracle):
    import torch

    n = 20
    A = oracle.uniform(61, 777, n)
    ref, _, _ = gpu_inverse(mi_gpu, A, "reference")
    for tpb in (32, 64, 96, 256):
        X, _, _ = gpu_inverse(mi_gpu, A, "reference", threads_per_block=tpb)
        assert np.array_equal(X, ref), tpb
    T = torch.from_numpy(A).cuda()
    mi_gpu.batched_inverse_(T, "reference", grid_blocks=1)
    assert np.array_equal(T.cpu().numpy(), ref)


def test_side_stream(mi_gpu, oracle):
    import torch

    n = 32
    A = oracle.uniform(62, 500, n)
    ref, _, _ = gpu_inverse(mi_gpu, A, "reference")
    s = torch.cuda.Stream()
    T = torch.from_numpy(A).cuda()
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        mi_gpu.batched_inverse_(T, "reference")
    s.synchronize()
    assert np.array_equal(T.cpu().numpy(), ref)


def test_full_size_batch_properties(mi_gpu, oracle):
    """n = 32, 1,000,000 matrices: pivots and residuals on a seeded sample,
    determinism, and alone-vs-batch equality."""
    import torch

    n, batch = 32, 1_000_000
    A = oracle.uniform(0, batch, n)
    dA = torch.from_numpy(A).cuda()
    X1, p1, i1 = mi_gpu.batched_inverse(dA, "reference")
    X2, p2, _ = mi_gpu.batched_inverse(dA, "reference")
    assert torch.equal(X1, X2) and torch.equal(p1, p2)
    idx = np.sort(np.random.RandomState(1).choice(batch, 1500, replace=False))
    idx = np.concatenate([idx, [0, batch - 1]])
    S = A[idx]
    Xs = X1[torch.from_numpy(idx).cuda()].cpu().numpy()
    ps = p1[torch.from_numpy(idx).cuda()].cpu().numpy()
    assert np.array_equal(ps, oracle.pivots(S, "reference"))
    check_pivoted_accuracy(oracle, S, Xs, "reference")
    Xa, _, _ = gpu_inverse(mi_gpu, S, "reference")
    assert np.array_equal(Xa, Xs)
    del dA, X1, X2
    torch.cuda.empty_cache()


def test_cublas_comparator_is_an_inverse(mi_gpu, oracle):
    import torch

    from matrixinversion_gb300 import cublas_ref

    A = oracle.uniform(71, 300, 16)
    (C, piv, info), (t1, t2) = cublas_ref.inverse(torch.from_numpy(A).cuda(), timed=True)
    X64, _, _ = oracle.inverse_f64(A, "partial")
    assert (info.cpu().numpy() == 0).all() and t1 > 0 and t2 > 0
    rel = np.abs(C.cpu().numpy() - X64).max((1, 2)) / np.abs(X64).max((1, 2))
    assert np.median(rel) < 1e-4


@pytest.mark.parametrize("n", [3, 5, 10, 13, 17, 25, 31])
@pytest.mark.parametrize("mode", ["none", "reference", "partial"])
def test_copy_paths_keep_neighbours_and_agree(mi_gpu, oracle, n, mode):
    """A batch placed inside a larger buffer: 16-byte-aligned starts take the
    windowed bulk copies (n not a multiple of 4), a 4-byte offset the plain
    copies.  Floats outside the batch must be untouched, and every copy path
    must give the same bits."""
    import torch

    sentinel = np.float32(12345.5)
    for batch in (1, 2, 3, 5, 17, 64, 129):
        A = oracle.uniform(70 + batch, batch, n)
        if mode == "none":
            A = A + np.float32(n) * np.eye(n, dtype=np.float32)
        results = []
        for off in (0, 4, 8, 1):
            total = off + batch * n * n + 11
            buf = torch.full((total,), float(sentinel), dtype=torch.float32, device="cuda")
            buf[off: off + batch * n * n] = torch.from_numpy(A.reshape(-1)).cuda()
            view = buf[off: off + batch * n * n].view(batch, n, n)
            mi_gpu.batched_inverse_(view, mode)
            torch.cuda.synchronize()
            h = buf.cpu().numpy()
            assert np.all(h[:off] == sentinel) and np.all(h[off + batch * n * n:] == sentinel), (batch, off)
            results.append(h[off: off + batch * n * n].copy())
        for r in results[1:]:
            assert np.array_equal(r, results[0]), batch
        X = results[0].reshape(batch, n, n)
        if mode != "none":          # per-matrix bound only: a median of a few matrices means nothing
            bound, _ = residual_bound(oracle, A, mode)
            assert np.all(oracle.residual(A, X)[:, 0] <= bound)
        else:
            assert np.all(oracle.residual(A, X)[:, 0] < 1e-5)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [11, 12, 15])
@pytest.mark.parametrize("mode", ["none", "reference", "partial"])
def test_small_and_large_batch_forms_agree(mi_gpu, n, mode):
    """n = 11..15 run the lane-group kernel below a batch of 12,288 matrices
    (4,096 in partial mode) and one thread per matrix above it; the same
    matrices give the same bits, pivots and info either way."""
    import torch

    g = torch.Generator(device="cuda").manual_seed(100 + n)
    big = torch.rand(20000, n, n, generator=g, device="cuda") * 2 - 1
    if mode == "none":
        big += n * torch.eye(n, device="cuda")
    big[5] = 0.0                                          # singular
    small = big[:2000].clone()
    Xb, Pb, Ib = mi_gpu.batched_inverse(big, mode)
    Xs, Ps, Is = mi_gpu.batched_inverse(small, mode)
    torch.cuda.synchronize()
    assert torch.equal(Xb[:2000].view(torch.int32), Xs.view(torch.int32))
    assert torch.equal(Pb[:2000], Ps) and torch.equal(Ib[:2000], Is)
    assert int(Is[5]) != 0
