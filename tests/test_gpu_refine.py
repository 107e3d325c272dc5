"""Newton-Schulz refinement on the tensor cores (mi_newton_schulz_f32).

Checked against the FP64 oracle (oracle.inverse_f64) on conditioned inputs:
  * one step equals the same step evaluated in FP64 from the same FP32 start,
    to within 3xTF32 accuracy: max |X1 - X1_64| <= 1e-4 * max |X1_64| at
    kappa = 1e1 and 1e3 (products carry ~2^-21 relative error, summed over 32
    terms and amplified by |X0| |A| |X0| <= kappa |X0|);
  * at kappa = 1e1 the refined inverse is FP32-accurate: max |X - X64| <=
    1e-5 * max |X64| for every matrix;
  * with an FP32-accurate residual a step cannot beat kappa * u, so on
    partial-pivoting inverses (already at that level) the median error stays
    within 1.5x of the plain one up to kappa = 1e3 (3x at 1e5, where the
    residual is mostly rounding noise); on inverses from the reference pivot rule
    (unstable, heavy-tailed) one step squares the error and two bring it
    down to the partial-pivoting level;
  * batch sizes not divisible by the 4-matrix tile leave the rest untouched;
  * the FP64 step on flagged matrices reaches FP32 accuracy at kappa = 1e5:
    max |X - X64| <= 1e-5 * max |X64| after one step (from ~1e-3 before),
    and leaves unlisted matrices unchanged.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(kappa, batch, seed):
    from matrixinversion_gb300 import refine

    return refine.conditioned(batch, kappa, seed=seed)


@pytest.mark.parametrize("kappa", [1e1, 1e3, 1e5])
def test_step_matches_fp64_step(mi_gpu, oracle, kappa):
    import torch

    from matrixinversion_gb300 import refine

    A = _inputs(kappa, 257, 5)
    X0, _, _ = mi_gpu.batched_inverse(A, "partial")
    X1 = X0.clone()
    refine.newton_schulz_(A, X1, steps=1)
    torch.cuda.synchronize()
    a = A.cpu().numpy().astype(np.float64)
    x0 = X0.cpu().numpy().astype(np.float64)
    x1_64 = x0 + x0 @ (np.eye(32) - a @ x0)
    x1 = X1.cpu().numpy().astype(np.float64)
    X64, _, _ = oracle.inverse_f64(A.cpu().numpy(), "partial")
    scale = np.abs(x1_64).max((1, 2))
    err_step = np.abs(x1 - x1_64).max((1, 2)) / scale
    if kappa <= 1e3:
        assert err_step.max() <= 1e-4, err_step.max()
    e0 = np.abs(x0 - X64).max((1, 2)) / np.abs(X64).max((1, 2))
    e1 = np.abs(x1 - X64).max((1, 2)) / np.abs(X64).max((1, 2))
    # at kappa = 1e5 the FP32 residual is mostly rounding noise: the step may
    # cost up to ~2x; the FP64 step (test below) is the remedy there
    assert np.median(e1) <= np.median(e0) * (1.5 if kappa <= 1e3 else 3.0) + 1e-7
    if kappa == 1e1:
        assert e1.max() <= 1e-5, e1.max()


def test_step_repairs_reference_rule_inverses(mi_gpu, oracle):
    import torch

    from matrixinversion_gb300 import refine

    A = _inputs(1e3, 1024, 13)
    X64, _, _ = oracle.inverse_f64(A.cpu().numpy(), "partial")
    Xr, _, _ = mi_gpu.batched_inverse(A, "reference")
    Xp, _, _ = mi_gpu.batched_inverse(A, "partial")
    X1 = Xr.clone()
    refine.newton_schulz_(A, X1, steps=1)
    torch.cuda.synchronize()

    def err(X):
        x = X.cpu().numpy().astype(np.float64)
        return np.abs(x - X64).max((1, 2)) / np.abs(X64).max((1, 2))

    X2 = Xr.clone()
    refine.newton_schulz_(A, X2, steps=2)
    torch.cuda.synchronize()
    er, ep, e1, e2 = err(Xr), err(Xp), err(X1), err(X2)
    assert er.max() > 4 * ep.max()                 # the reference rule's tail
    # one step squares the error (the worst matrix drops by orders of magnitude),
    # two reach the partial-pivoting level
    assert e1.max() <= er.max() / 4 and np.median(e1) <= 2 * np.median(ep)
    assert e2.max() <= 2 * ep.max()


def test_two_steps_and_ragged_batch(mi_gpu, oracle):
    import torch

    from matrixinversion_gb300 import refine

    for batch in (1, 3, 5, 6):
        A = _inputs(1e3, batch, 9)
        X0, _, _ = mi_gpu.batched_inverse(A, "partial")
        big = torch.zeros(batch + 2, 32, 32, device="cuda")
        big[:batch] = X0
        big[batch:] = 7.0
        Xv = X0.clone()
        refine.newton_schulz_(A, Xv, steps=2)
        Xs = X0.clone()
        refine.newton_schulz_(A, Xs, steps=1)
        refine.newton_schulz_(A, Xs, steps=1)
        torch.cuda.synchronize()
        # two fused steps == two single steps (same arithmetic)
        assert torch.equal(Xv, Xs), batch
        # a view that ends inside a larger buffer: the floats after it are untouched
        view = big[:batch]
        refine.newton_schulz_(A, view, steps=1)
        torch.cuda.synchronize()
        assert torch.all(big[batch:] == 7.0)


def test_argument_errors(mi_gpu):
    import torch

    from matrixinversion_gb300 import _lib

    L = _lib.load()
    A = torch.zeros(4, 32, 32, device="cuda")
    assert L.mi_newton_schulz_f32(A.data_ptr(), A.data_ptr(), 4, 16, 1, None) == _lib.MI_ERR_INVALID_VALUE
    assert L.mi_newton_schulz_f32(A.data_ptr(), A.data_ptr(), 4, 32, 0, None) == _lib.MI_ERR_INVALID_VALUE
    assert L.mi_newton_schulz_f32(A.data_ptr() + 4, A.data_ptr(), 4, 32, 1, None) == _lib.MI_ERR_MISALIGNED
    assert L.mi_newton_schulz_f32(None, A.data_ptr(), 4, 32, 1, None) == _lib.MI_ERR_NULL_POINTER


def test_fp64_step_on_flagged(mi_gpu, oracle):
    import torch

    from matrixinversion_gb300 import refine

    A = torch.cat([_inputs(1e1, 64, 21), _inputs(1e5, 64, 22)])
    X0, _, _ = mi_gpu.batched_inverse(A, "partial")
    idx = refine.flag_ill_conditioned(A, X0, threshold=1e4)
    flagged = set(idx.cpu().numpy().tolist())
    assert flagged >= set(range(64, 128)) and not (flagged & set(range(64)))
    X = X0.clone()
    refine.refine_fp64_(A, X, idx)
    torch.cuda.synchronize()
    X64, _, _ = oracle.inverse_f64(A.cpu().numpy(), "partial")
    x, x0 = X.cpu().numpy().astype(np.float64), X0.cpu().numpy().astype(np.float64)
    e = np.abs(x - X64).max((1, 2)) / np.abs(X64).max((1, 2))
    e0 = np.abs(x0 - X64).max((1, 2)) / np.abs(X64).max((1, 2))
    assert e[64:].max() <= 1e-5 and e0[64:].max() > 1e-4, (e[64:].max(), e0[64:].max())
    assert np.array_equal(x[:64], x0[:64])


def test_float_float_step_matches_fp64_step(mi_gpu, oracle):
    """The float-float residual step reaches the FP64 step's accuracy: at
    kappa = 1e5, max |X - X64| <= 2e-6 * max |X64| after one step from the plain
    inverse (FP64 step: same bound), <= 1e-6 after two."""
    import torch

    from matrixinversion_gb300 import refine

    A = _inputs(1e5, 256, 31)
    X0, _, _ = mi_gpu.batched_inverse(A, "partial")
    idx = torch.arange(A.shape[0], dtype=torch.int32, device="cuda")
    X64, _, _ = oracle.inverse_f64(A.cpu().numpy(), "partial")

    def err(X):
        x = X.cpu().numpy().astype(np.float64)
        return np.abs(x - X64).max((1, 2)) / np.abs(X64).max((1, 2))

    Xd = X0.clone()
    refine.refine_df_(A, Xd, idx)
    Xf = X0.clone()
    refine.refine_fp64_(A, Xf, idx)
    torch.cuda.synchronize()
    ed, ef, e0 = err(Xd), err(Xf), err(X0)
    assert e0.max() > 1e-4
    assert ed.max() <= 2e-6 and ef.max() <= 2e-6, (ed.max(), ef.max())
    refine.refine_df_(A, Xd, idx)
    torch.cuda.synchronize()
    assert err(Xd).max() <= 1e-6


def test_device_flag_list_matches_host_flags(mi_gpu):
    import torch

    from matrixinversion_gb300 import refine

    A = torch.cat([_inputs(1e1, 40, 41), _inputs(1e5, 40, 42)])
    X, _, _ = mi_gpu.batched_inverse(A, "partial")
    X[3] = float("nan")                                   # a non-finite inverse is flagged
    lst = refine.flag_list(A, X, threshold=1e4).cpu().numpy()
    want = set(refine.flag_ill_conditioned(A, X, threshold=1e4).cpu().numpy().tolist())
    assert set(int(v) for v in lst if v >= 0) == want
    assert all(v in (-1, b) for b, v in enumerate(lst))
    assert 3 in want and set(range(40, 80)) <= want


@pytest.mark.gpu
def test_second_step_estimate(mi_gpu, oracle):
    """mi_refine_df_next_f32: the step itself is bit-identical to
    mi_refine_df_f32; a matrix left off the second-step list has error
    <= tol + 1e-7 (the estimate max|X R^2| / max|X| is first-order, the step
    adds rounding of about u); skipped and non-finite entries behave; the
    list may be written over the index array."""
    import torch

    from matrixinversion_gb300 import refine

    tol = 3e-7
    A = torch.cat([_inputs(1e3, 64, 51), _inputs(1e5, 448, 52)])
    X0, _, _ = mi_gpu.batched_inverse(A, "partial")
    X0[7] = float("nan")
    batch = A.shape[0]
    idx = torch.arange(batch, dtype=torch.int32, device="cuda")
    idx[5] = -1                                           # skipped entries
    idx[9] = batch + 3
    X64, _, _ = oracle.inverse_f64(A.cpu().numpy(), "partial")

    Xa = X0.clone()
    refine.refine_df_(A, Xa, idx)
    Xb = X0.clone()
    nxt = refine.refine_df_(A, Xb, idx, next_tol=tol)
    Xc = X0.clone()
    lst = idx.clone()
    same = refine.refine_df_(A, Xc, lst, next_tol=tol, next_out=lst)
    torch.cuda.synchronize()
    assert same.data_ptr() == lst.data_ptr()
    assert torch.equal(Xa.view(torch.int32), Xb.view(torch.int32))
    assert torch.equal(Xb.view(torch.int32), Xc.view(torch.int32))
    nx, lc = nxt.cpu().numpy(), lst.cpu().numpy()
    assert np.array_equal(nx, lc)
    ix = idx.cpu().numpy()
    assert nx[5] == -1 and nx[9] == -1 and nx[7] == 7
    assert all(v in (-1, ix[t]) for t, v in enumerate(nx))
    x = Xb.cpu().numpy().astype(np.float64)
    err = np.abs(x - X64).max((1, 2)) / np.abs(X64).max((1, 2))
    keep = [b for b in range(batch) if b not in (5, 7, 9) and nx[b] == -1]
    assert len(keep) > batch // 2
    assert err[keep].max() <= tol + 1e-7, err[keep].max()
    assert all(nx[b] == -1 for b in range(64) if b != 7)  # kappa = 1e3: one step is enough


@pytest.mark.gpu
def test_refined_inverse_reaches_1e6(mi_gpu, oracle):
    """The refined form meets max |X - X64| <= 1e-6 max |X64| per matrix in
    every bucket up to kappa = 1e5, with no second step below kappa = 1e4."""
    import torch

    from matrixinversion_gb300 import refine

    for kappa, seed in ((3.0, 61), (1e1, 62), (1e3, 63), (1e5, 64)):
        A = _inputs(kappa, 256, seed)
        X, perm, info, first, second = refine.refined_inverse(A, lists=True)
        torch.cuda.synchronize()
        assert (info.cpu().numpy() == 0).all()
        X64, _, _ = oracle.inverse_f64(A.cpu().numpy(), "partial")
        x = X.cpu().numpy().astype(np.float64)
        err = np.abs(x - X64).max((1, 2)) / np.abs(X64).max((1, 2))
        assert err.max() <= 1e-6, (kappa, err.max())
        assert int((first >= 0).sum()) == 256
        if kappa < 1e4:
            assert int((second >= 0).sum()) == 0


@pytest.mark.gpu
@pytest.mark.parametrize("kappa", [1e1, 1e3, 1e5, 1e6])
def test_tensor_core_step_matches_its_restatement(mi_gpu, kappa):
    """mi_refine_tc_f32 against its CPU restatement (tests/test_refine_design.py):
    the digit groups are exact integers and the float-float combination runs in
    the same order, so R is the same bits; only the tensor core's summation
    order in C = X R differs, so X + C agrees to within 4 units in the last
    place of max|X|.  Out-of-range list entries leave their matrices as they
    were."""
    import torch

    from matrixinversion_gb300 import refine
    from test_refine_design import _tc_step

    A = _inputs(kappa, 96, 71)
    X0, _, _ = mi_gpu.batched_inverse(A, "partial")
    idx = torch.arange(A.shape[0], dtype=torch.int32, device="cuda")
    idx[10] = -1
    idx[20] = A.shape[0] + 7
    X1 = X0.clone()
    refine.refine_tc_(A, X1, idx)
    torch.cuda.synchronize()
    a, x0, x1 = A.cpu().numpy(), X0.cpu().numpy(), X1.cpu().numpy()
    want = _tc_step(a, x0)[0]
    assert np.array_equal(x1[10], x0[10]) and np.array_equal(x1[20], x0[20])
    live = [b for b in range(A.shape[0]) if b not in (10, 20)]
    diff = np.abs(x1[live].astype(np.float64) - want[live]).max((1, 2)) / np.abs(want[live]).max((1, 2))
    assert diff.max() <= 2.0 ** -22, diff.max()


@pytest.mark.gpu
def test_tensor_core_second_step_estimate(mi_gpu, oracle):
    """mi_refine_tc_next_f32: the step is bit-identical to mi_refine_tc_f32;
    a matrix left off the second-step list has error <= tol + 1e-7; skipped
    and non-finite entries behave; the list may overwrite the index array."""
    import torch

    from matrixinversion_gb300 import refine

    tol = 3e-7
    A = torch.cat([_inputs(1e3, 64, 81), _inputs(1e5, 448, 82)])
    X0, _, _ = mi_gpu.batched_inverse(A, "partial")
    X0[7] = float("nan")
    batch = A.shape[0]
    idx = torch.arange(batch, dtype=torch.int32, device="cuda")
    idx[5] = -1
    idx[9] = batch + 3
    X64, _, _ = oracle.inverse_f64(A.cpu().numpy(), "partial")
    Xa = X0.clone()
    refine.refine_tc_(A, Xa, idx)
    Xb = X0.clone()
    nxt = refine.refine_tc_(A, Xb, idx, next_tol=tol)
    Xc = X0.clone()
    lst = idx.clone()
    same = refine.refine_tc_(A, Xc, lst, next_tol=tol, next_out=lst)
    torch.cuda.synchronize()
    assert same.data_ptr() == lst.data_ptr()
    assert torch.equal(Xa.view(torch.int32), Xb.view(torch.int32))
    assert torch.equal(Xb.view(torch.int32), Xc.view(torch.int32))
    nx = nxt.cpu().numpy()
    assert np.array_equal(nx, lst.cpu().numpy())
    assert nx[5] == -1 and nx[9] == -1 and nx[7] == 7
    ix = idx.cpu().numpy()
    assert all(v in (-1, ix[t]) for t, v in enumerate(nx))
    x = Xb.cpu().numpy().astype(np.float64)
    err = np.abs(x - X64).max((1, 2)) / np.abs(X64).max((1, 2))
    keep = [b for b in range(batch) if b not in (5, 7, 9) and nx[b] == -1]
    assert len(keep) > batch // 2
    assert err[keep].max() <= tol + 1e-7, err[keep].max()
    assert all(nx[b] == -1 for b in range(64) if b != 7)


@pytest.mark.gpu
def test_refined_inverse_both_steps_reach_1e6_up_to_kappa_1e6(mi_gpu, oracle):
    """The refined form with either step -- the residual on the tensor cores
    (the default at n = 32) or in float-float on the FP32 pipes -- meets
    max |X - X64| <= 1e-6 max |X64| per matrix in every bucket up to
    kappa = 1e6."""
    import torch

    from matrixinversion_gb300 import refine

    for kappa, seed in ((1e1, 91), (1e4, 92), (1e6, 93)):
        A = _inputs(kappa, 256, seed)
        X64, _, _ = oracle.inverse_f64(A.cpu().numpy(), "partial")
        for step in ("tc", "df"):
            X, _, info = refine.refined_inverse(A, step=step)
            torch.cuda.synchronize()
            assert (info.cpu().numpy() == 0).all()
            x = X.cpu().numpy().astype(np.float64)
            err = np.abs(x - X64).max((1, 2)) / np.abs(X64).max((1, 2))
            assert err.max() <= 1e-6, (kappa, step, err.max())


@pytest.mark.gpu
def test_fused_flag_and_step_equals_flag_then_step(mi_gpu):
    """mi_refine_tc_flagged_f32 (flag and first step in one pass) gives the
    same bits and the same second-step list as mi_flag_condition_f32 followed
    by mi_refine_tc_next_f32, on a batch whose condition estimates sit far on
    either side of the threshold (kappa 10 below 1e4, kappa 1e5 above); a NaN
    inverse is flagged and listed; matrices below the threshold are left as
    they were."""
    import torch

    from matrixinversion_gb300 import refine

    A = torch.cat([_inputs(1e1, 96, 101), _inputs(1e5, 160, 102)])
    X0, _, _ = mi_gpu.batched_inverse(A, "partial")
    X0[100] = float("nan")
    thr, tol = 1e4, 3e-7
    Xa = X0.clone()
    lst = refine.flag_list(A, Xa, threshold=thr)
    nxt_a = refine.refine_tc_(A, Xa, lst, next_tol=tol)
    Xb = X0.clone()
    nxt_b = refine.refine_tc_flagged_(A, Xb, thr, tol)
    torch.cuda.synchronize()
    assert torch.equal(Xa.view(torch.int32), Xb.view(torch.int32))
    assert torch.equal(nxt_a, nxt_b)
    f = lst.cpu().numpy()
    assert (f[:96] == -1).all() and (f[96:] >= 0).all()
    assert torch.equal(Xb[:96].view(torch.int32), X0[:96].view(torch.int32))
    assert int(nxt_b[100]) == 100
