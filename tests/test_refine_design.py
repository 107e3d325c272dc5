"""The float-float refinement step, restated on the CPU.  CPU only.

mi_refine_df_kernel forms R = I - A X with each product split exactly
(p = a*x, e = fma(a, x, -p)) and summed by Knuth's TwoSum into a (hi, lo)
pair, rounds hi + lo + delta once, then X <- X + X R in FP32, and estimates
the error left as max|X R^2| / max|X|.  This restatement follows that
arithmetic operation for operation (FP32 rounding by numpy, exact products
in float64) on conditioned 32 x 32 matrices with FP32 LAPACK inverses, and
checks the design claims the refined form rests on:
  * the residual carries far more than FP32's 24 bits;
  * one step brings the error of an FP32 inverse from about kappa * u to the
    u level while kappa * u < 1;
  * a matrix the estimate does not list for a second step (estimate <= tol)
    has error <= tol + 5e-8;
  * the refined form (one step, a second one on the listed matrices) reaches
    1e-6 relative error in every kappa bucket up to 1e6.
"""
import numpy as np
import pytest

F = np.float32
TOL = 3e-7


def _exact_product_error(a, x, p):
    """fma(a, x, -p) for FP32 a, x and p = fl(a * x): exact in float64."""
    return (a.astype(np.float64) * x.astype(np.float64) - p.astype(np.float64)).astype(F)


def _two_sum(s, p):
    t = s + p
    z = t - s
    r = (s - (t - z)) + (p - z)
    return t, r


def _fma32(x, y, acc):
    """fma(x, y, acc) in FP32 (the product is exact in float64)."""
    return (x.astype(np.float64) * y.astype(np.float64) + acc.astype(np.float64)).astype(F)


def _df_step(A, X, tol=None):
    """One step of the kernel on a batch [B, n, n]; returns (X_new, listed)."""
    B, n, _ = A.shape
    s = np.zeros((B, n, n), F)
    c = np.zeros((B, n, n), F)
    for k in range(n):
        a = -A[:, :, k][:, :, None]                      # -A[i][k]
        x = X[:, k, :][:, None, :]                       # X[k][j]
        p = (a * x).astype(F)
        e = _exact_product_error(np.broadcast_to(a, p.shape), np.broadcast_to(x, p.shape), p)
        s, r = _two_sum(s, p)
        c = c + (r + e)
    d = np.broadcast_to(np.eye(n, dtype=F), s.shape)
    t, r = _two_sum(s, d)
    R = t + (c + r)
    acc = np.zeros((B, n, n), F)
    for k in range(n):
        acc = _fma32(X[:, :, k][:, :, None], R[:, k, :][:, None, :], acc)
    Xn = X + acc
    listed = None
    if tol is not None:
        e2 = np.zeros((B, n, n), F)
        for k in range(n):
            e2 = _fma32(acc[:, :, k][:, :, None], R[:, k, :][:, None, :], e2)
        emax = np.abs(e2).max(axis=(1, 2))
        xm = np.abs(X).max(axis=(1, 2))
        listed = np.isnan(e2).any(axis=(1, 2)) | ~(emax <= F(tol) * xm)
    return Xn, R, listed


def _rel_err(X, X64):
    return np.abs(X.astype(np.float64) - X64).max(axis=(1, 2)) / np.abs(X64).max(axis=(1, 2))


def _inv_fp32(A):
    """FP32 LAPACK inverses (sgetrf + sgetri, computed in single precision;
    numpy.linalg.inv would compute in double and round)."""
    lapack = pytest.importorskip("scipy.linalg.lapack")
    out = np.empty_like(A)
    for b in range(A.shape[0]):
        lu, piv, info = lapack.sgetrf(A[b])
        assert info == 0
        inv, info = lapack.sgetri(lu, piv)
        assert info == 0 and inv.dtype == np.float32
        out[b] = inv
    return out


@pytest.fixture(scope="module")
def buckets():
    from matrixinversion_gb300 import refine

    out = {}
    for kappa in (1e1, 1e3, 1e5, 1e6):
        A = refine.conditioned(192, kappa, n=32, seed=int(np.log10(kappa)), device="cpu").numpy()
        out[kappa] = (A, _inv_fp32(A), np.linalg.inv(A.astype(np.float64)))
    return out


def test_residual_carries_far_more_than_fp32(buckets):
    for kappa, (A, X0, _) in buckets.items():
        _, R, _ = _df_step(A, X0)
        exact = np.eye(32) - np.einsum("bik,bkj->bij", A.astype(np.float64), X0.astype(np.float64))
        # error of the rounded residual against the float64 one, relative to
        # the scale of the products summed, |A||X|
        scale = np.einsum("bik,bkj->bij", np.abs(A.astype(np.float64)), np.abs(X0.astype(np.float64))).max((1, 2))
        err = np.abs(R - exact).max((1, 2)) / scale
        # FP32 accumulation alone would leave about 2^-24 * 32 of the scale
        assert err.max() < 2.0 ** -36, (kappa, err.max())


def test_one_step_reaches_the_u_level_and_the_estimate_is_safe(buckets):
    for kappa, (A, X0, X64) in buckets.items():
        e0 = _rel_err(X0, X64)
        X1, _, listed = _df_step(A, X0, tol=TOL)
        e1 = _rel_err(X1, X64)
        if kappa <= 1e5:
            assert e1.max() < 0.05 * e0.max() + 2e-7, (kappa, e0.max(), e1.max())
        # every matrix left off the second-step list is within tol (+ rounding)
        assert np.all(e1[~listed] <= TOL + 5e-8), (kappa, e1[~listed].max())


def test_refined_form_meets_1e6_in_every_bucket(buckets):
    for kappa, (A, X0, X64) in buckets.items():
        X1, _, listed = _df_step(A, X0, tol=TOL)
        X2 = X1.copy()
        if listed.any():
            X2[listed], _, _ = _df_step(A[listed], X1[listed])
        e2 = _rel_err(X2, X64)
        assert e2.max() <= 1e-6, (kappa, e2.max(), int(listed.sum()))
