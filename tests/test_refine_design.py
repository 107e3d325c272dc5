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


# ---------------------------------------------------------------------------
# The tensor-core step (mi_refine_tc_kernel), restated on the CPU: rows of A
# and columns of X scaled by powers of two to below 256 and cut into digits
# on the grids 2^(-8s) (round to nearest by adding and subtracting
# 1.5 * 2^(23 - 8s) in FP32, exact in bf16), digit-product groups d = s + t
# summed in the kernel's FP32 tensor-core accumulators (exactly for groups
# 0..2; groups 3 and up share one accumulator) and combined as the kernel
# does: TwoSum(G0, G1), then G2 and the rest added to the low part, scaled
# back, R rounded once; the correction C = X R from two-term bf16 splits of X
# and R.

DIGITS, LOW_GROUPS, DEEP_EXP = 6, 5, 16


def _bf16(x):
    """Round FP32 to bf16 (nearest, ties to even), returned as FP32."""
    u = np.ascontiguousarray(x, dtype=F).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(F)


def _line_exp(mx):
    """e with mx < 2^e (frexp's exponent; 0 for 0), clamped to [-100, 120]."""
    return np.clip(np.frexp(mx.astype(F))[1], -100, 120).astype(np.int64)


def _digits(M, inv_scale, ndig):
    v = (M * inv_scale).astype(F)                        # exact: powers of two
    out = []
    for s in range(ndig):
        c = F(1.5 * 2.0 ** (23 - 8 * s))
        q = ((v + c) - c).astype(F)                      # v rounded to a multiple of 2^(-8s)
        assert np.array_equal(_bf16(q), q)               # 8 significant bits at most
        out.append(q.astype(np.float64))
        v = (v - q).astype(F)                            # exact
    return out


def _tc_step(A, X, tol=None):
    B, n, _ = A.shape
    ea = _line_exp(np.abs(A).max(axis=2))                # [B, n] rows of A
    ex = _line_exp(np.abs(X).max(axis=1))                # [B, n] columns of X
    deep = ea.max(axis=1) + ex.max(axis=1) >= DEEP_EXP
    sa = np.ldexp(F(1), ea - 8).astype(F)[:, :, None]
    sx = np.ldexp(F(1), ex - 8).astype(F)[:, None, :]
    ad = _digits(A, np.ldexp(F(1), 8 - ea).astype(F)[:, :, None], DIGITS)
    xd = _digits(X, np.ldexp(F(1), 8 - ex).astype(F)[:, None, :], DIGITS)
    gmax = 0.0
    G = []
    for d in range(DIGITS):
        g = sum(np.einsum("bik,bkj->bij", ad[s], xd[d - s]) for s in range(d + 1))
        gmax = max(gmax, float(np.abs(g * 2.0 ** (8 * d)).max()))          # in units of the grid 2^(-8d)
        if d < 3:
            assert np.array_equal(g.astype(F).astype(np.float64), g)         # groups 0..2 exact in FP32
        if d >= LOW_GROUPS:
            g = np.where(deep[:, None, None], g, 0.0)
        G.append(g)
    # TwoSum(G0, G1) = hi + lo exactly; lo += G2; lo += the groups from 3 up,
    # which the kernel sums in one tensor-core accumulator (rounded here once
    # per group, the accumulator's order aside)
    hi, lo = _two_sum(G[0].astype(F), G[1].astype(F))
    lo = (lo + G[2].astype(F)).astype(F)
    tail = G[3].astype(F)
    for g in G[4:]:
        tail = (tail + g.astype(F)).astype(F)
    lo = (lo + tail).astype(F)
    s2 = (sa * sx).astype(F)
    R = ((np.eye(n, dtype=F) - (hi * s2).astype(F)) - (lo * s2).astype(F)).astype(F)
    rh = _bf16(R)
    rl = _bf16(R - rh)
    xh = _bf16(X)
    xl = _bf16(X - xh)
    f64 = lambda M: M.astype(np.float64)
    C = (np.einsum("bik,bkj->bij", f64(xh), f64(rh) + f64(rl))
         + np.einsum("bik,bkj->bij", f64(xl), f64(rh))).astype(F)
    Xn = (X + C).astype(F)
    listed = None
    if tol is not None:
        e2 = np.einsum("bik,bkj->bij", f64(_bf16(C)), f64(rh)).astype(F)
        listed = np.isnan(e2).any(axis=(1, 2)) | ~(np.abs(e2).max(axis=(1, 2)) <= F(tol) * np.abs(X).max(axis=(1, 2)))
    return Xn, R, listed, deep, gmax


def test_tc_groups_are_exact_and_the_residual_deep_enough(buckets):
    """Every digit-product group stays below 2^22 units of its grid (groups
    0..2, summed alone, are exact in FP32); the residual's error is below 2^-36
    of the |A||X| scale with groups 0..4 and below 2^-39 where the matrix takes
    group 5 (there the additions to the low part, G2 up to 2^6 units, round at
    about 2^-40 of the scale)."""
    for kappa, (A, X0, _) in buckets.items():
        _, R, _, deep, gmax = _tc_step(A, X0)
        assert gmax <= 2.0 ** 22                       # bound: 32 * (8 * 2^14) for group 5
        exact = np.eye(32) - np.einsum("bik,bkj->bij", A.astype(np.float64), X0.astype(np.float64))
        scale = np.einsum("bik,bkj->bij", np.abs(A.astype(np.float64)), np.abs(X0.astype(np.float64))).max((1, 2))
        err = np.abs(R - exact) - np.abs(exact) * 2.0 ** -24   # less R's own final rounding
        err = err.max((1, 2)) / scale
        assert err[~deep].max(initial=0) < 2.0 ** -36, (kappa, err[~deep].max(initial=0))
        assert err[deep].max(initial=0) < 2.0 ** -39, (kappa, err[deep].max(initial=0))
        if kappa >= 1e6:
            assert deep.mean() > 0.9
        if kappa <= 1e5:
            assert not deep.any()


def test_tc_step_reaches_the_u_level_and_its_estimate_is_safe(buckets):
    for kappa, (A, X0, X64) in buckets.items():
        e0 = _rel_err(X0, X64)
        X1, _, listed, _, _ = _tc_step(A, X0, tol=TOL)
        e1 = _rel_err(X1, X64)
        if kappa <= 1e5:
            assert e1.max() < 0.05 * e0.max() + 2e-7, (kappa, e0.max(), e1.max())
        assert np.all(e1[~listed] <= TOL + 5e-8), (kappa, e1[~listed].max())


def test_tc_refined_form_meets_1e6_in_every_bucket(buckets):
    for kappa, (A, X0, X64) in buckets.items():
        X1, _, listed, _, _ = _tc_step(A, X0, tol=TOL)
        X2 = X1.copy()
        if listed.any():
            X2[listed] = _tc_step(A[listed], X1[listed])[0]
        e2 = _rel_err(X2, X64)
        assert e2.max() <= 1e-6, (kappa, e2.max(), int(listed.sum()))


def test_pivot_growth_cannot_flag_ill_conditioning(buckets):
    """Why the refined form flags by the condition estimate ||A||_1 ||X||_1
    and not by pivot growth max|U| / max|A| (U from partial-pivoting LU, as
    the elimination forms it): with partial pivoting the growth stays O(1) in
    every kappa bucket -- the ill-conditioned buckets do not grow more -- so
    no growth threshold separates kappa = 1e1 (FP32 error ~1e-6) from
    kappa = 1e6 (~1e-2); the estimate tracks kappa within a small factor."""
    sl = pytest.importorskip("scipy.linalg")
    growth, est = {}, {}
    for kappa, (A, X0, _) in buckets.items():
        g = []
        for b in range(64):
            _, _, U = sl.lu(A[b].astype(np.float64))
            g.append(np.abs(U).max() / np.abs(A[b]).max())
        growth[kappa] = np.array(g)
        est[kappa] = np.abs(A).sum(1).max(1) * np.abs(X0).sum(1).max(1)
    assert growth[1e6].max() < growth[1e1].max() and growth[1e6].min() < 1.0 < growth[1e1].max()
    for kappa, e in est.items():
        assert np.all(e >= kappa) and np.all(e <= 64 * kappa), (kappa, e.min(), e.max())
