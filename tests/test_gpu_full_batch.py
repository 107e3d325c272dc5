"""Pivot parity on whole 1,000,000-matrix batches.

The partial-pivoting sweep's configuration (entries uniform [-1, 1) from
MT19937 seed 0, no diagonal shift) at its full batch: every one of the
1,000,000 pivot vectors the kernels return must equal the oracle's replay of
the reference rule (bit-exact, comparisons only), at the sizes where the
reference tree drops slots (n = 6, 12, 24, 31) and at n = 32, the headline
size, for the parallel rule, plus the serial rule at n = 31 and 32.  The
inverses are checked on a 20,000-matrix sample with the per-matrix bound of
test_gpu_parity.
"""
import numpy as np
import pytest

from test_gpu_parity import check_pivoted_accuracy

pytestmark = pytest.mark.gpu

BATCH = 1_000_000
CASES = [(6, "reference"), (12, "reference"), (24, "reference"), (31, "reference"), (31, "reference_serial"),
         (32, "reference"), (32, "reference_serial")]
_BATCH_CACHE: dict = {}


def batch_of(oracle, n):
    if n not in _BATCH_CACHE:
        _BATCH_CACHE.clear()
        _BATCH_CACHE[n] = oracle.uniform(0, BATCH, n)
    return _BATCH_CACHE[n]


@pytest.mark.parametrize("n,mode", CASES)
def test_full_batch_pivots_bit_exact(mi_gpu, oracle, n, mode):
    import torch

    A = batch_of(oracle, n)
    dA = torch.from_numpy(A).cuda()
    perm = torch.empty((BATCH, n), dtype=torch.int32, device="cuda")
    info = torch.empty((BATCH,), dtype=torch.int32, device="cuda")
    mi_gpu.batched_inverse_(dA, mode, perm=perm, info=info)
    torch.cuda.synchronize()
    got = perm.cpu().numpy()
    want = oracle.pivots(A, mode)
    bad = np.nonzero((got != want).any(axis=1))[0]
    assert bad.size == 0, f"{bad.size} of {BATCH} pivot vectors differ, e.g. matrix {bad[:3]}"
    assert (info.cpu().numpy() == 0).all()
    idx = np.sort(np.random.RandomState(n).choice(BATCH, 20_000, replace=False))
    X = dA[torch.from_numpy(idx).cuda()].cpu().numpy()
    check_pivoted_accuracy(oracle, A[idx], X, mode)
