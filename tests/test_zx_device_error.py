"""Waits that ran out on the device, read through the C ABI (mi_device_error).

Every wait of the kernels on a tile copy or a tensor-core product gives up
after about two seconds and records a flag instead of hanging.  The first test
checks the reading side: after normal work in every kernel family the flags
read 0, reading with and without clearing.  The second makes a wait run out
without any fault: through the test hook mi_set_wait_test the warps arm their
copy barrier with the bytes they expect but issue no copy, so the barrier never
completes and nothing is in flight; every warp's bounded wait (shortened to
10^5 clocks) gives up, the warps vote, record MI_DEVERR_COPY_TIMEOUT, wait once
more (bounded) and return.  The flag must read set, clear when cleared, and the
next normal call must give correct results with clear flags.  The file sorts
after the parity tests.
"""
import pytest

pytestmark = pytest.mark.gpu


def test_flags_stay_clear_after_normal_work(mi_gpu, oracle):
    import torch

    from matrixinversion_gb300 import refine

    for n, mode in ((32, "reference"), (17, "reference"), (12, "none"), (32, "partial"), (30, "partial"), (3, "reference")):
        A = torch.from_numpy(oracle.uniform(90 + n, 2048, n)).cuda()
        if mode == "none":
            A += n * torch.eye(n, device="cuda")
        mi_gpu.batched_inverse(A, mode)
    A = torch.from_numpy(oracle.uniform(99, 64, 32)).cuda()
    X, _, _ = mi_gpu.batched_inverse(A, "partial")
    refine.newton_schulz_(A, X, steps=1)
    torch.cuda.synchronize()
    assert mi_gpu.device_error(clear=False) == 0
    assert mi_gpu.device_error(clear=True) == 0
    assert mi_gpu.device_error(clear=False) == 0


@pytest.mark.parametrize("n", [32, 20, 18])
def test_wait_that_runs_out_is_reported_and_cleared(mi_gpu, oracle, n):
    import numpy as np
    import torch

    from matrixinversion_gb300 import _lib

    # n = 32: the eight-lane kernel (tensor copies); 20: the lane-group kernel
    # with tensor copies; 18: the lane-group kernel with windowed bulk copies
    L = _lib.load()
    A = oracle.uniform(123 + n, 256, n)
    dA = torch.from_numpy(A).cuda()
    assert mi_gpu.device_error(clear=True) == 0
    try:
        _lib.check(L.mi_set_wait_test(100_000, 1))
        mi_gpu.batched_inverse(dA, "reference")
        torch.cuda.synchronize()
    finally:
        _lib.check(L.mi_set_wait_test(0, 0))
    assert mi_gpu.device_error(clear=True) & _lib.MI_DEVERR_COPY_TIMEOUT
    assert mi_gpu.device_error(clear=False) == 0
    X, perm, info = mi_gpu.batched_inverse(dA, "reference")
    torch.cuda.synchronize()
    assert np.array_equal(perm.cpu().numpy(), oracle.pivots(A, "reference"))
    assert (info.cpu().numpy() == 0).all()
    r = oracle.residual(A, X.cpu().numpy())[:, 0]
    assert np.median(r) < 1e-3, np.median(r)
    assert mi_gpu.device_error(clear=False) == 0
