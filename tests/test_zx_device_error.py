"""Waits that ran out on the device, read through the C ABI (mi_device_error).

Every wait of the kernels on a tile copy or a tensor-core product gives up
after about two seconds and records a flag instead of hanging; nothing here
makes a wait run out (a fault or a stalled copy engine is not something a test
may cause on a shared GPU).  The test checks the reading side: after normal
work in every kernel family the flags read 0, reading with and without
clearing.  The file sorts after the parity tests.
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
