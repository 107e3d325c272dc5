import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "ref_kernels.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    if not os.path.exists(O.LIB_PATH):
        O.build()
    return O


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(GOLDEN))


@pytest.fixture(scope="session")
def mi_gpu():
    """The package with its CUDA library built and a device present."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device in this environment")
    import matrixinversion_gb300 as mi
    from matrixinversion_gb300 import build as B

    B.build()
    mi._lib.load()
    return mi
