"""Launch-configuration table (CPU: the table itself) and the autotuner (GPU)."""
import json

import numpy as np
import pytest

from matrixinversion_gb300 import _lib, autotune


@pytest.fixture(scope="module")
def lib():
    from matrixinversion_gb300 import build

    build.build()
    return _lib.load()


def test_set_get_and_file_round_trip(lib, tmp_path):
    shipped = autotune.get_config(12, "reference")                # the table measured on GB300
    assert shipped in range(32, 257, 32)
    autotune.set_config(12, "reference", 64)
    assert autotune.get_config(12, "reference") == 64
    table = {(12, "reference"): {"best": 192, "ms": {64: 1.0, 192: 0.5}}}
    path = str(tmp_path / "t.json")
    autotune.save(table, path)
    assert json.load(open(path))[0]["best"] == 192
    assert autotune.load(path) == table
    assert autotune.get_config(12, "reference") == 192
    autotune.set_config(12, "reference", 0)                        # back to the shipped entry
    assert autotune.get_config(12, "reference") == shipped
    for bad in ((0, "none", 64), (33, "none", 64), (8, "none", 48), (8, "none", 288)):
        with pytest.raises(_lib.MatrixInversionError):
            autotune.set_config(*bad)


@pytest.mark.gpu
def test_tuning_installs_best_and_keeps_results(mi_gpu, oracle):
    import torch

    A = torch.from_numpy(oracle.uniform(4, 3000, 8)).cuda()
    ref, _, _ = mi_gpu.batched_inverse(A, "reference")
    table = autotune.tune([8], ["reference"], batch=4096, iters=2, candidates=(64, 256))
    best = table[(8, "reference")]["best"]
    assert best in (64, 256) and autotune.get_config(8, "reference") == best
    X, _, _ = mi_gpu.batched_inverse(A, "reference")
    assert torch.equal(X, ref)
    autotune.set_config(8, "reference", 0)
