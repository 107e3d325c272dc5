"""Launch-configuration table (CPU: the table itself) and the autotuner (GPU)."""
import json

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


def test_skipped_pairs_round_trip_and_install_nothing(lib, tmp_path):
    shipped = autotune.get_config(8, "none")
    table = {(8, "none"): {"best": 0, "ms": {}, "form": "thread"},
             (20, "reference"): {"best": 64, "ms": {64: 1.0, 256: 1.5}}}
    path = str(tmp_path / "t.json")
    autotune.save(table, path)
    assert autotune.load(path) == table
    assert autotune.get_config(8, "none") == shipped              # a fixed-block pair installs nothing
    assert autotune.get_config(20, "reference") == 64
    autotune.set_config(20, "reference", 0)


@pytest.mark.gpu
def test_tuning_installs_best_and_keeps_results(mi_gpu, oracle):
    import torch

    # n = 20 with the reference rule runs the lane-group form, whose block
    # size is the knob; n = 8 runs one thread per matrix with a fixed block
    A = torch.from_numpy(oracle.uniform(4, 3000, 20)).cuda()
    ref, _, _ = mi_gpu.batched_inverse(A, "reference")
    shipped8 = autotune.get_config(8, "reference")
    table = autotune.tune([8, 20], ["reference"], batch=4096, iters=2, candidates=(64, 256))
    assert table[(8, "reference")] == {"best": 0, "ms": {}, "form": "thread"}
    assert autotune.get_config(8, "reference") == shipped8
    best = table[(20, "reference")]["best"]
    assert best in (64, 256) and autotune.get_config(20, "reference") == best
    X, _, _ = mi_gpu.batched_inverse(A, "reference")
    assert torch.equal(X, ref)
    autotune.set_config(20, "reference", 0)


def test_fixed_block_sizes_are_reported_not_timed(lib):
    """Sizes whose contiguous launch has a fixed block are skipped without
    touching a device: nothing is timed or installed for them."""
    before = {(n, m): autotune.get_config(n, m) for n in (1, 8, 16) for m in ("none", "reference", "partial")}
    table = autotune.tune([1, 8], ["none", "reference"], batch=4096)
    assert table == {(n, m): {"best": 0, "ms": {}, "form": "thread"} for n in (1, 8) for m in ("none", "reference")}
    table = autotune.tune([16], ["partial"], batch=4096)
    assert table == {(16, "partial"): {"best": 0, "ms": {}, "form": "rows"}}
    assert {(n, m): autotune.get_config(n, m) for n in (1, 8, 16) for m in ("none", "reference", "partial")} == before
