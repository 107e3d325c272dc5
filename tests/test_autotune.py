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
    # below MI_LANES_ALT_MIN_BATCH every call runs at the default width, so
    # the tuner compares widths only from that batch up
    assert "lanes" not in table[(20, "reference")]
    X, _, _ = mi_gpu.batched_inverse(A, "reference")
    assert torch.equal(X, ref)
    autotune.set_config(20, "reference", 0)
    autotune.set_lanes(20, "reference", 0)


def test_fixed_block_sizes_are_reported_not_timed(lib):
    """Sizes whose contiguous launch has a fixed block are skipped without
    touching a device: nothing is timed or installed for them."""
    before = {(n, m): autotune.get_config(n, m) for n in (1, 8, 16) for m in ("none", "reference", "partial")}
    table = autotune.tune([1, 8], ["none", "reference"], batch=4096)
    assert table == {(n, m): {"best": 0, "ms": {}, "form": "thread"} for n in (1, 8) for m in ("none", "reference")}
    table = autotune.tune([16], ["partial"], batch=4096)
    assert table == {(16, "partial"): {"best": 0, "ms": {}, "form": "rows"}}
    assert {(n, m): autotune.get_config(n, m) for n in (1, 8, 16) for m in ("none", "reference", "partial")} == before


def test_lanes_per_matrix_knob(lib, tmp_path):
    """Sizes 17..31 without partial pivoting run at 16 or 8 lanes per matrix,
    every other (n, mode) at one width; the entry installs, restores, and
    round-trips through a saved table; mi_query_launch reports it."""
    import matrixinversion_gb300 as mi

    shipped, other = autotune.get_lanes(24, "reference")
    assert {shipped, other} == {8, 16}
    for lanes in (8, 16):
        autotune.set_lanes(24, "reference", lanes)
        assert autotune.get_lanes(24, "reference") == (lanes, 24 - lanes)
        assert mi.query_launch(24, "reference", 10**6)["lanes_per_matrix"] == lanes
    autotune.set_lanes(24, "reference", 0)
    assert autotune.get_lanes(24, "reference") == (shipped, other)
    assert autotune.get_lanes(12, "reference") == (8, 0)          # one width
    assert autotune.get_lanes(24, "partial")[1] == 0
    assert autotune.get_lanes(32, "reference")[1] == 0
    for bad in ((24, "reference", 4), (24, "reference", 32), (12, "reference", 16), (24, "partial", 8),
                (0, "none", 8), (33, "none", 8)):
        with pytest.raises(_lib.MatrixInversionError):
            autotune.set_lanes(*bad)
    table = {(24, "none"): {"best": 128, "ms": {128: 0.5}, "lanes": 8,
                            "ms_by_lanes": {8: {128: 0.5}, 16: {128: 0.6}}}}
    path = str(tmp_path / "t.json")
    autotune.save(table, path)
    assert autotune.load(path) == table
    assert autotune.get_lanes(24, "none")[0] == 8 and autotune.get_config(24, "none") == 128
    autotune.set_lanes(24, "none", 0)
    autotune.set_config(24, "none", 0)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [17, 24, 29, 31])
def test_both_widths_give_the_same_bits(mi_gpu, oracle, n):
    """16 and 8 lanes per matrix run the same arithmetic per element: a
    contiguous batch large enough to follow the entry (MI_LANES_ALT_MIN_BATCH
    matrices) gives the same inverse, pivots and info at either width in every
    non-partial mode, and so does a descriptor bucket of its first matrices
    (which runs at the default width); a smaller batch runs at the default
    width whatever the entry."""
    import torch

    import matrixinversion_gb300 as mi
    from matrixinversion_gb300 import descr

    big = _lib.MI_LANES_ALT_MIN_BATCH
    g = torch.Generator(device="cuda").manual_seed(700 + n)
    A = torch.rand(big, n, n, generator=g, device="cuda") * 2 - 1
    A[7] = 0.0                                                     # singular: info set
    for mode in ("none", "reference", "reference_serial"):
        M = A + n * torch.eye(n, device="cuda") if mode == "none" else A
        out = {}
        for lanes in (16, 8):
            autotune.set_lanes(n, mode, lanes)
            assert mi.query_launch(n, mode, big)["lanes_per_matrix"] == lanes
            assert mi.query_launch(n, mode, big - 1)["lanes_per_matrix"] == 16
            X, P, I = mi_gpu.batched_inverse(M, mode)
            out[lanes] = (X, P, I)
        autotune.set_lanes(n, mode, 0)
        (x16, p16, i16), (x8, p8, i8) = out[16], out[8]
        assert torch.equal(x16.view(torch.int32), x8.view(torch.int32)), (n, mode)
        assert torch.equal(p16, p8) and torch.equal(i16, i8)
        assert (int(i8[7]) != 0) == (mode != "none")             # + n I makes it regular without pivoting
        # a descriptor bucket of the first 300 matrices: the same bits
        head = [m for m in M[:300].cpu().numpy()]
        packed, offsets, ns = descr.pack(head)
        d = torch.from_numpy(packed).cuda()
        perm = torch.empty((len(head), 32), dtype=torch.int32, device="cuda")
        flags = torch.full((len(head),), _lib.PIVOT_MODES[mode], dtype=torch.int32, device="cuda")
        descr.batched_inverse_descr_(d, torch.from_numpy(offsets).cuda(), torch.from_numpy(ns).cuda(), flags,
                                     perm=perm)
        got = descr.unpack(d.cpu().numpy(), offsets, ns)
        x8h = x8[:300].cpu().numpy()
        assert all(np.array_equal(a.view(np.int32), x8h[i].view(np.int32)) for i, a in enumerate(got))
        assert np.array_equal(perm.cpu().numpy()[:, :n], p8[:300].cpu().numpy())


@pytest.mark.gpu
def test_tuning_compares_widths_from_the_batch_threshold(mi_gpu):
    """At MI_LANES_ALT_MIN_BATCH matrices the tuner times both widths of a
    size that has two and installs the faster, leaving the results unchanged."""
    import torch

    shipped = autotune.get_lanes(25, "none")[0]
    table = autotune.tune([25], ["none"], batch=_lib.MI_LANES_ALT_MIN_BATCH, iters=1, candidates=(256,))
    e = table[(25, "none")]
    assert e["lanes"] in (8, 16) and set(e["ms_by_lanes"]) == {8, 16}
    assert autotune.get_lanes(25, "none")[0] == e["lanes"]
    autotune.set_lanes(25, "none", 0)
    autotune.set_config(25, "none", 0)
    assert autotune.get_lanes(25, "none")[0] == shipped
