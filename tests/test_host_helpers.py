"""Host-side helpers of the workloads and the descriptor batch.  CPU only.

Descriptor packing and masks, the sweep's range syntax (MATRIXSIZE /
NUMMATRICES values such as "2-32" or "1000,1000000"), the seeded input
generators against the oracle's MT19937 stream, and the precision workload's
condition numbers.
"""
import numpy as np
import pytest


def test_pack_unpack_round_trip_and_alignment():
    from matrixinversion_gb300 import descr, data

    rng = np.random.RandomState(3)
    ns = [int(n) for n in rng.randint(1, 33, size=200)]
    mats = [data.uniform(100 + i, 1, n)[0] for i, n in enumerate(ns)]
    for align in (1, 4, 8):
        packed, offsets, got_ns = descr.pack(mats, align=align)
        assert packed.dtype == np.float32 and offsets.dtype == np.int64 and got_ns.dtype == np.int32
        assert list(got_ns) == ns
        assert np.all(offsets % align == 0)
        ends = offsets + got_ns.astype(np.int64) ** 2
        assert np.all(offsets[1:] >= ends[:-1])                 # no overlap, in order
        assert ends[-1] <= packed.size
        for a, b in zip(mats, descr.unpack(packed, offsets, got_ns)):
            assert np.array_equal(a, b)
        if align == 1:
            assert packed.size == sum(n * n for n in ns)          # densely packed
    packed, offsets, got_ns = descr.pack([])
    assert packed.size == 1 and offsets.size == 0 and got_ns.size == 0


def test_masks_cover_exactly_the_sizes_and_modes_present():
    from matrixinversion_gb300 import descr

    n_mask, mode_mask = descr.masks([1, 5, 5, 32], [0, 3, 3, 0])
    assert n_mask == (1 << 0) | (1 << 4) | (1 << 31)
    assert mode_mask == 0b1001
    # malformed entries (the kernel reports them through info = -1) add no bits
    assert descr.masks([0, 33, 7], [4, -1, 2]) == (1 << 6, 1 << 2)


def test_parse_range():
    from matrixinversion_gb300.sweep import parse_range

    assert parse_range("2-5") == [2, 3, 4, 5]
    assert parse_range("32") == [32]
    assert parse_range("2-4,8,16-17") == [2, 3, 4, 8, 16, 17]
    assert parse_range("1000,1000000") == [1000, 1000000]


@pytest.mark.parametrize("n", [1, 7, 32])
def test_generators_match_the_oracle_stream(oracle, n):
    from matrixinversion_gb300 import data

    A = data.uniform(11, 50, n)
    assert A.dtype == np.float32 and A.shape == (50, n, n)
    assert np.array_equal(A, oracle.uniform(11, 50, n))
    assert A.min() >= -1.0 and A.max() < 1.0
    # 2^-23 grid of [-1, 1): every value is an integer multiple of 2^-23
    assert np.array_equal(np.round(A * 2.0**23), A * 2.0**23)
    D = data.diagonally_dominant(11, 50, n)
    assert np.array_equal(D, A + np.float32(n) * np.eye(n, dtype=np.float32))    # FP32 sum, as generated
    D32 = data.diagonally_dominant(0, 3, n, shift=32.0)
    assert np.array_equal(D32, data.uniform(0, 3, n) + np.float32(32.0) * np.eye(n, dtype=np.float32))
    off = ~np.eye(n, dtype=bool)
    assert np.array_equal(D32[:, off], data.uniform(0, 3, n)[:, off])


@pytest.mark.parametrize("kappa", [1e1, 1e3, 1e5])
def test_conditioned_matrices_hit_their_bucket(kappa):
    from matrixinversion_gb300 import refine

    A = refine.conditioned(8, kappa, n=32, seed=5, device="cpu").double().numpy()
    c = np.linalg.cond(A)
    # the FP32 rounding of A moves the smallest singular value by ~kappa * 2^-24
    assert np.all(np.abs(c / kappa - 1.0) < 0.01 + kappa * 2.0**-24 * 8), c


def test_rel_error_is_max_abs_over_max_abs():
    import torch

    from matrixinversion_gb300 import refine

    X64 = torch.tensor([[[2.0, -4.0], [1.0, 0.5]]], dtype=torch.float64)
    X = (X64 + torch.tensor([[[0.0, 0.0], [0.1, 0.0]]], dtype=torch.float64)).float()
    r = refine.rel_error(X, X64)
    assert r.shape == (1,) and abs(float(r[0]) - 0.1 / 4.0) < 1e-7


def test_clock_summary_reads_nvidia_smi_rows(tmp_path):
    """The bench's clock record: median SM clock over the loaded samples and
    every throttle reason seen Active (the rows nvidia-smi prints with
    --format=csv,noheader,nounits)."""
    import bench

    rows = ["0, 345, 2070, 110.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"] * 3
    rows += [f"0, {mhz}, 2070, 1200.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"
             for mhz in (1965, 1980, 2010)]
    rows += ["0, 1500, 2070, 1390.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
             "0, [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A]"]
    cs = bench.ClockSampler(0)
    cs.file = open(tmp_path / "clocks.csv", "w+")
    cs.file.write("\n".join(rows) + "\n")
    s = cs.summary()
    assert s["sm_max_mhz"] == 2070.0 and s["samples"] == len(rows)
    assert s["sm_mhz"] == 1980.0                       # idle samples below half the peak are left out
    assert s["reasons"] == ["sw_power_cap"]


def test_reference_arm_line(capsys):
    """bench.py --impl reference: the oracle's port of the reference algorithm
    on the host cores, one JSON line with the contract's keys."""
    import argparse
    import json

    import bench

    args = argparse.Namespace(gpus=1, steps=1, warmup=0, impl="reference", n=8, batch=1000, pivot="reference",
                              seed=0, no_e2e=True, no_cpu=False)
    bench.run_reference_arm(args, rank=0)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "matrices/s" and line["value"] > 0
    assert line["metric"] == bench.METRIC and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "matrices/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["n"] == 8 and line["config"]["pivot"] == "reference"
    bench.run_reference_arm(args, rank=1)              # other ranks print nothing
    assert capsys.readouterr().out == ""
    assert bench.algorithmic_bytes(32) == 8324


def test_wrappers_reject_host_tensors_before_any_call():
    """The refinement and descriptor wrappers take device tensors only: a host
    tensor is an error before the library is called (there is no host path)."""
    import torch

    from matrixinversion_gb300 import descr, refine

    A = torch.zeros(2, 32, 32)
    idx = torch.zeros(2, dtype=torch.int32)
    for call in (lambda: refine.newton_schulz_(A, A.clone()), lambda: refine.refine_fp64_(A, A.clone(), idx),
                 lambda: refine.refine_df_(A, A.clone(), idx), lambda: refine.flag_list(A, A.clone()),
                 lambda: descr.batched_inverse_descr_(torch.zeros(16), torch.zeros(1, dtype=torch.int64),
                                                      torch.ones(1, dtype=torch.int32),
                                                      torch.ones(1, dtype=torch.int32))):
        with pytest.raises(TypeError):
            call()


def test_residual_reports():
    """The sweep's residual statistics and the serving loop's residual check,
    on host tensors: exact inverses give ~0, a perturbed one is counted."""
    import torch

    from matrixinversion_gb300 import serving, sweep

    A = torch.from_numpy(np.linalg.qr(np.random.RandomState(4).randn(64, 8, 8))[0]).float()  # orthogonal
    X = A.transpose(1, 2).contiguous()
    X[5, 0, 0] += 0.01                                   # one matrix off by 1e-2 in one entry
    st = sweep.residual_stats(A, X, sample=64)
    assert st["median"] < 1e-5 and st["max"] > 5e-3
    assert abs(st["fail_1e-3"] - 1 / 64) < 1e-9           # verifyInv's criterion fails for exactly one
    r = serving.residual_max(A.numpy(), X.numpy())
    assert abs(r - st["max"]) < 1e-6


def test_condition_flags_on_host_tensors():
    """flag_ill_conditioned: ||A||_1 ||X||_1 >= threshold, or not finite."""
    import torch

    from matrixinversion_gb300 import refine

    A = torch.eye(4).repeat(3, 1, 1)
    X = torch.eye(4).repeat(3, 1, 1)
    X[1] *= 1e5                                          # estimate 1e5
    X[2, 0, 0] = float("nan")                            # not finite
    idx = refine.flag_ill_conditioned(A, X, threshold=1e4)
    assert idx.dtype == torch.int32 and idx.tolist() == [1, 2]
    assert refine.flag_ill_conditioned(A, X, threshold=1e6).tolist() == [2]
