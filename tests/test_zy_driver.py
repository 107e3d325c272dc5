"""The command-line driver bin/mi_driver: the reference's per-run stdout
contract over the C ABI.

The reference's sweep script runs one binary per configuration and reads
"Kernel execution time: <ms> milliseconds" (parallel_pivot/
luBatchedInplace.cu:133, parsed at parallel_pivot/run.py:136-143) and the
"Correct inversions" / "Incorrect inversions" counts (parallel_pivot/
verify.hpp:101-102) from its stdout.  CPU tests: the driver builds, parses its
knobs (MATRIXSIZE / NUMMATRICES / NUMTHREADS or flags), rejects bad ones and
generates the workloads' inputs bit for bit.  GPU test: the lines parse as the
reference's script parses them, and the inverses equal the library's.
The file sorts after the parity tests and before the no-allocation test.
"""
import os
import subprocess

import numpy as np
import pytest


@pytest.fixture(scope="module")
def exe():
    from matrixinversion_gb300 import build

    build.build()
    return build.build_driver()


def run(exe, args, env=None, timeout=600):
    e = dict(os.environ)
    for k in ("MATRIXSIZE", "NUMMATRICES", "NUMTHREADS"):
        e.pop(k, None)
    e.update(env or {})
    return subprocess.run([exe, *args], env=e, capture_output=True, text=True, timeout=timeout)


def kernel_ms(stdout):
    """The runtime as the reference's sweep script reads it: the number after
    the colon of the first "Kernel execution time" line."""
    for line in stdout.splitlines():
        if "Kernel execution time" in line:
            return float(line.split(":", 1)[1].split()[0])
    raise AssertionError("no 'Kernel execution time' line:\n" + stdout)


def field(stdout, name):
    for line in stdout.splitlines():
        if line.startswith(name + ":"):
            return line.split(":", 1)[1].strip()
    raise AssertionError(f"no '{name}' line:\n" + stdout)


def test_usage(exe):
    r = run(exe, ["--help"])
    assert r.returncode == 0 and "MATRIXSIZE" in r.stdout and "NUMTHREADS" in r.stdout


@pytest.mark.parametrize("args,env", [
    (["--n", "33"], None), (["--n", "0"], None), (["--batch", "0"], None), (["--threads", "-1"], None),
    (["--pivot", "lapack"], None), (["--shift", "-1"], None), (["--bogus", "1"], None), (["--n"], None),
    ([], {"MATRIXSIZE": "40"}), ([], {"NUMMATRICES": "x"}), ([], {"NUMTHREADS": "2000"}),
])
def test_bad_knobs_exit_1_before_any_work(exe, args, env):
    r = run(exe, args, env)
    assert r.returncode == 1 and r.stderr.startswith("mi_driver: ") and r.stdout == ""


def _inputs(exe, tmp_path, args, env=None):
    path = tmp_path / "in.bin"
    r = run(exe, [*args, "--write-input", str(path), "--no-verify"], env)
    # on a host without a GPU the run stops at the first CUDA call, after the
    # input was written
    assert r.returncode == 0 or "CUDA error" in r.stderr, r.stderr
    return np.fromfile(path, dtype=np.float32), r


def test_seeded_inputs_are_the_workload_generators(exe, tmp_path):
    from matrixinversion_gb300 import data

    x, r = _inputs(exe, tmp_path, ["--seed", "3", "--pivot", "none"], {"MATRIXSIZE": "5", "NUMMATRICES": "7"})
    assert np.array_equal(x.reshape(7, 5, 5), data.diagonally_dominant(3, 7, 5))      # default shift n
    assert field(r.stdout, "Matrix size") == "5" and field(r.stdout, "Number of matrices") == "7"
    assert field(r.stdout, "Pivoting") == "none"
    x, _ = _inputs(exe, tmp_path, ["--n", "32", "--batch", "3"])                          # seed 0, no shift
    assert np.array_equal(x.reshape(3, 32, 32), data.uniform(0, 3, 32))
    x, _ = _inputs(exe, tmp_path, ["--n", "32", "--batch", "2", "--pivot", "none", "--shift", "32"])
    assert np.array_equal(x.reshape(2, 32, 32), data.diagonally_dominant(0, 2, 32, shift=32.0))


def test_file_template_is_replicated(exe, tmp_path):
    # the reference's input mode: the first n*n values of a text file
    vals = np.arange(1, 21, dtype=np.float32) / np.float32(7.0)
    src = tmp_path / "template.txt"
    src.write_text("\n".join(repr(float(v)) for v in vals) + "\n")
    x, _ = _inputs(exe, tmp_path, ["--n", "4", "--batch", "3", "--input", str(src)])
    assert np.array_equal(x.reshape(3, 4, 4), np.broadcast_to(vals[:16].reshape(4, 4), (3, 4, 4)))
    short = tmp_path / "short.txt"
    short.write_text("1 2 3\n")
    r = run(exe, ["--n", "2", "--input", str(short)])
    assert r.returncode == 1 and "fewer than n*n" in r.stderr


def test_reported_geometry_is_the_launch_query(exe):
    import matrixinversion_gb300 as mi

    for n, pivot, batch, threads in ((32, "reference", 1000, 0), (17, "partial", 100, 64), (12, "none", 20000, 96)):
        r = run(exe, ["--n", str(n), "--pivot", pivot, "--batch", str(batch), "--threads", str(threads),
                      "--no-verify"])
        q = mi.query_launch(n, pivot, batch, threads)
        assert int(field(r.stdout, "Number of threads per block")) == q["threads_per_block"]
        assert int(field(r.stdout, "Threads per matrix")) == q["lanes_per_matrix"]


@pytest.mark.gpu
def test_stdout_contract_and_results_equal_the_library(mi_gpu, exe, tmp_path):
    import torch

    from matrixinversion_gb300 import data

    # 1,000 FP32 32 x 32, seed 0, +32 on the diagonal, no pivoting
    out = tmp_path / "x.bin"
    r = run(exe, ["--pivot", "none", "--seed", "0", "--out", str(out)],
            {"MATRIXSIZE": "32", "NUMMATRICES": "1000", "NUMTHREADS": "128"})
    assert r.returncode == 0, r.stderr
    assert kernel_ms(r.stdout) > 0.0
    assert field(r.stdout, "Correct inversions") == "1000" and field(r.stdout, "Incorrect inversions") == "0"
    assert field(r.stdout, "Singular matrices") == "0"
    A = data.diagonally_dominant(0, 1000, 32)
    Xg, _, _ = mi_gpu.batched_inverse(torch.from_numpy(A).cuda(), "none")
    assert np.array_equal(np.fromfile(out, dtype=np.float32).reshape(1000, 32, 32), Xg.cpu().numpy())

    # reference rule at an odd size with an explicit NUMTHREADS
    r = run(exe, ["--n", "17", "--batch", "777", "--threads", "64", "--pivot", "reference", "--seed", "5",
                  "--out", str(out)])
    assert r.returncode == 0, r.stderr
    assert kernel_ms(r.stdout) > 0.0
    A = data.uniform(5, 777, 17)
    Xg, _, _ = mi_gpu.batched_inverse(torch.from_numpy(A).cuda(), "reference")
    X = np.fromfile(out, dtype=np.float32).reshape(777, 17, 17)
    assert np.array_equal(X, Xg.cpu().numpy())
    good = int(field(r.stdout, "Correct inversions"))
    assert good + int(field(r.stdout, "Incorrect inversions")) == 777
    R = np.abs(np.einsum("bij,bjk->bik", A.astype(np.float64), X.astype(np.float64)) - np.eye(17))
    expect = int((R < 1e-3).all(axis=(1, 2)).sum())
    assert abs(good - expect) <= 1, (good, expect)      # summation order may move a value at the threshold
