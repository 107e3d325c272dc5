"""Generate tests/golden/ref_kernels.npz from the reference's own kernel code.

Runs where the reference sources are present (its headers are compiled
unchanged against the host-thread CUDA stand-in in oracle/ref_emu and built
by oracle/Makefile).  The committed .npz is what the tests read; this script
only regenerates it:

    python tests/golden/make_golden.py REF_ROOT      (or MI_REF_ROOT=... in the environment)

Contents, for every n in 1..32:
  uniform inputs   : MT19937(seed) uniform [-1, 1) batches (regenerated by the
                     tests from the seed; a CRC of the bytes is stored to check
                     the regeneration), with the pivots[] arrays of
                     parallel_pivot and serial_pivot;
  tie-heavy inputs : small-integer matrices (many equal |entries|, so the
                     argmax tie rules decide), stored as int8, with both
                     kernels' pivots;
  NaN inputs       : uniform matrices with NaN planted on and off the
                     diagonal, with both kernels' pivots;
  no-pivot inputs  : uniform + n on the diagonal, with the templated kernel's
                     inverse (the only reference output that is race-free
                     when emulated on host threads).
Plus the reference's own fixtures: the 4x4 literal of
parallel_pivot/luBatchedInplace.cu:22 and the template matrix read from
parallel_pivot/mtrand32_new1.txt (luBatchedInplace.cu:44-53), with pivots
for every leading n x n block.
"""
from __future__ import annotations

import os
import subprocess
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

N_UNIFORM = 48
N_TIES = 12
SEED_BASE = 20250


def tie_matrices(rng: np.random.RandomState, count: int, n: int) -> np.ndarray:
    return rng.randint(-3, 4, size=(count, n, n)).astype(np.int8)


def main(ref_root: str | None = None) -> None:
    ref_root = ref_root or os.environ.get("MI_REF_ROOT")
    if not ref_root:
        raise SystemExit("usage: make_golden.py REF_ROOT (or set MI_REF_ROOT): the reference project's root")
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "all", f"REF_ROOT={ref_root}"], check=True)
    if not O.ref_available():
        raise SystemExit("reference emulation was not built")
    out = {}
    rng = np.random.RandomState(7)
    for n in range(1, 33):
        seed = SEED_BASE + n
        A = O.uniform(seed, N_UNIFORM, n)
        _, pp = O.ref_kernel_run("parallel_pivot", A)
        _, ps = O.ref_kernel_run("serial_pivot", A)
        out[f"n{n}_uniform_seed"] = np.array([seed, N_UNIFORM], dtype=np.int64)
        out[f"n{n}_uniform_crc"] = np.array([zlib.crc32(A.tobytes())], dtype=np.int64)
        out[f"n{n}_uniform_piv_parallel"] = pp.astype(np.int8)
        out[f"n{n}_uniform_piv_serial"] = ps.astype(np.int8)

        T = tie_matrices(rng, N_TIES, n)
        _, tp = O.ref_kernel_run("parallel_pivot", T.astype(np.float32))
        _, tsr = O.ref_kernel_run("serial_pivot", T.astype(np.float32))
        out[f"n{n}_ties_A"] = T
        out[f"n{n}_ties_piv_parallel"] = tp.astype(np.int8)
        out[f"n{n}_ties_piv_serial"] = tsr.astype(np.int8)

        Z = O.uniform(seed + 1000, 4, n)
        for b in range(4):
            i, j = rng.randint(0, n, size=2)
            Z[b, i, j] = np.nan
            if b % 2 == 0:
                k = rng.randint(0, n)
                Z[b, k, k] = np.nan
        _, zp = O.ref_kernel_run("parallel_pivot", Z)
        _, zs = O.ref_kernel_run("serial_pivot", Z)
        out[f"n{n}_nan_A"] = Z
        out[f"n{n}_nan_piv_parallel"] = zp.astype(np.int8)
        out[f"n{n}_nan_piv_serial"] = zs.astype(np.int8)

        D = O.uniform(seed + 2000, 4, n) + np.float32(n) * np.eye(n, dtype=np.float32)
        Xt, _ = O.ref_kernel_run("templated", D)
        out[f"n{n}_nopiv_A"] = D
        out[f"n{n}_nopiv_X"] = Xt
        print(f"n={n} done", flush=True)

    lit = np.array([4, 11, 3, 7, 4, 10, 4, 9, 2, 4, 2, 1, 7, 9, 18, 30], dtype=np.float32).reshape(1, 4, 4)
    _, lp = O.ref_kernel_run("parallel_pivot", lit)
    _, ls = O.ref_kernel_run("serial_pivot", lit)
    out["literal4_A"] = lit
    out["literal4_piv_parallel"] = lp.astype(np.int8)
    out["literal4_piv_serial"] = ls.astype(np.int8)

    with open(os.path.join(ref_root, "parallel_pivot", "mtrand32_new1.txt")) as f:
        tmpl = np.array([float(x) for x in f.read().split()[: 32 * 32]], dtype=np.float32)
    out["mtrand32_template"] = tmpl
    for n in range(1, 33):
        # the driver reads the first n*n values as the n x n template
        M = tmpl[: n * n].reshape(1, n, n).copy()
        _, mp = O.ref_kernel_run("parallel_pivot", M)
        _, ms = O.ref_kernel_run("serial_pivot", M)
        out[f"mtrand_n{n}_piv_parallel"] = mp.astype(np.int8)
        out[f"mtrand_n{n}_piv_serial"] = ms.astype(np.int8)

    path = os.path.join(HERE, "ref_kernels.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main(*sys.argv[1:])
