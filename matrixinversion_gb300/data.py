"""Seeded synthetic inputs of the benchmark workloads (no datasets involved).

uniform(seed, batch, n): i.i.d. uniform [-1, 1) FP32 entries from one
MT19937 stream seeded with `seed` (std::mt19937 seeding), each 32-bit draw u
mapped to ((u >> 8) - 2^23) * 2^-23, row-major matrices back to back.  The
reference's own driver replicates one text-file matrix
(parallel_pivot/luBatchedInplace.cu:44-53, 89-101); per-matrix seeded data
replaces it here.
"""
from __future__ import annotations

import numpy as np


def uniform(seed: int, batch: int, n: int) -> np.ndarray:
    u = np.random.RandomState(seed & 0xFFFFFFFF).randint(0, 2**32, size=batch * n * n, dtype=np.uint32)
    x = ((u >> np.uint32(8)).astype(np.int32) - np.int32(1 << 23)).astype(np.float32)
    x *= np.float32(2.0**-23)
    return x.reshape(batch, n, n)


def diagonally_dominant(seed: int, batch: int, n: int, shift: float | None = None) -> np.ndarray:
    """uniform() plus `shift` (default n) on the diagonal: the no-pivot workload."""
    A = uniform(seed, batch, n)
    A += np.float32(n if shift is None else shift) * np.eye(n, dtype=np.float32)
    return A
