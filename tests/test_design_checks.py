"""CPU restatements of two design choices in the kernels (no GPU).

* The whole-row partial-pivoting kernel (csrc/mi_rows.cuh) picks each step's
  pivot with one maximum over 64-bit words key << 16 | (255 - logical row) << 8
  | slot, where it used two 32-bit maxima (the largest key, then the lowest
  logical row among the lanes holding it).  Both must pick the same winner on
  every input: ties of keys across lanes and within a lane, keys of zero (rows
  already placed, or exact zeros), and NaN keys (1, below every number).
* The single persistent descriptor launch (csrc/mi_descr_persist.cu) cuts
  every bucket into chunks of k groups (k = chunk_floats / (group matrices x
  n^2), clamped to 1..8) and hands chunk numbers out in the order of its plan;
  every group of every bucket inside the masks must be walked exactly once.
"""
import numpy as np


def rows_key(x):
    """|x| bits + 2; a NaN is 1 (never beats a number), as rows_key."""
    b = np.float32(x).view(np.uint32) & np.uint32(0x7FFFFFFF)
    return 1 if b > 0x7F800000 else int(b) + 2


def two_maxima(keys, lps, slots):
    """The two-step search: each lane's best (largest key, then lowest
    logical row), the group's largest key, then the best candidate among the
    lanes holding it; returns (255 - lp) << 8 | slot (0 for none)."""
    cands = []
    for lk, ll, ls in zip(keys, lps, slots):
        bk, bl, bs = 0, 255, 0
        for k, l, s in zip(lk, ll, ls):
            if k > bk or (k == bk and k != 0 and l < bl):
                bk, bl, bs = k, l, s
        cands.append((bk, bl, bs))
    mx = max(c[0] for c in cands)
    return max((((255 - bl) << 8) | bs) if (bk != 0 and bk == mx) else 0 for bk, bl, bs in cands)


def one_maximum(keys, lps, slots):
    best = 0
    for lk, ll, ls in zip(keys, lps, slots):
        for k, l, s in zip(lk, ll, ls):
            w = 0 if k == 0 else (k << 16) | ((255 - l) << 8) | s
            best = max(best, w)
    return best & 0xFFFF


def test_one_64bit_maximum_picks_the_two_step_winner():
    rng = np.random.RandomState(3)
    lanes, rows = 16, 2
    cases = 0
    for trial in range(4000):
        n = rng.randint(2, 33)
        # logical rows: a permutation of the slots (distinct, as in the kernel)
        lp = rng.permutation(lanes * rows)
        kind = trial % 4
        if kind == 0:        # uniform values
            vals = rng.uniform(-1, 1, size=lanes * rows).astype(np.float32)
        elif kind == 1:      # small integers: many equal keys across and within lanes
            vals = rng.randint(-2, 3, size=lanes * rows).astype(np.float32)
        elif kind == 2:      # zeros and a few NaNs
            vals = np.where(rng.rand(lanes * rows) < 0.6, 0.0, rng.uniform(-1, 1, lanes * rows)).astype(np.float32)
            vals[rng.rand(lanes * rows) < 0.1] = np.nan
        else:                # all rows placed or zero: no candidate at all
            vals = np.zeros(lanes * rows, dtype=np.float32)
        placed = rng.rand(lanes * rows) < 0.3
        keys = [0 if (placed[i] or i >= n) else rows_key(vals[i]) for i in range(lanes * rows)]
        # lane s owns slots s and s + 16 (rows = 2)
        lk = [[keys[s + lanes * r] for r in range(rows)] for s in range(lanes)]
        ll = [[int(lp[s + lanes * r]) for r in range(rows)] for s in range(lanes)]
        ls = [[s + lanes * r for r in range(rows)] for s in range(lanes)]
        assert one_maximum(lk, ll, ls) == two_maxima(lk, ll, ls), (trial, keys, lp)
        cases += 1
    assert cases == 4000


def plan(counts, n_mask, mode_mask, chunk_floats, max_groups=8):
    """The persistent launch's plan: per plan entry (n from 32 down, modes
    0..3) its bucket, groups per chunk and first chunk."""
    def lanes(n, mode):      # persist_lanes
        if mode != 3 and 17 <= n <= 31:
            return 8
        if mode == 3:
            return 4 if n <= 4 else (8 if n <= 8 else (16 if n <= 16 else 32))
        return 16 if n > 16 else (8 if n > 10 else 4)

    def group(n, mode):      # persist_group
        if n <= 14:
            return 32
        if n == 32 and mode != 3:
            return 4
        return 32 // lanes(n, mode)

    entries, first = [], [0]
    for i in range(128):
        b = (31 - i // 4) * 4 + (i & 3)
        n, mode = b // 4 + 1, b & 3
        on = (n_mask >> (n - 1)) & 1 and (mode_mask >> mode) & 1
        cnt = counts[b] if on else 0
        m = group(n, mode)
        groups = (cnt + m - 1) // m
        k = min(max(chunk_floats // (m * n * n), 1), max_groups)
        entries.append((b, k, groups))
        first.append(first[-1] + (groups + k - 1) // k)
    return entries, first


def test_persistent_plan_walks_every_group_once():
    rng = np.random.RandomState(8)
    for trial in range(200):
        counts = [int(c) for c in rng.randint(0, 3000, size=128) * (rng.rand(128) < 0.5)]
        n_mask = 0xFFFFFFFF if trial % 3 else int(rng.randint(1, 2**31))
        mode_mask = 0xF if trial % 5 else int(rng.randint(1, 16))
        chunk = int(rng.choice([1, 7, 4096, 16384, 1 << 22]))
        entries, first = plan(counts, n_mask, mode_mask, chunk)
        walked = {}
        i = 0
        for c in range(first[-1]):                  # chunk numbers in the order the counter hands them out
            while first[i + 1] <= c:
                i += 1
            b, k, groups = entries[i]
            g0 = (c - first[i]) * k
            g1 = min(g0 + k, groups)
            assert 0 <= g0 < g1 <= groups and g1 - g0 <= 8
            for g in range(g0, g1):
                assert (b, g) not in walked
                walked[(b, g)] = c
        for b, k, groups in entries:
            n, mode = b // 4 + 1, b & 3
            for g in range(groups):
                assert (b, g) in walked
        # buckets outside the masks are never walked
        for b in range(128):
            n, mode = b // 4 + 1, b & 3
            if not ((n_mask >> (n - 1)) & 1 and (mode_mask >> mode) & 1):
                assert all(key[0] != b for key in walked)
