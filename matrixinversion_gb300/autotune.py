"""Launch autotuner for the reference's NUMTHREADS knob and lanes per matrix.

For each (n, pivot mode) it times the kernel at every candidate
threads-per-block value (matrices per block = threads / lanes per matrix) and,
where the size can run at two widths (n = 17..31 without partial pivoting:
16 or 8 lanes per matrix, mi_get_launch_lanes), at both widths, on a seeded
uniform batch, each launch on a fresh copy of the batch, and installs the
fastest pair with mi_set_launch_config and mi_set_launch_lanes.  Both entry points use the installed value whenever the
caller passes threads_per_block = 0: the contiguous call and the lane-group
buckets of a descriptor call.  Sizes whose contiguous launch at the tuning
batch has a fixed block (one thread per matrix, or whole rows per lane in
partial mode: mi_query_launch) are not timed -- the knob does not reach that
launch -- and are reported with ``best`` 0 and their form.  Tables can be
saved and loaded as JSON.

    python -m matrixinversion_gb300.autotune --n 2-32 --modes none,reference --out tuned.json
"""
from __future__ import annotations

import argparse
import ctypes
import json
import sys

from . import _lib

CANDIDATES = (32, 64, 96, 128, 160, 192, 224, 256)


def _time_one(n: int, mode: str, tpb: int, src, work, iters: int) -> float:
    import torch

    import matrixinversion_gb300 as mi

    times = []
    for it in range(iters + 1):
        work.copy_(src)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda._sleep(200_000)       # the host issues the launch while the device waits
        e0.record()
        mi.batched_inverse_(work, mode, threads_per_block=tpb)
        e1.record()
        torch.cuda.synchronize()
        if it > 0:
            times.append(e0.elapsed_time(e1))
    times.sort()
    return times[len(times) // 2]


def tune(ns=range(1, 33), modes=("none", "reference"), batch: int = 262144, iters: int = 5,
         candidates=CANDIDATES, install: bool = True, seed: int = 0) -> dict:
    """{(n, mode): {"best": tpb, "ms": {tpb: ms}}}, plus for pairs with two
    widths {"lanes": best width, "ms_by_lanes": {lanes: {tpb: ms}}} ("ms" is
    then the best width's row); installs the best values.

    Pairs the knob does not reach at `batch` get {"best": 0, "ms": {},
    "form": <form>} and nothing is installed for them."""
    import torch

    import matrixinversion_gb300 as mi

    table = {}
    g = None                          # made on the first size that is timed
    for n in ns:
        tunable = [m for m in modes if mi.query_launch(n, m, batch)["knob"]]
        for m in modes:
            if m not in tunable:
                table[(n, m)] = {"best": 0, "ms": {}, "form": mi.query_launch(n, m, batch)["form"]}
        if not tunable:
            continue
        if g is None:
            g = torch.Generator(device="cuda").manual_seed(seed)
        src = torch.rand(batch, n, n, generator=g, device="cuda") * 2 - 1
        work = torch.empty_like(src)
        for mode in tunable:
            s = src + n * torch.eye(n, device="cuda") if mode == "none" else src
            installed, other = get_lanes(n, mode)
            # below MI_LANES_ALT_MIN_BATCH every call runs at the default width
            widths = [installed] + ([other] if other and batch >= _lib.MI_LANES_ALT_MIN_BATCH else [])
            by_lanes = {}
            for lanes in widths:
                if len(widths) > 1:
                    set_lanes(n, mode, lanes)
                by_lanes[lanes] = {tpb: _time_one(n, mode, tpb, s, work, iters) for tpb in candidates}
            lanes, best = min(((l, t) for l in by_lanes for t in by_lanes[l]), key=lambda lt: by_lanes[lt[0]][lt[1]])
            entry = {"best": best, "ms": by_lanes[lanes]}
            if len(widths) > 1:
                entry.update(lanes=lanes, ms_by_lanes=by_lanes)
                set_lanes(n, mode, lanes if install else installed)
            table[(n, mode)] = entry
            if install:
                set_config(n, mode, best)
        del src, work
    return table


def set_config(n: int, mode: str, threads_per_block: int) -> None:
    _lib.check(_lib.load().mi_set_launch_config(int(n), _lib.PIVOT_MODES[mode], int(threads_per_block)))


def get_config(n: int, mode: str) -> int:
    v = ctypes.c_int(0)
    _lib.check(_lib.load().mi_get_launch_config(int(n), _lib.PIVOT_MODES[mode], ctypes.byref(v)))
    return v.value


def set_lanes(n: int, mode: str, lanes_per_matrix: int) -> None:
    """Install a width for (n, mode): its one width, its alternative, or 0
    for the shipped entry."""
    _lib.check(_lib.load().mi_set_launch_lanes(int(n), _lib.PIVOT_MODES[mode], int(lanes_per_matrix)))


def get_lanes(n: int, mode: str) -> tuple[int, int]:
    """(installed lanes per matrix, the other width the size can run at, or 0)."""
    v, alt = ctypes.c_int(0), ctypes.c_int(0)
    _lib.check(_lib.load().mi_get_launch_lanes(int(n), _lib.PIVOT_MODES[mode], ctypes.byref(v), ctypes.byref(alt)))
    return v.value, alt.value


def save(table: dict, path: str) -> None:
    def row(n, m, v):
        r = {"n": n, "mode": m, **v, "ms": {str(k): t for k, t in v["ms"].items()}}
        if "ms_by_lanes" in v:
            r["ms_by_lanes"] = {str(l): {str(k): t for k, t in ms.items()} for l, ms in v["ms_by_lanes"].items()}
        return r

    with open(path, "w") as f:
        json.dump([row(n, m, v) for (n, m), v in sorted(table.items())], f, indent=1)


def load(path: str, install: bool = True) -> dict:
    with open(path) as f:
        rows = json.load(f)
    table = {}
    for r in rows:
        v = {"best": r["best"], "ms": {int(k): t for k, t in r["ms"].items()}}
        if "form" in r:
            v["form"] = r["form"]
        if "lanes" in r:
            v["lanes"] = r["lanes"]
            v["ms_by_lanes"] = {int(l): {int(k): t for k, t in ms.items()} for l, ms in r["ms_by_lanes"].items()}
        table[(r["n"], r["mode"])] = v
    if install:
        for (n, m), v in table.items():
            if v["best"]:
                set_config(n, m, v["best"])
            if "lanes" in v:
                set_lanes(n, m, v["lanes"])
    return table


def main(argv=None):
    from .sweep import parse_range

    p = argparse.ArgumentParser()
    p.add_argument("--n", default="2-32")
    p.add_argument("--modes", default="none,reference")
    p.add_argument("--batch", type=int, default=262144)
    p.add_argument("--iters", type=int, default=5)
    p.add_argument("--out", default=None)
    a = p.parse_args(argv)
    table = tune(parse_range(a.n), a.modes.split(","), a.batch, a.iters)
    for (n, m), v in sorted(table.items()):
        if not v["best"]:
            print(json.dumps({"n": n, "mode": m, "fixed_block": v["form"]}), flush=True)
            continue
        line = {"n": n, "mode": m, "best": v["best"], "ms_best": round(v["ms"][v["best"]], 4),
                "ms_default": round(v["ms"].get(128, float("nan")), 4)}
        if "lanes" in v:
            line["lanes"] = v["lanes"]
            line["ms_best_by_lanes"] = {l: round(min(ms.values()), 4) for l, ms in v["ms_by_lanes"].items()}
        print(json.dumps(line), flush=True)
    if a.out:
        save(table, a.out)


if __name__ == "__main__":
    main(sys.argv[1:])
