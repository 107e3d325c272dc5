"""Benchmark: batched FP32 inverse, n = 32, batch 1,000,000, reference pivoting.

One step = one in-place pass of the sm_103a kernel over a batch of 1,000,000
seeded 32 x 32 matrices (uniform [-1, 1), MT19937 seed 0) with the
reference's parallel-argmax pivot rule -- the partial-pivoting sweep's n = 32
point, which carries the headline metric.  Each timed step works on its own
4.2 GB copy of the batch (inputs far larger than L2, no re-use between steps).

Prints one JSON line (rank 0):
  value      matrices/s of the kernel, inputs resident in HBM;
  e2e        matrices/s through HostPipeline (pinned host buffers, chunked
             H2D -> kernel -> D2H on three streams), copies inside the timing;
  roofline   achieved algorithmic GB/s of the kernel (8n^2 + 4n + 4 bytes per
             matrix: A in, A^-1 out, pivots, info) vs the measured HBM peak;
  cpu_baseline  the reference algorithm (FP32 Doolittle LU + comp_inv,
             restated in C) on all host cores over a bounded sample.
--impl reference times that CPU implementation alone (the reference has no
CPU path of its own; its kernels are GPU-only).
Under torchrun each rank inverts its own batch (weak scaling, no collective
on the data path; a barrier and a max-reduction of the timings only).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "matrices/s at n=32,1M batch (% HBM roofline) vs plain; p99 serve latency @same err"
UNIT = "matrices/s"
FALLBACK_HBM_GBS = 6800.0


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=40)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--n", type=int, default=32)
    p.add_argument("--batch", type=int, default=1_000_000)
    p.add_argument("--pivot", default="reference", choices=["reference", "reference_serial", "partial", "none"])
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    return p.parse_args()


def algorithmic_bytes(n: int) -> int:
    return 8 * n * n + 4 * n + 4


def hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic_per_matrix(n: int, pivot: str):
    """DRAM bytes per matrix from the committed ncu summary, if one covers this case."""
    path = os.path.join(ROOT, "profiles", f"mi_inverse_n{n}_{pivot}.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_matrix:"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 20 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def __enter__(self):
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        self.file.flush()

    def summary(self):
        self.file.seek(0)
        rows = [r.split(",") for r in self.file.read().strip().splitlines() if r.strip()]
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = sorted(float(r[1]) for r in rows if len(r) > 2 and r[1].strip().replace(".", "").isdigit())
        mx = max((float(r[2]) for r in rows if len(r) > 2 and r[2].strip().replace(".", "").isdigit()), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = []
        for k, name in enumerate(names):
            if any(len(r) > 5 + k and r[5 + k].strip() == "Active" for r in rows):
                reasons.append(name)
        # the load region only: samples taken while the SM clock was above idle
        load = [v for v in sm if sm and v >= 0.5 * sm[-1]]
        med = load[len(load) // 2] if load else None
        return {"sm_mhz": med, "sm_max_mhz": mx, "reasons": reasons, "samples": len(rows)}


def cpu_baseline(n: int, pivot: str, seed: int, budget_s: float = 12.0):
    """The reference algorithm on all host cores over a bounded sample."""
    import numpy as np

    from matrixinversion_gb300 import data
    from oracle import oracle as O

    threads = O.num_threads()
    probe = data.uniform(seed + 1, 4096, n)
    t0 = time.perf_counter()
    O.ref_inverse_f32(probe, pivot)
    rate = probe.shape[0] / max(time.perf_counter() - t0, 1e-9)
    count = int(min(1_000_000, max(4096, rate * budget_s)))
    A = data.uniform(seed, count, n)
    t0 = time.perf_counter()
    X, perm, info = O.ref_inverse_f32(A, pivot)
    dt = time.perf_counter() - t0
    del X, perm, info, A, np
    return {"value": count / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {count} matrices of the workload (n={n}, {pivot} pivoting), {dt:.1f} s on {threads} threads"}


def run_reference_arm(args, rank: int):
    if rank != 0:
        return
    from matrixinversion_gb300 import data
    from oracle import oracle as O

    O.build()
    threads = O.num_threads()
    per_step = 20_000
    A = data.uniform(args.seed, per_step, args.n)
    for _ in range(args.warmup):
        O.ref_inverse_f32(A[:2000], args.pivot)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.ref_inverse_f32(A, args.pivot)
    dt = time.perf_counter() - t0
    value = per_step * args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args, args.batch),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"first {per_step} matrices of the workload per step, on {threads} threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(args, batch):
    return {
        "workload": f"batched FP32 inverse, n={args.n}, batch={batch}, pivot={args.pivot}, "
                    f"uniform[-1,1) MT19937 seed {args.seed}",
        "n": args.n, "batch": batch, "pivot": args.pivot,
        "l2": "inputs larger than L2 (a separate copy of the batch per timed step)",
        "parallelism": f"batch shards x{args.gpus}",
    }


def main():
    args = parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference_arm(args, rank)
        return

    import numpy as np
    import torch

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    import matrixinversion_gb300 as mi
    from matrixinversion_gb300 import build as B
    from matrixinversion_gb300 import data
    from matrixinversion_gb300 import shards
    from matrixinversion_gb300.host import HostPipeline

    if rank == 0 or not os.path.exists(B.LIB):
        B.build()
    if world > 1:
        torch.distributed.barrier()
    mi._lib.load()

    n, batch = args.n, args.batch
    host = data.uniform(shards.shard_seed(args.seed, rank), batch, n)
    if args.pivot == "none":
        host += np.float32(n) * np.eye(n, dtype=np.float32)
    src = torch.from_numpy(host).to(dev)
    free = torch.cuda.mem_get_info(dev)[0]
    # one pristine copy of the batch per timed step, up to 60% of free HBM;
    # past that, buffers are reused (a reused buffer holds the last inverse)
    nbuf = max(1, min(args.steps, int(0.6 * free // (src.numel() * 4)) - 1))
    bufs = [src.clone() for _ in range(nbuf)]
    perm = torch.empty((batch, n), dtype=torch.int32, device=dev)
    info = torch.empty((batch,), dtype=torch.int32, device=dev)

    for i in range(args.warmup):
        w = src.clone()
        mi.batched_inverse_(w, args.pivot, perm=perm, info=info)
        del w
    barrier()

    stream = torch.cuda.current_stream(dev)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clocks:
        barrier()
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        t_start.record(stream)
        for i in range(args.steps):
            ev[i][0].record(stream)
            mi.batched_inverse_(bufs[i % nbuf], args.pivot, perm=perm, info=info)
            ev[i][1].record(stream)
        t_end.record(stream)
        barrier()
    total_ms = t_start.elapsed_time(t_end)
    launch_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = shards.max_over_ranks(total_ms, device=dev)
    value = shards.aggregate_rate(batch * args.steps, total_ms / 1e3, world)
    # the freed batch copies stay in torch's cache: handing some 170 GB back to
    # the driver here made the next host-pipeline step take about 200 ms
    del bufs

    # end to end through the host-buffer pipeline
    e2e = None
    e2e_launches = 0
    if not args.no_e2e:
        pipe = HostPipeline(n, chunk=65536, streams=4, device=dev)
        hA = torch.from_numpy(host).pin_memory()
        hX = torch.empty_like(hA).pin_memory()
        hP = torch.empty((batch, n), dtype=torch.int32).pin_memory()
        hI = torch.empty((batch,), dtype=torch.int32).pin_memory()
        from matrixinversion_gb300.host import link_bandwidth

        # the link's rates before the warm-up steps and just after the timed
        # ones: the host memory behind the link is shared with whatever else
        # runs on the machine, and a rate that drops during the run shows up
        # here.  (The probe pins 2 GB of fresh host memory; the pipeline's
        # warm-up steps run after it, not the timed ones.)
        link_before = link_bandwidth(dev)
        for _ in range(3):
            pipe.run(hA, args.pivot, hX, hP, hI)
        e2e_steps = max(1, min(args.steps, 5))
        step_times = []
        barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            t1 = time.perf_counter()
            pipe.run(hA, args.pivot, hX, hP, hI)
            step_times.append((time.perf_counter() - t1) * 1e3)
        barrier()
        dt = time.perf_counter() - t0
        dt = shards.max_over_ranks(dt, device=dev)
        h2d_bytes = batch * n * n * 4
        d2h_bytes = batch * n * n * 4 + batch * n * 4 + batch * 4
        link = link_bandwidth(dev)
        # both directions overlap, each at the rate they reach together
        floor_ms = max(h2d_bytes, d2h_bytes) / (link["both_each_way_gbs"] * 1e9) * 1e3
        step_ms = dt / e2e_steps * 1e3
        e2e = {"value": shards.aggregate_rate(batch * e2e_steps, dt, world), "unit": UNIT,
               "h2d_bytes_per_step": h2d_bytes, "d2h_bytes_per_step": d2h_bytes,
               "steps": e2e_steps, "chunk_matrices": 65536, "slots": 4, "ms_per_step": step_ms,
               "step_ms": [round(t, 2) for t in step_times],
               "link": {**link, "floor_ms": floor_ms, "frac": floor_ms / step_ms,
                        "before": link_before}}
        e2e_launches = pipe.launches_per_call(batch) * e2e_steps

    peak, peak_kind = hbm_peak()
    avg_launch_ms = sum(launch_ms) / len(launch_ms)
    achieved = batch * algorithmic_bytes(n) / (avg_launch_ms / 1e3) / 1e9
    tpm = ncu_traffic_per_matrix(n, args.pivot)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": (tpm * batch if tpm is not None else None), "peak_source": peak_kind,
                "bytes_per_matrix": algorithmic_bytes(n), "avg_launch_ms": avg_launch_ms}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(n, args.pivot, args.seed)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(args, batch),
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks.summary(),
            "gpu_launches": args.steps + e2e_launches,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
