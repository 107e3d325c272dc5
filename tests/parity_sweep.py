"""Parity of the partial-pivoting sweep configuration on whole batches.

For every n and pivot rule: 1,000,000 matrices (entries uniform [-1, 1) from
MT19937 seed 0), inverted on the GPU through the library; every pivot vector
is compared with the oracle's replay of the rule, and on a 20,000-matrix sample
the per-matrix residual ||AX - I||_inf is compared with the reference
algorithm's own (the oracle's FP32 port, same pivots) and with the
componentwise bound of an LU-based inverse with the same pivot sequence,
n u || |L| |U| |X64| ||_inf (L U = P A in FP64): the tolerance of the parity
tests is max(8 n u || |L||U||X64| ||, 2 r_port).  Test infrastructure: prints
one JSON line per case and, with --md, a markdown table.

    python tests/parity_sweep.py --n 2-32 --modes reference,reference_serial --md out.md
"""
import argparse
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

U = 2.0 ** -24


def parse_range(text):
    out = []
    for part in text.split(","):
        if "-" in part:
            a, b = part.split("-")
            out.extend(range(int(a), int(b) + 1))
        elif part:
            out.append(int(part))
    return out


def run(n, modes, batch, sample, O, mi):
    import torch

    A = O.uniform(0, batch, n)
    rows = []
    for mode in modes:
        dA = torch.from_numpy(A).cuda()
        perm = torch.empty((batch, n), dtype=torch.int32, device="cuda")
        info = torch.empty((batch,), dtype=torch.int32, device="cuda")
        mi.batched_inverse_(dA, mode, perm=perm, info=info)
        torch.cuda.synchronize()
        got = perm.cpu().numpy()
        want = O.pivots(A, mode)
        exact = int((got == want).all(axis=1).sum())
        idx = np.sort(np.random.RandomState(n).choice(batch, min(sample, batch), replace=False))
        X = dA[torch.from_numpy(idx).cuda()].cpu().numpy()
        As = A[idx]
        rg = O.residual(As, X)[:, 0]
        Xp, _, _ = O.ref_inverse_f32(As, mode)
        rp = O.residual(As, Xp)[:, 0]
        growth = n * U * O.lu_growth_bound(As, want[idx])
        ok = np.isfinite(rg) & np.isfinite(rp) & (rp > 0)
        ratio = rg[ok] / rp[ok]
        lu_ratio = rg[ok] / growth[ok]                # the constant on n u |L||U||X| the kernel needs
        within = np.all(rg <= np.maximum(8.0 * growth, 2.0 * rp))
        rows.append({
            "n": n, "mode": mode, "batch": batch, "pivots_exact": exact, "singular": int((info != 0).sum().item()),
            "sample": int(idx.size), "res_median": float(np.median(rg)), "port_median": float(np.median(rp)),
            "ratio_median": float(np.median(ratio)), "ratio_max": float(ratio.max()),
            "lu_ratio_median": float(np.median(lu_ratio)), "lu_ratio_max": float(lu_ratio.max()),
            "above_8": int((lu_ratio > 8.0).sum()), "within_tolerance": bool(within),
        })
        del dA, perm, info
        torch.cuda.empty_cache()
    return rows


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--n", default="2-32")
    p.add_argument("--modes", default="reference,reference_serial")
    p.add_argument("--batch", type=int, default=1_000_000)
    p.add_argument("--sample", type=int, default=20_000)
    p.add_argument("--md", default=None)
    args = p.parse_args(argv)
    from oracle import oracle as O
    import matrixinversion_gb300 as mi

    O.build()
    mi._lib.load()
    rows = []
    for n in parse_range(args.n):
        for r in run(n, args.modes.split(","), args.batch, args.sample, O, mi):
            print(json.dumps(r), flush=True)
            rows.append(r)
    if args.md:
        with open(args.md, "w") as f:
            f.write("| n | rule | pivots bit-exact | residual median (kernel / port) | r_gpu / r_port median, max "
                    "| r_gpu / (n u ‖|L||U||X|‖) median, max | above 8 | within tolerance |\n"
                    "|---|---|---|---|---|---|---|---|\n")
            for r in rows:
                f.write(f"| {r['n']} | {r['mode']} | {r['pivots_exact']:,} / {r['batch']:,} | "
                        f"{r['res_median']:.2e} / {r['port_median']:.2e} | {r['ratio_median']:.2f}, "
                        f"{r['ratio_max']:.1f} | {r['lu_ratio_median']:.4f}, {r['lu_ratio_max']:.2f} | "
                        f"{r['above_8']} | {'yes' if r['within_tolerance'] else 'NO'} |\n")
    return rows


if __name__ == "__main__":
    main(sys.argv[1:])
