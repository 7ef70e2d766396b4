"""Autotuner for the size classes: threads per CTA, the CTA shared-memory
budget (which fixes each LP's cluster size), the cap on CTAs per SM (how
many small LPs share an SM) and, for the FP32 tableau, the FP64 refresh
period.

For a representative batch it times every candidate configuration on the
device (CUDA events around whole-batch plan replays), checks that the
statuses and objectives do not change, and writes the best one as the JSON
table that ``blpg_set_tuning`` reads::

    {"fp64_k1": 256, "fp64_smem": 115712, "fp64_ctas": 4, ...,
     "refactor_period": 0, "measured": {...}}

``load(path)`` applies a table to the library (``solve`` and plans created
afterwards use it).

    python -m simplexprojects_gb300.autotune --workload 1 --out tuning.json
"""
from __future__ import annotations

import argparse
import itertools
import json
import statistics
from pathlib import Path

import numpy as np

from . import _native as N
from .lp import generate


def _time(db, steps=5, warmup=2):
    import torch
    for _ in range(warmup):
        db.run()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    s = torch.cuda.current_stream()
    for a, b in ev:
        a.record(s)
        db.run()
        b.record(s)
    torch.cuda.synchronize()
    return statistics.median(a.elapsed_time(b) for a, b in ev)


def tune(batch, precision: str = "fp64", threads=(128, 256, 384, 512),
         budgets=(114 * 1024 - 1024, 227 * 1024), ctas=(1, 2, 4, 16),
         periods=(0,), pricing: str = "dantzig", steps: int = 5, log=print) -> dict:
    from .solver import DeviceBatch
    results = []
    ref = None
    for nt, bud, cps, per in itertools.product(threads, budgets, ctas, periods):
        table = {f"{precision}_k{k}": nt for k in (1, 2, 4, 8)}
        table[f"{precision}_ctas"] = cps
        N.lib().blpg_set_tuning(json.dumps(table).encode())
        db = DeviceBatch(batch, precision, cta_smem_budget=bud, refactor_period=per,
                         pricing=pricing)
        ms = _time(db, steps)
        r = db.result()
        if ref is None:
            ref = r
        same = bool(np.array_equal(r.status, ref.status))
        results.append(dict(threads=nt, smem_budget=bud, ctas=cps, period=per, ms=ms,
                            statuses_equal=same, classes=db.plan.classes()))
        if log:
            log(f"threads {nt:4d} budget {bud:7d} ctas/SM {cps:2d} period {per:3d}: {ms:8.3f} ms")
        db.plan.close()
    N.lib().blpg_set_tuning(None)
    best = min((r for r in results if r["statuses_equal"]), key=lambda r: r["ms"])
    table = {f"{precision}_k{k}": best["threads"] for k in (1, 2, 4, 8)}
    table[f"{precision}_smem"] = best["smem_budget"]
    table[f"{precision}_ctas"] = best["ctas"]
    table["refactor_period"] = best["period"]
    table["measured"] = results
    return table


def load(path: str) -> dict:
    """Apply a tuning table to the library."""
    table = json.loads(Path(path).read_text())
    keep = {k: v for k, v in table.items() if isinstance(v, int)}
    N.check(N.lib().blpg_set_tuning(json.dumps(keep).encode()), "blpg_set_tuning")
    return table


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", type=int, default=1)
    ap.add_argument("--count", type=int, default=4096)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--pricing", default="dantzig", choices=["dantzig", "steepest"])
    ap.add_argument("--periods", default="0", help="FP32 refresh periods to try, e.g. 0,16,32")
    ap.add_argument("--out", default="tuning.json")
    args = ap.parse_args()
    batch = generate(args.workload, args.count, share_family_A=True)
    periods = tuple(int(x) for x in args.periods.split(",")) if args.precision == "fp32" else (0,)
    table = tune(batch, args.precision, periods=periods, pricing=args.pricing)
    Path(args.out).write_text(json.dumps(table, indent=1))
    print(json.dumps({k: v for k, v in table.items() if k != "measured"}))


if __name__ == "__main__":
    main()
