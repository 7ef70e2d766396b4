"""Per-configuration report: throughput and accuracy of every solver mode on
one workload, as JSON lines.

For workload `kind` it times (CUDA events, device-resident data, median of
`steps` replays) the plain FP64 tableau, the FP32 tableau with the FP64
refresh at termination, and the FP32 tableau with periodic FP64 refreshes
every k pivots (k in --periods), with Dantzig and with steepest-edge
pricing, and reports for each:
  LPs/s, pivots/s, status agreement with the FP64 path, maximum relative
  objective difference to the FP64 path, and the maximum primal residual
  max_i (A x - b)_i and most negative x_j of the returned solutions.
The FP64 path is the reference here: it is bit-identical to the CPU
restatement of the method (tests/test_gpu_parity.py), whose objectives agree
with exact rational optima to 1e-9 (tests/test_oracle.py).

    python -m simplexprojects_gb300.report --workload 2 --count 2048
"""
from __future__ import annotations

import argparse
import json
import statistics

import numpy as np

from .lp import WORKLOAD_COUNTS, generate
from .solver import DeviceBatch


def _time(db, steps, warmup=2):
    import torch
    for _ in range(warmup):
        db.run()
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    for a, b in ev:
        a.record(s)
        db.run()
        b.record(s)
    torch.cuda.synchronize()
    return statistics.median(a.elapsed_time(b) for a, b in ev)


def residuals(batch, x, status=None):
    """(max_i (A x - b)_i, min_j x_j) over the LPs of a batch whose status is
    optimal (all LPs when no status is given); x in the off_c layout."""
    worst, neg = -np.inf, np.inf
    for k in range(batch.count):
        if status is not None and status[k] != 5:
            continue
        A, b, _ = batch.lp(k)
        _, _, oc = batch.offsets()
        xk = x[oc[k]:oc[k] + A.shape[1]]
        worst = max(worst, float((A @ xk - b).max()))
        neg = min(neg, float(xk.min()))
    return worst, neg


def run(kind: int, count: int, steps: int, periods=(16, 32, 64), check: int = 256):
    batch = generate(kind, count, share_family_A=True)
    out = []
    ref = None
    modes = ([("fp64", 0, "dantzig"), ("fp32", 0, "dantzig")]
             + [("fp32", k, "dantzig") for k in periods]
             + [("fp32", 0, "steepest")] + [("fp32", k, "steepest") for k in periods])
    for prec, period, pricing in modes:
        db = DeviceBatch(batch, prec, want_x=True, refactor_period=period, pricing=pricing)
        ms = _time(db, steps)
        r = db.result()
        if ref is None:
            ref = r
        ok = ref.status == 5
        rel = np.abs(r.objective[ok] - ref.objective[ok]) / np.maximum(np.abs(ref.objective[ok]), 1.0)
        sub = batch.head(min(check, batch.count))
        res, neg = residuals(sub, r.x, r.status)
        out.append(dict(workload=kind, lps=batch.count, precision=prec, refresh_period=period,
                        pricing=pricing,
                        ms=ms, lps_per_s=batch.count / (ms * 1e-3),
                        pivots_per_s=float(r.pivots.sum()) / (ms * 1e-3),
                        mean_pivots=float(r.pivots.mean()),
                        status_match_fp64=float((r.status == ref.status).mean()),
                        max_rel_obj_diff_fp64=float(rel.max()) if rel.size else 0.0,
                        max_primal_residual=res, min_x=neg, classes=db.plan.classes()))
        db.plan.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", type=int, default=2)
    ap.add_argument("--count", type=int, default=0)
    ap.add_argument("--steps", type=int, default=3)
    args = ap.parse_args()
    count = args.count or WORKLOAD_COUNTS[args.workload]
    for line in run(args.workload, count, args.steps):
        print(json.dumps(line))


if __name__ == "__main__":
    main()
