"""Autotuner for the size classes: threads per CTA and CTAs per SM of every
size class of a plan, timed on the device class by class.

A plan groups its LPs into size classes (single-CTA LPs by how many CTAs of
their layout fit an SM, cluster LPs by cluster size K); every class has a
tuning key (``blpg_plan_class_key``: that CTA count, or 100 + K).  For each
class of a representative batch the tuner takes the class's LPs alone (a
batch sharing the original arrays), times whole-batch plan replays (CUDA
events) for candidate (threads per CTA, CTAs per SM), checks that statuses
and objectives do not change, and keeps the fastest.  The result is the JSON
table that ``blpg_set_tuning`` reads::

    {"fp32_c2": 224, "fp32_c2_ctas": 2, "fp64_c104": 512, ...,
     "measured": {...}}

The table tuned on GB300 for the benchmark workloads is committed as
``tuning/gb300.json`` and compiled into the library as its default table
(``build.py``); ``load(path)`` applies another one, ``reset()`` restores the
compiled-in one.

    python -m simplexprojects_gb300.autotune --out simplexprojects_gb300/tuning/gb300.json

tunes FP32 steepest edge on workload 3 and FP32 / FP64 on workload 4 (every
shape of the other workloads occurs there) and merges the three.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import statistics
from pathlib import Path

import numpy as np

from . import _native as N
from .lp import LPBatch, generate


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


def class_members(plan) -> list:
    """(tuning key, LP ids, class info) of every size class of a Plan."""
    out = []
    for i, info in enumerate(plan.classes()):
        key = C.c_int32()
        ids = np.zeros(max(1, info["lps"]), np.int32)
        N.check(N.lib().blpg_plan_class_key(plan._h, i, C.byref(key),
                                            ids.ctypes.data_as(C.POINTER(C.c_int32))),
                "blpg_plan_class_key")
        out.append((key.value, ids[:info["lps"]].copy(), info))
    return out


def _select(batch: LPBatch, ids) -> LPBatch:
    """The LPs `ids` of a batch, sharing its arrays through offsets."""
    oA, ob, oc = batch.offsets()
    fam = batch.family[ids] if batch.family is not None else None
    return LPBatch(batch.m[ids], batch.n[ids], batch.A, batch.b, batch.c, off_A=oA[ids],
                   off_b=ob[ids], off_c=oc[ids], family=fam)


def tune(batch: LPBatch, precision: str = "fp32", pricing: str = "dantzig",
         threads=(96, 128, 160, 192, 224, 256, 320, 384, 448, 512), steps: int = 5,
         base: dict | None = None, log=print) -> dict:
    """Per-class table for `batch` (entries "<precision>_c<key>" and
    "<precision>_c<key>_ctas"), starting from `base` (default: empty)."""
    from .solver import DeviceBatch, Plan
    table = dict(base or {})
    measured = {}
    N.check(N.lib().blpg_set_tuning(json.dumps(table).encode()), "blpg_set_tuning")
    plan = Plan(batch, precision, pricing=pricing)
    classes = class_members(plan)
    plan.close()
    for key, ids, info in classes:
        sub = _select(batch, ids)
        cps_max = key if key < 100 else 1
        seen, results, ref = set(), [], None
        for cps in sorted({1, 2, 3, 4, cps_max} & set(range(1, cps_max + 1))):
            for nt in threads:
                trial = dict(table)
                trial[f"{precision}_c{key}"] = nt
                trial[f"{precision}_c{key}_ctas"] = cps
                N.lib().blpg_set_tuning(json.dumps(trial).encode())
                db = DeviceBatch(sub, precision, pricing=pricing)
                cls = db.plan.classes()[0]
                shape = (cls["threads"], cls["ctas_per_sm"])
                if shape in seen:
                    db.plan.close()
                    continue
                seen.add(shape)
                ms = _time(db, steps)
                r = db.result()
                if ref is None:
                    ref = r
                same = bool(np.array_equal(r.status, ref.status))
                results.append(dict(threads=nt, ctas=cps, actual=list(shape), ms=ms,
                                    statuses_equal=same))
                if log:
                    log(f"{precision} class {key} ({len(ids)} LPs): threads {shape[0]:4d} "
                        f"CTAs/SM {shape[1]:2d}: {ms:8.3f} ms")
                db.plan.close()
        ok = [r for r in results if r["statuses_equal"]]
        if ok:
            best = min(ok, key=lambda r: r["ms"])
            # the shape the plan actually took (residency follows occupancy)
            table[f"{precision}_c{key}"] = best["actual"][0]
            table[f"{precision}_c{key}_ctas"] = best["actual"][1]
        measured[f"{precision}_c{key}"] = dict(lps=int(len(ids)), results=results)
    N.lib().blpg_set_tuning(None)
    table.setdefault("measured", {}).update(measured)
    return table


def load(path: str) -> dict:
    """Apply a tuning table to the library (later plans and solves use it)."""
    table = json.loads(Path(path).read_text())
    keep = {k: v for k, v in table.items() if isinstance(v, int)}
    N.check(N.lib().blpg_set_tuning(json.dumps(keep).encode()), "blpg_set_tuning")
    return table


def override(entries: dict) -> None:
    """Apply the compiled-in table (tuning/gb300.json) with `entries` laid
    over it; a table given to blpg_set_tuning replaces the whole table."""
    table = json.loads((Path(__file__).parent / "tuning" / "gb300.json").read_text())
    table = {k: v for k, v in table.items() if isinstance(v, int)}
    table.update(entries)
    N.check(N.lib().blpg_set_tuning(json.dumps(table).encode()), "blpg_set_tuning")


def reset() -> None:
    """Restore the library's compiled-in table (tuning/gb300.json)."""
    N.check(N.lib().blpg_set_tuning(None), "blpg_set_tuning")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--count", type=int, default=4096)
    ap.add_argument("--out", default="tuning.json")
    args = ap.parse_args()
    table = {}
    runs = [(3, "fp32", "steepest"), (4, "fp32", "steepest"), (4, "fp64", "dantzig")]
    for kind, prec, pricing in runs:
        batch = generate(kind, args.count, share_family_A=True)
        tuned = tune(batch, prec, pricing=pricing, base={})
        for k, v in tuned.items():
            if k == "measured":
                table.setdefault("measured", {})[f"kind{kind}_{prec}_{pricing}"] = v
            elif k not in table:  # the first workload that tunes a class keeps it
                table[k] = v
    Path(args.out).parent.mkdir(parents=True, exist_ok=True)
    Path(args.out).write_text(json.dumps(table, indent=1))
    print(json.dumps({k: v for k, v in table.items() if k != "measured"}))


if __name__ == "__main__":
    main()
