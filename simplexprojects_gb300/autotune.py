"""Autotuner for the size classes: threads per CTA and CTAs per SM of every
size class of a plan, timed on the device class by class.

A plan groups its LPs into size classes (single-CTA LPs by how many CTAs of
their layout fit an SM, cluster LPs by cluster size K); every class has a
tuning key (``blpg_plan_class_key``: that CTA count, or 100 + K).  The tuner
takes, for each key, that class's LPs from every workload it is given, each
repeated until they fill the GPU ``waves`` times over (a class of a few
dozen LPs timed alone rewards wide CTAs that a full batch of them does not),
times whole-batch plan replays (CUDA events) for candidate (threads per CTA,
CTAs per SM), checks that statuses do not change, and keeps the candidate
with the lowest sum over workloads of its time over that workload's best
time.  The result is the JSON table that ``blpg_set_tuning`` reads::

    {"fp32_c2": 224, "fp32_c2_ctas": 2, "fp64_c104": 512, ...,
     "measured": {...}}

The table tuned on GB300 for the benchmark workloads is committed as
``tuning/gb300.json`` and compiled into the library as its default table
(``build.py``); ``load(path)`` applies another one, ``override(entries)``
lays entries over the compiled-in one and ``reset()`` restores it.

    python -m simplexprojects_gb300.autotune --out simplexprojects_gb300/tuning/gb300.json

tunes FP32 steepest edge on workloads 0-4 and FP64 Dantzig on workloads 1, 2
and 4, then the FP32 refresh period (an FP64 refresh every k pivots, or only
at termination) on workloads 1-4.
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
    """The LPs `ids` of a batch (repeats allowed), sharing its arrays through
    offsets."""
    oA, ob, oc = batch.offsets()
    fam = batch.family[ids] if batch.family is not None else None
    return LPBatch(batch.m[ids], batch.n[ids], batch.A, batch.b, batch.c, off_A=oA[ids],
                   off_b=ob[ids], off_c=oc[ids], family=fam)


def _sm_count() -> int:
    import torch
    return torch.cuda.get_device_properties(0).multi_processor_count


def tune(batches: dict, precision: str = "fp32", pricing: str = "dantzig",
         threads=(32, 64, 96, 128, 160, 192, 224, 256, 320, 384, 448, 512), steps: int = 5,
         waves: int = 4, base: dict | None = None, log=print) -> dict:
    """Per-class table (entries "<precision>_c<key>" and
    "<precision>_c<key>_ctas") for the workloads `batches` (name -> LPBatch),
    starting from `base` (default: empty)."""
    from .solver import DeviceBatch, Plan
    table = dict(base or {})
    measured = {}
    N.check(N.lib().blpg_set_tuning(json.dumps(table).encode()), "blpg_set_tuning")
    members = {}
    for name, batch in batches.items():
        plan = Plan(batch, precision, pricing=pricing)
        for key, ids, _ in class_members(plan):
            members.setdefault(key, []).append((name, batch, ids))
        plan.close()
    sms = _sm_count()
    for key in sorted(members):
        cps_max = key if key < 100 else 1
        subs = []
        for name, batch, ids in members[key]:
            reps = max(1, -(-waves * sms * cps_max // len(ids)))
            sub = _select(batch, np.tile(ids, reps))
            subs.append((name, len(ids), sub, DeviceBatch(sub, precision, pricing=pricing)))
        rows, seen, ref = [], set(), {}
        for cps in sorted({1, 2, 3, 4, cps_max} & set(range(1, cps_max + 1))):
            for nt in threads:
                trial = dict(table)
                trial[f"{precision}_c{key}"] = nt
                trial[f"{precision}_c{key}_ctas"] = cps
                N.check(N.lib().blpg_set_tuning(json.dumps(trial).encode()), "blpg_set_tuning")
                shapes = []
                for name, _, sub, db in subs:
                    db.plan.close()
                    db.plan = Plan(sub, precision, pricing=pricing)
                    cls = [c for c in db.plan.classes() if c["key"] == key][0]
                    shapes.append((cls["threads"], cls["ctas_per_sm"]))
                if tuple(shapes) in seen:  # the plans capped this candidate to one already timed
                    continue
                seen.add(tuple(shapes))
                times, same = [], True
                for name, _, sub, db in subs:
                    times.append(_time(db, steps))
                    st = db.result().status
                    ref.setdefault(name, st)
                    same &= bool(np.array_equal(st, ref[name]))
                rows.append(dict(threads=nt, ctas=cps, actual=[list(x) for x in shapes],
                                 ms=dict(zip([s[0] for s in subs], times)), statuses_equal=same))
                if log:
                    log(f"{precision} class {key}: threads {nt:4d} CTAs/SM {cps:2d} -> "
                        + ", ".join(f"{s[0]} {t:8.3f} ms" for s, t in zip(subs, times)))
        for *_, db in subs:
            db.plan.close()
        ok = [r for r in rows if r["statuses_equal"]]
        if ok:
            best_ms = {name: min(r["ms"][name] for r in ok) for name, *_ in subs}
            for r in ok:
                r["score"] = sum(r["ms"][name] / best_ms[name] for name in best_ms)
            best = min(ok, key=lambda r: r["score"])
            # the entries as requested: a plan maps them to the same shapes
            table[f"{precision}_c{key}"] = best["threads"]
            table[f"{precision}_c{key}_ctas"] = best["ctas"]
        measured[f"{precision}_c{key}"] = dict(
            lps={name: n for name, n, *_ in subs}, waves=waves, results=rows)
    N.lib().blpg_set_tuning(None)
    table.setdefault("measured", {}).update(measured)
    return table


def tune_refresh(batches: dict, periods=(0, 16, 32, 64), steps: int = 5, log=print) -> dict:
    """The FP32 refresh period: FP32 steepest edge on each workload with an
    FP64 refresh every k pivots (0: at termination only), statuses checked;
    the period with the lowest sum of time over each workload's best."""
    from .solver import DeviceBatch
    rows, ref = [], {}
    for k in periods:
        times, same = {}, True
        for name, batch in batches.items():
            db = DeviceBatch(batch, "fp32", pricing="steepest", refactor_period=k if k > 0 else -1)
            times[name] = _time(db, steps)
            st = db.result().status
            ref.setdefault(name, st)
            same &= bool(np.array_equal(st, ref[name]))
            db.plan.close()
        rows.append(dict(period=k, ms=times, statuses_equal=same))
        if log:
            log(f"fp32 refresh every {k or 'end'}: " +
                ", ".join(f"{n} {t:8.3f} ms" for n, t in times.items()))
    ok = [r for r in rows if r["statuses_equal"]]
    best_ms = {n: min(r["ms"][n] for r in ok) for n in batches}
    for r in ok:
        r["score"] = sum(r["ms"][n] / best_ms[n] for n in batches)
    best = min(ok, key=lambda r: r["score"])
    return {"fp32_refresh_period": best["period"], "measured": {"fp32_refresh_period": rows}}


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
    ap.add_argument("--out", default="tuning.json")
    ap.add_argument("--waves", type=int, default=4)
    ap.add_argument("--only", choices=["classes", "refresh"], default=None,
                    help="tune one part and merge it into --merge (default: both)")
    ap.add_argument("--merge", default=None, help="existing table to update")
    args = ap.parse_args()
    sizes = {0: 1024, 1: 10_000, 2: 2048, 3: 10_000, 4: 20_000}
    work = {k: generate(k, n, share_family_A=k in (3, 4)) for k, n in sizes.items()}
    table = {"measured": {}}
    if args.merge:
        table = json.loads(Path(args.merge).read_text())
        table.setdefault("measured", {})
    if args.only in (None, "classes"):
        runs = [("fp32", "steepest", (0, 1, 2, 3, 4)), ("fp64", "dantzig", (1, 2, 4))]
        for prec, pricing, kinds in runs:
            tuned = tune({f"kind{k}": work[k] for k in kinds}, prec, pricing=pricing,
                         waves=args.waves, base={})
            table["measured"].update({f"{k}_{pricing}": v for k, v in tuned.pop("measured").items()})
            table.update(tuned)
        table["how"] = ("python -m simplexprojects_gb300.autotune: per class key, the class's LPs "
                        "of each workload repeated to %d waves of the GPU; the lowest sum of time "
                        "over each workload's best time; the FP32 refresh period on workloads 1-4 "
                        "the same way" % args.waves)
    if args.only in (None, "refresh"):
        tuned = tune_refresh({f"kind{k}": work[k] for k in (1, 2, 3, 4)})
        table["measured"].update(tuned.pop("measured"))
        table.update(tuned)
    Path(args.out).parent.mkdir(parents=True, exist_ok=True)
    Path(args.out).write_text(json.dumps(table, indent=1))
    print(json.dumps({k: v for k, v in table.items() if k not in ("measured", "how")}))


if __name__ == "__main__":
    main()
