"""Benchmark: batched LP solve throughput (LPs/s, pivots/s) on one GB300.

Default workload: kind 3 (the metric's configuration): 64 base LPs (m=174,
n=142), 40,000 perturbed instances solved by the plain FP64 solver to train
the warm-start network, 10,000 held-out instances timed with the learned warm
start + FP32 tableau (value: the network's basis probabilities weight
steepest-edge pricing) beside the plain FP64 cold solver (plain_fp64, the
reference's Dantzig method) and, in `variants`, the crash-mode warm start and
the cold FP32 solver under both pricing rules.

Workloads are the synthetic configurations of include/blpg.h (seeded,
deterministic; they stand in for the Netlib-sized LPs the reference was run
on).  One step = one solve of the whole workload batch.

  value        LPs/s with A, b, c already resident in HBM (plan replay; each
               step re-solves from the input data, nothing is cached)
  e2e          LPs/s through the public C ABI from host buffers
               (blpg_learned_solve for the learned warm start of workload 3,
               blpg_solve_batch for the others): host->device copy of A, b, c
               (and the family ids) and device->host copy of
               status/objective/pivots inside the timed region
  roofline     algorithmic bytes per pivot of the condensed tableau
               s * (2 (m+1) W + 4 (m+1)), W = n + 1 stored columns (nonbasic
               + RHS), s = 8 (FP64) / 4 (FP32), summed over the LPs' pivots,
               divided by the CUDA-event time of the solve kernels; peak =
               shared-memory bandwidth measured live on the device.  The FP64
               tableau is also bound by the FP64 FMA pipe (one FMA per stored
               element per pivot): reported beside it.
  cpu_baseline the CPU oracle (plain-C restatement of the reference method,
               all host threads) on a bounded sample of the same workload

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload 0..4]
                  [--precision fp64|fp32] [--impl blpg|reference]
  python bench.py --profile-case N [--workload K] [--precision P] [--pricing R]
               a small solve for ncu captures: N LPs of the workload (families
               sharing A) solved twice on a device-resident plan (the second
               launch is the capture target); prints the class plan, the
               status histogram and the pivot total.  A few MB on the device,
               so a full-metric capture of one solve launch ends in a minute.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD_NAMES = {
    0: "kind0: 1,024 LPs m=28 n=32 density 0.6",
    1: "kind1: 10,000 LPs m in {50,56,74,105}, n~U[m,1.8m], 10% unbounded, 5% zero-b rows",
    2: "kind2: 2,048 LPs m=205 n=203 density 0.15",
    3: "kind3 eval: 10,000 perturbed LPs (m=174, n=142, 64 families)",
    4: "kind4: 200,000 LPs m log-uniform [16,256], n~U[m/2,2m]",
}
L2_BYTES = 129 * 1024 * 1024


def workload(kind: int, rank: int = 0, world: int = 1):
    import simplexprojects_gb300 as sp
    if kind == 3:
        count, first = 10_000, 40_000  # the evaluation split
    else:
        count, first = sp.WORKLOAD_COUNTS[kind], 0
    lo, n = sp.shard(count, first, rank, world)
    return sp.generate(kind, n, seed=sp.DEFAULT_SEED, first=lo, share_family_A=True), count


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of
# solve_kernel<float> at the default workload (10,000 LPs), from an ncu
# capture of this bench's timed region (one pass, the full-size launch; the
# two captured launches read 59.24 / 59.12 MB and wrote 6.98 / 6.52 MB).  The
# writes are mostly lines the L2 flush between steps left dirty.
KIND3_SOLVE_DRAM_BYTES = (59242240 + 6981120 + 59117824 + 6521856) / 2
KIND3_SOLVE_DRAM_SOURCE = ("ncu --metrics gpu__time_duration.sum,dram__bytes_read.sum,"
                           "dram__bytes_write.sum --clock-control none --nvtx --nvtx-include "
                           "timed_region/ python bench.py --steps 2 --warmup 3 --epochs 4 "
                           "--no-cpu-baseline (mean of the two solve launches)")


def pinned(batch):
    """The same batch with A, b, c in pinned (page-locked) host memory, as the
    end-to-end measurement copies from: numpy views of pinned torch tensors,
    kept alive by the batch's meta."""
    import torch
    import simplexprojects_gb300 as sp
    keep, arrs = [], []
    for a in (batch.A, batch.b, batch.c):
        t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
        v = t.numpy()
        v[...] = a
        keep.append(t)
        arrs.append(v)
    meta = dict(batch.meta, pinned_host_buffers=keep)
    return sp.LPBatch(batch.m, batch.n, arrs[0], arrs[1], arrs[2], off_A=batch.off_A,
                      off_b=batch.off_b, off_c=batch.off_c, family=batch.family, meta=meta)


def bytes_per_pivot(m, n, s):
    """Shared-memory bytes one pivot of the condensed tableau must move: the
    (m + 1) x (n + 1) stored entries (n nonbasic columns + RHS) read and
    written once, plus the pivot column and RHS extracted (written, then
    read by the ratio test).  Element size s."""
    W = n + 1
    return s * (2.0 * (m + 1) * W + 4.0 * (m + 1))


class Clocks:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.p is not None:
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
                self.out = ""

    def summary(self):
        rows = []
        for line in (self.out or "").splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append(dict(sm=float(parts[1]), max=float(parts[2]), power=float(parts[3]),
                                 hw=parts[5], hwt=parts[6], swt=parts[7], pcap=parts[8]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        loaded = [r for r in rows if r["power"] > 250] or rows
        reasons = set()
        for r in loaded:
            for key, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"),
                              ("swt", "sw_thermal_slowdown"), ("pcap", "sw_power_cap")):
                if r[key].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r["sm"] for r in loaded),
                "sm_max_mhz": max(r["max"] for r in loaded), "reasons": sorted(reasons),
                "samples": len(loaded)}


def cpu_baseline(batch, precision: str, budget_s: float = 12.0):
    """The CPU oracle on a bounded sample: LPs/s with all host threads."""
    from oracle import ref  # CPU baseline leg only
    threads = os.cpu_count() or 1
    k = min(batch.count, max(threads * 4, 64))
    t0 = time.perf_counter()
    ref.solve_batch(batch.head(k), precision, threads=threads)
    dt = time.perf_counter() - t0
    rate = k / dt
    k2 = int(min(batch.count, max(k, rate * budget_s)))
    sample = batch.head(k2)
    t0 = time.perf_counter()
    r = ref.solve_batch(sample, precision, threads=threads)
    dt = time.perf_counter() - t0
    return {"value": k2 / dt, "unit": "LPs/s", "cores": threads, "kind": "port",
            "pivots_per_s": float(r.pivots.sum()) / dt, "ms": dt * 1e3, "lps": k2,
            "sample": f"first {k2} LPs of the workload, {precision} oracle, {dt:.1f}s"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    batch, total = workload(args.workload)
    warm = [cpu_baseline(batch, args.precision, budget_s=2.0) for _ in range(max(1, args.warmup // 3))]
    vals = [cpu_baseline(batch, args.precision, budget_s=8.0) for _ in range(args.steps)]
    v = statistics.median(x["value"] for x in vals)
    cb = dict(vals[-1], value=v)
    print(json.dumps({
        "impl": "reference", "metric": "LPs/s", "value": v, "unit": "LPs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        # one step = one timed sample of the workload (a bounded CPU run)
        "ms_per_step": statistics.median(x["ms"] for x in vals),
        "step_ms_all": [x["ms"] for x in vals],
        "dtype": "f64" if args.precision == "fp64" else "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD_NAMES[args.workload], "precision": args.precision,
                   "lps": total},
        "cpu_baseline": cb,
        "e2e": {"value": v, "unit": "LPs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference arm = CPU oracle (plain-C restatement of BLPG-Solver's method); the "
                "reference's own CUDA/boost/GLPK build cannot be compiled here",
        "warm_runs": len(warm),
    }))


def run_learned(args, rank, world, local, dist=None):
    """Workload 3: the learned warm start + FP32 tableau on the 10,000
    evaluation LPs, against the plain FP64 cold solver on the same LPs."""
    import torch
    import ctypes as C
    import simplexprojects_gb300 as sp
    from simplexprojects_gb300 import _native as N
    from simplexprojects_gb300.warmstart import WarmStart, LearnedSolver, basis_accuracy

    dev = f"cuda:{local}"
    t_setup = time.perf_counter()
    lo, n_eval = sp.shard(10_000, 40_000, rank, world)
    train = sp.generate(3, 40_000, seed=sp.DEFAULT_SEED, first=0, share_family_A=True)
    evalb = sp.generate(3, n_eval, seed=sp.DEFAULT_SEED, first=lo, share_family_A=True)
    # the end-to-end inputs in pinned host memory, allocated before the device
    # holds anything large (a pinned buffer allocated later can land on host
    # memory farther from the GPU, and its uploads then run slower)
    evalp = pinned(evalb)
    tb = sp.solve(train, "fp64", want_basis=True)  # plain FP64 solver labels its own bases
    # inference runs the whole evaluation batch as one chunk (one GEMM per layer)
    ws = WarmStart(174, 142, 64, seed=7, device=dev, max_batch=(max(n_eval, 1) + 63) // 64 * 64)
    rep = ws.train(train, tb.basis, epochs=args.epochs, lr=1e-3, batch_size=512)
    del train
    ls = LearnedSolver(ws, evalb, "fp32", mode="guided")
    crash = LearnedSolver(ws, evalb, "fp32", mode="crash")
    plain = sp.DeviceBatch(evalb, "fp64", device=dev)
    cold32 = sp.DeviceBatch(evalb, "fp32", device=dev)
    cold32se = sp.DeviceBatch(evalb, "fp32", device=dev, pricing="steepest")
    setup_s = time.perf_counter() - t_setup
    stream = torch.cuda.current_stream()
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)

    def timed(fn, steps):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        for i in range(steps):
            flush.fill_(float(i))
            ev[i][0].record(stream)
            fn()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in ev]

    def barrier():
        if dist is not None:
            dist.barrier()

    def max_over_ranks(v: float) -> float:
        """Whole-job time: the slowest rank's."""
        if dist is None:
            return v
        t = torch.tensor([v], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    for _ in range(args.warmup):
        ls.run()
        plain.run()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        barrier()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("timed_region")
        t_learned = timed(ls.run, args.steps)
        torch.cuda.nvtx.range_pop()
        barrier()
    t_plain = timed(plain.run, args.steps)
    ls.predict()
    t_solve = timed(lambda: ls.db.run(weight=ls.weight), args.steps)  # the FP32 solve alone
    t_pred = timed(ls.predict, args.steps)
    res = ls.result()
    pres = plain.result()
    variants = {}
    for name, fn, obj in (("learned_crash_fp32_dantzig", crash.run, crash.db),
                          ("cold_fp32_dantzig", cold32.run, cold32),
                          ("cold_fp32_steepest", cold32se.run, cold32se)):
        for _ in range(2):
            fn()
        barrier()
        tv = max_over_ranks(statistics.median(timed(fn, max(3, args.steps // 2))))
        rv = obj.result()
        variants[name] = {"value": len(rv.status) * world / (tv * 1e-3), "unit": "LPs/s",
                          "ms_per_step": tv, "mean_pivots": float(rv.pivots.mean()),
                          "status_match": float((rv.status == pres.status).mean())}
    cres = crash.db.result()
    hint = crash.hint.cpu().numpy()
    plain_b = sp.solve(evalb, "fp64", want_basis=True)
    acc, exact = basis_accuracy(hint, plain_b.basis, 174)
    ms = max_over_ranks(statistics.median(t_learned))
    ms_plain = max_over_ranks(statistics.median(t_plain))
    ms_solve = max_over_ranks(statistics.median(t_solve))
    ok = pres.status == 5
    rel = np.abs(res.objective[ok] - pres.objective[ok]) / np.maximum(np.abs(pres.objective[ok]), 1.0)
    # e2e through the public C ABI call (blpg_learned_solve) from host arrays (pinned)
    e2e = []
    for i in range(args.warmup + args.steps):
        barrier()
        t0 = time.perf_counter()
        r2 = ls.solve(evalp)
        if i >= args.warmup:
            e2e.append(time.perf_counter() - t0)
    e2e_ms = max_over_ranks(statistics.median(e2e) * 1e3)
    assert np.array_equal(r2.status, res.status)
    if rank != 0:
        return
    smem, f64, f32 = C.c_double(), C.c_double(), C.c_double()
    N.check(N.lib().blpg_measure_peaks(local, C.byref(smem), C.byref(f64), C.byref(f32)),
            "blpg_measure_peaks")
    piv = res.pivots.astype(np.float64)
    m, n = 174.0, 142.0
    alg_bytes = float((piv * bytes_per_pivot(m, n, 4)).sum())
    ach = alg_bytes / (ms_solve * 1e-3) / 1e9
    flops = float((piv * 2.0 * (m + 1) * (n + 1)).sum())
    ach_tf = flops / (ms_solve * 1e-3) / 1e12
    cpu = None if args.no_cpu_baseline else cpu_baseline(evalb, "fp64")
    h2d = int(evalb.A.nbytes + evalb.b.nbytes + evalb.c.nbytes + 4 * evalb.count)
    total = 10_000
    out = {
        "metric": "LPs/s", "value": total / (ms * 1e-3), "unit": "LPs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generator, include/blpg.h)",
        "config": {"workload": WORKLOAD_NAMES[3], "lps": total, "precision": "fp32+fp64 refresh",
                   "method": "learned warm start (MLP 3x512 bf16): network probabilities "
                             "weight steepest-edge pricing of the FP32 tableau",
                   "train_lps": 40_000, "epochs": args.epochs,
                   "parallelism": "replicas" if world > 1 else "1gpu",
                   "l2": "L2 flushed between iterations",
                   "classes": ls.db.plan.classes()},
        "pivots_per_s": float(piv.sum()) * world / (ms * 1e-3),
        "plain_fp64": {"value": total / (ms_plain * 1e-3), "unit": "LPs/s", "ms_per_step": ms_plain,
                       "pivots_per_s": float(pres.pivots.sum()) * world / (ms_plain * 1e-3),
                       "mean_pivots": float(pres.pivots.mean()),
                       "method": "FP64 tableau, Dantzig pricing, cold slack basis"},
        "speedup_vs_plain_fp64": ms_plain / ms,
        "variants": variants,
        "learned": {"mean_pivots": float(piv.mean()),
                    "pivots_saved": 1.0 - float(piv.sum()) / float(pres.pivots.sum()),
                    "pivots_saved_vs_cold_steepest":
                        1.0 - float(piv.mean()) / variants["cold_fp32_steepest"]["mean_pivots"],
                    "crash_mode": {"mean_pivots": float(cres.pivots.mean()),
                                   "fallback_rate": float(((cres.info & 2) > 0).mean()),
                                   "shifted_rate": float(((cres.info & 64) > 0).mean()),
                                   "dual_rate": float(((cres.info & 8) > 0).mean()),
                                   "basis_column_accuracy": acc, "exact_basis_rate": exact},
                    "predict_ms": statistics.median(t_pred), "solve_ms": ms_solve,
                    "train_s": rep.seconds, "setup_s": setup_s,
                    "final_train_bce": rep.losses[-1] if rep.losses else None},
        "status_match": float((res.status == pres.status).mean()),
        "max_rel_obj_err_vs_fp64": float(rel.max()) if rel.size else 0.0,
        "e2e": {"value": total / (e2e_ms * 1e-3), "unit": "LPs/s", "h2d_bytes_per_step": h2d,
                # status, pivots, info (4 bytes each) and the objective (8)
                "d2h_bytes_per_step": int(total * 20), "ms_per_step": e2e_ms,
                "step_ms_all": [round(t * 1e3, 3) for t in e2e],
                "call": "blpg_learned_solve (include/blpg.h)"},
        "roofline": {"bound": "smem", "achieved": ach, "peak": smem.value, "unit": "GB/s",
                     "frac": ach / smem.value, "traffic": KIND3_SOLVE_DRAM_BYTES,
                     "traffic_source": KIND3_SOLVE_DRAM_SOURCE,
                     "hbm": {"achieved": KIND3_SOLVE_DRAM_BYTES / (ms_solve * 1e-3) / 1e9,
                             "unit": "GB/s", "note": "DRAM bytes of one solve launch over its "
                             "CUDA-event time: the inputs are read once per LP"},
                     "kernel": "solve_kernel<float> (FP32 condensed tableau pivots)",
                     "bytes_per_pivot": bytes_per_pivot(m, n, 4),
                     "peak_source": "measured live (blpg_measure_peaks: shared-memory stream probe)",
                     "fma_pipe": {"achieved": ach_tf, "peak": f32.value, "unit": "TFLOP/s",
                                  "frac": ach_tf / f32.value, "pipe": "fp32"}},
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "gpu_launches": args.steps * ls.launches(),
        "step_ms_all": t_learned,
    }
    print(json.dumps(out))


def run_profile_case(args):
    import simplexprojects_gb300 as sp
    batch = sp.generate(args.workload, args.profile_case, seed=sp.DEFAULT_SEED,
                        share_family_A=True)
    db = sp.DeviceBatch(batch, args.precision, pricing=args.pricing)
    for _ in range(2):
        db.run()
    r = db.result()
    print("classes", db.plan.classes())
    print("status", np.bincount(r.status).tolist(), "pivots", int(r.pivots.sum()))
    db.plan.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", type=int, default=3)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--impl", default="blpg", choices=["blpg", "reference"])
    ap.add_argument("--pricing", default="dantzig", choices=["dantzig", "steepest"],
                    help="pricing rule of workloads 0-2, 4 (3 runs every variant)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-case", type=int, default=0, metavar="N",
                    help="small solve of N LPs for ncu captures (see the module docstring)")
    ap.add_argument("--measure-peaks", action="store_true",
                    help="print the live shared-memory / FP64 / FP32 peak probes and exit")
    args = ap.parse_args()
    if args.profile_case > 0:
        return run_profile_case(args)
    if args.measure_peaks:
        import ctypes as C
        from simplexprojects_gb300 import _native as N
        smem, f64, f32 = C.c_double(), C.c_double(), C.c_double()
        N.check(N.lib().blpg_measure_peaks(0, C.byref(smem), C.byref(f64), C.byref(f32)),
                "blpg_measure_peaks")
        print(json.dumps({"smem_gbs": smem.value, "fp64_tflops": f64.value,
                          "fp32_tflops": f32.value}))
        return
    args.warmup = max(3, args.warmup)

    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    import simplexprojects_gb300 as sp
    from simplexprojects_gb300 import _native as N
    import ctypes as C

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    if args.workload == 3:
        run_learned(args, rank, world, local, dist)
        if dist is not None:
            dist.destroy_process_group()
        return

    def barrier():
        if dist is not None:
            dist.barrier()

    batch, total = workload(args.workload, rank, world)
    # the end-to-end inputs in pinned host memory, allocated before the device
    # holds anything large (a pinned buffer allocated later can land on host
    # memory farther from the GPU, and its uploads then run slower)
    batchp = pinned(batch)
    s = 8 if args.precision == "fp64" else 4
    db = sp.DeviceBatch(batch, args.precision, device=f"cuda:{local}", pricing=args.pricing)
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        db.run()
    torch.cuda.synchronize()
    res = db.result()
    pivots = res.pivots.astype(np.float64)
    alg_bytes = float((pivots * bytes_per_pivot(batch.m.astype(np.float64),
                                                 batch.n.astype(np.float64), s)).sum())
    flops = float((pivots * 2.0 * (batch.m + 1.0) * (batch.n + 1.0)).sum())

    # ---- value: device-resident inputs (larger than L2 for kinds 1-4) ----
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=f"cuda:{local}")
    with Clocks(local) as clk:
        barrier()
        torch.cuda.synchronize()
        for i in range(args.steps):
            flush.fill_(float(i))  # L2 flush between iterations
            ev[i][0].record(stream)
            db.run()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        barrier()
    times = [a.elapsed_time(b) for a, b in ev]
    ms = statistics.median(times)
    if dist is not None:
        t = torch.tensor([ms], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = total / (ms * 1e-3)

    # ---- e2e: the public C ABI from host buffers (pinned) ----
    e2e_times = []
    for i in range(args.warmup + args.steps):
        barrier()
        t0 = time.perf_counter()
        r = sp.solve(batchp, args.precision, pricing=args.pricing)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            e2e_times.append(dt)
    e2e_ms = statistics.median(e2e_times) * 1e3
    if dist is not None:
        t = torch.tensor([e2e_ms], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    assert np.array_equal(r.status, res.status) and np.array_equal(r.objective, res.objective)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    smem, f64, f32 = C.c_double(), C.c_double(), C.c_double()
    N.check(N.lib().blpg_measure_peaks(local, C.byref(smem), C.byref(f64), C.byref(f32)),
            "blpg_measure_peaks")
    ach = alg_bytes / (ms * 1e-3) / 1e9
    ach_tf = flops / (ms * 1e-3) / 1e12
    fp_peak = f64.value if args.precision == "fp64" else f32.value
    roof = {"bound": "smem", "achieved": ach, "peak": smem.value, "unit": "GB/s",
            "frac": ach / smem.value, "traffic": None,
            "peak_source": "measured live (blpg_measure_peaks: shared-memory stream probe)",
            "fma_pipe": {"achieved": ach_tf, "peak": fp_peak, "unit": "TFLOP/s",
                         "frac": ach_tf / fp_peak, "pipe": args.precision}}
    if roof["fma_pipe"]["frac"] > roof["frac"]:
        roof["bound_by"] = f"{args.precision} FMA pipe"
    cpu = None if args.no_cpu_baseline else cpu_baseline(batch, args.precision)
    h2d = int(batch.A.nbytes + batch.b.nbytes + batch.c.nbytes)
    d2h = int(batch.count * (4 + 8 + 4))
    launches = db.plan.launches()
    out = {
        "metric": "LPs/s", "value": value, "unit": "LPs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak" if world > 1 else "weak",
        "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32",
        "data": "synthetic (seeded generator, include/blpg.h)",
        "config": {"workload": WORKLOAD_NAMES[args.workload], "lps": total,
                   "precision": args.precision, "pricing": args.pricing,
                   "parallelism": "replicas" if world > 1 else "1gpu",
                   "l2": "inputs larger than L2; L2 flushed between iterations",
                   "classes": db.plan.classes()},
        "pivots_per_s": float(pivots.sum()) * world / (ms * 1e-3),
        "mean_pivots": float(pivots.mean()),
        "status_counts": np.bincount(res.status, minlength=7).tolist(),
        "e2e": {"value": total / (e2e_ms * 1e-3), "unit": "LPs/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
                "step_ms_all": [round(t * 1e3, 3) for t in e2e_times],
                "call": "blpg_solve_batch", "chunks": int(N.lib().blpg_solve_batch_chunks())},
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "gpu_launches": launches * args.steps,
        "step_ms_all": times,
    }
    print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
