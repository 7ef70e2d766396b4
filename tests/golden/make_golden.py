"""Generate the committed golden fixtures (tests/golden/*.json).

Runs in the x86 container only: it calls GLPK 4.45 from the reference's
prebuilt lib/libglpk.so.0.30.0 (glp_simplex with default parameters, as the
reference's glpk_lp_solver.cpp:435-454).  The exact verdict of each LP is an
exact certificate: GLPK's final basis is proven optimal by solving
B x_B = b and B^T y = c_B in rational arithmetic and checking the signs of
x_B and of every reduced cost (oracle/exact.py), or unboundedness is proven
by a column with no positive entry and a positive cost; glp_exact (GMP) is
used for the small hand LPs.  The LP data itself is not stored: every
fixture names the workload kind, seed and LP indices, and a SHA-256 of the
generated A, b, c so that a change of the generator is caught.

Fixtures:
  workloads.json   per workload kind 0..4, a sample of seeded LPs with GLPK's
                   status/objective and the exact status/objective
  known.json       the reference's hand LPs (parseBenchmark.cpp:128-319,
                   GPU_Tester.cu:80-86) and the 8 Netlib LPs it ships
                   (benchmarks/*.txt, listed optima parseBenchmark.cpp:15-25),
                   solved by GLPK with exact verdicts
  netlib/          byte-for-byte copies of those 8 Netlib LPs' A/B/C text
                   files (public Netlib data in the reference's dense format,
                   parseBenchmark.cpp:59-126), so that the GPU tests and the
                   reference-compatible CLI can solve them where the
                   reference checkout is absent

The reference checkout is read from $BLPG_REFERENCE (default /root/reference).

Usage:  python tests/golden/make_golden.py [--quick] [--known-only] [--netlib-copy]
"""
from __future__ import annotations

import argparse
import hashlib
import json
import multiprocessing as mp
import os
import shutil
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

SEED = 20240611
# (kind, first, count): LP indices of each workload's sample
SAMPLES = {0: (0, 48), 1: (0, 40), 2: (0, 3), 3: (39_990, 6), 4: (0, 40)}
REF = Path(os.environ.get("BLPG_REFERENCE", "/root/reference"))
NETLIB = ["ADLITTLE", "AFIRO", "BLEND", "ISRAEL", "SC105", "SC205", "SC50A", "SC50B"]
# listed optima of the minimisation files (parseBenchmark.cpp:15-25)
NETLIB_LISTED = {
    "ADLITTLE": 2.2549496316e05, "AFIRO": -4.6475314286e02, "BLEND": -3.0812149846e01,
    "ISRAEL": -8.9664482186e05, "SC105": -5.2202061212e01, "SC205": -5.2202061212e01,
    "SC50A": -6.4575077059e01, "SC50B": -7.0000000000e01,
}


def hand_lps():
    """The reference's hand-written LPs (max c^T x, A x <= b, x >= 0), with the
    answers its comments state (None where the comment is wrong or absent)."""
    lps = {
        # parseSmallLP, parseBenchmark.cpp:128-148 ("unbounded ... at 2")
        "SmallLP": ([[2, -1], [1, -5]], [2, -4], [2, -1], None),
        # parseSmallLP2, :151-173, "has solution 39.44444"
        "SmallLP2": ([[1, 1], [-1, 1], [5, 4]], [10, -3, 35], [5, 6], 39.44444),
        # parseSmallLP3, :175-197, "has solution 21.33333"
        "SmallLP3": ([[1, -1], [-1, -1], [-1, 4]], [8, -3, 2], [1, 3], 21.33333),
        # parseSmallLP4, :199-221, "has solution 9.33333"
        "SmallLP4": ([[1, 1, -1], [-3, 1, 0], [1, -2, -2]], [7, -8, 0], [2, 0, -6], 9.33333),
        # parseSmallLP5, :223-245 (its comment repeats LP2's value)
        "SmallLP5": ([[4, -1], [2, 1], [-5, 2]], [8, 10, 2], [1, 1], None),
    }
    # parse5Dim, :252-277: box 0.99 <= x1 <= 1.01, |x_i| <= 0.01 otherwise
    A5 = np.zeros((10, 5))
    for i in range(5):
        A5[2 * i, i] = 1
        A5[2 * i + 1, i] = -1
    b5 = [1.01, -0.99] + [0.01] * 8
    lps["FiveDim_x1"] = (A5.tolist(), b5, [1, 0, 0, 0, 0], 1.01)
    lps["FiveDim_x2"] = (A5.tolist(), b5, [0, 1, 0, 0, 0], None)
    # parse28DimHelicopter, :282-319
    AH = np.zeros((56, 28))
    bH = np.zeros(56)
    for i in range(28):
        AH[2 * i, i] = 1
        AH[2 * i + 1, i] = -1
        if i < 8:
            bH[2 * i] = 0.1
    cH = np.zeros(28)
    cH[0] = 1
    lps["Helicopter28"] = (AH.tolist(), bH.tolist(), cH.tolist(), None)
    return lps


def fingerprint(batch) -> str:
    h = hashlib.sha256()
    for a in (batch.m, batch.n, batch.A, batch.b, batch.c):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def _solve_one(args):
    """GLPK (glp_simplex, default parameters) and an exact verdict: the exact
    optimality certificate of GLPK's final basis (oracle/exact.py: rational
    solves of B x_B = b and B^T y = c_B, sign checks of x_B and of every
    reduced cost), an exact unbounded ray, or glp_exact for small LPs."""
    A, b, c = args
    from oracle import exact, glpk
    m = len(A)
    small = m <= 40
    r = glpk.solve(np.asarray(A), np.asarray(b), np.asarray(c), exact=small)
    out = {"status": r["status"], "objective": r["objective"]}
    est, eobj, how = None, None, None
    if r["status"] == glpk.GLP_OPT:
        ok, obj = exact.certify(A, b, c, r["basis"])
        if ok:
            est, eobj, how = 5, float(obj), "certificate"
    if est is None and r["status"] == glpk.GLP_UNBND and exact.unbounded_ray(A, c):
        est, how = 6, "ray"
    if est is None and small:
        est, eobj, how = r["exact_status"], r["exact_objective"], "glp_exact"
    if est is None:
        st, obj = exact.solve(A, b, c) if m <= 60 else (None, None)
        if st is not None:
            est, eobj, how = st, (float(obj) if obj is not None else None), "fraction_simplex"
    out.update(exact_status=est, exact_objective=eobj, exact_method=how)
    return out


def copy_netlib() -> list[str]:
    """Copy the reference's Netlib A/B/C files into tests/golden/netlib/."""
    dst = HERE / "netlib"
    dst.mkdir(exist_ok=True)
    copied = []
    for nm in NETLIB:
        srcs = [REF / "benchmarks" / f"{nm}_{s}.txt" for s in "ABC"]
        if not all(p.exists() for p in srcs):
            continue
        for p in srcs:
            shutil.copyfile(p, dst / p.name)
        copied.append(nm)
    return copied


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true", help="smaller samples (smoke the script)")
    ap.add_argument("--procs", type=int, default=8)
    ap.add_argument("--known-only", action="store_true", help="regenerate known.json only")
    ap.add_argument("--netlib-copy", action="store_true",
                    help="only copy the Netlib A/B/C files into tests/golden/netlib/")
    args = ap.parse_args()
    print("netlib files copied:", copy_netlib())
    if args.netlib_copy:
        return
    import simplexprojects_gb300 as sp
    from oracle import glpk
    if not glpk.available():
        sys.exit("GLPK library not found (the reference's lib/ is needed)")
    ctx = mp.get_context("spawn")
    t0 = time.time()
    out = {"seed": SEED, "glpk_version": glpk.lib().glp_version().decode(), "workloads": {}}
    with ctx.Pool(args.procs) as pool:
        for kind, (first, count) in ({} if args.known_only else SAMPLES).items():
            if args.quick:
                count = min(count, 4)
            batch = sp.generate(kind, count, seed=SEED, first=first)
            jobs = [batch.lp(k) for k in range(count)]
            res = pool.map(_solve_one, [(A.tolist(), b.tolist(), c.tolist()) for A, b, c in jobs])
            out["workloads"][str(kind)] = {
                "first": first, "count": count, "sha256": fingerprint(batch),
                "m": batch.m.tolist(), "n": batch.n.tolist(), "lps": res,
            }
            print(f"kind {kind}: {count} LPs, {time.time() - t0:.0f}s", flush=True)
        if not args.known_only:
            (HERE / "workloads.json").write_text(json.dumps(out, indent=1))
        known = {"hand": {}, "netlib": {}}
        for name, (A, b, c, stated) in hand_lps().items():
            r = _solve_one((A, b, c))
            known["hand"][name] = dict(r, A=A, b=b, c=c, stated=stated)
        names = [nm for nm in NETLIB if (REF / "benchmarks" / f"{nm}_A.txt").exists()]
        jobs = []
        for nm in names:
            A, b, c = sp.read_abc(*(str(REF / "benchmarks" / f"{nm}_{s}.txt") for s in "ABC"))
            jobs.append((A.tolist(), b.tolist(), (-c).tolist()))  # max form (GPU_Tester.cu:119-127)
        res = pool.map(_solve_one, jobs)
        for nm, (A, b, c), r in zip(names, jobs, res):
            Aa = np.asarray(A)
            known["netlib"][nm] = dict(r, m=Aa.shape[0], n=Aa.shape[1],
                                       negative_b=int((np.asarray(b) < 0).sum()),
                                       listed_min=NETLIB_LISTED[nm])
        (HERE / "known.json").write_text(json.dumps(known, indent=1))
    print(f"done in {time.time() - t0:.0f}s")


if __name__ == "__main__":
    main()
