"""A small, self-contained solve for kernel profiling.

Generates `count` LPs of workload `kind` (the seeded generator behind
include/blpg.h, families sharing A), builds a device-resident batch, and runs
the solve twice (one warm-up, one capture target), then prints the class plan,
the status histogram and the pivot total. It holds a few MB on the device, so
a full-metric capture of one solve_kernel launch ends within a minute:

    python -m simplexprojects_gb300.profile_case 3 304 fp32 steepest
    ncu --set full --clock-control none -k regex:solve_kernel -s 1 -c 1 \
        -o prof python -m simplexprojects_gb300.profile_case 3 304 fp32 steepest

Arguments: workload kind, LP count, precision (fp64 | fp32), pricing
(dantzig | steepest; default dantzig).
"""
from __future__ import annotations

import sys

import numpy as np


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    kind = int(argv[0]) if len(argv) > 0 else 1
    count = int(argv[1]) if len(argv) > 1 else 1500
    prec = argv[2] if len(argv) > 2 else "fp64"
    pricing = argv[3] if len(argv) > 3 else "dantzig"
    from .lp import DEFAULT_SEED, generate
    from .solver import DeviceBatch
    batch = generate(kind, count, seed=DEFAULT_SEED, share_family_A=True)
    db = DeviceBatch(batch, prec, pricing=pricing)
    for _ in range(2):
        db.run()
    r = db.result()
    print("classes", db.plan.classes())
    print("status", np.bincount(r.status).tolist(), "pivots", int(r.pivots.sum()))
    db.plan.close()


if __name__ == "__main__":
    main()
