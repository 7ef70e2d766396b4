"""simplexprojects_gb300 — batched dense-tableau LP solver for one GB300 GPU.

Public API:
    generate(kind, count, seed)     synthetic workloads 0..4 (include/blpg.h)
    read_abc(A, B, C)               the reference's dense text files
    write_batch, read_batch         a whole batch in one binary file
    write_results                   per-LP status, objective and x as text
    solve(batch, precision)         blocking host-buffer solve (C ABI)
    Plan, DeviceBatch               plans on device-resident data
    Simplex                         mirror of the reference's host class
"""
from . import _native
from ._native import BlpgError
from .lp import (LPBatch, generate, read_abc, read_batch, shard, write_batch, write_results,
                 WORKLOAD_COUNTS, DEFAULT_SEED)
from .solver import DeviceBatch, Plan, Simplex, SolveResult, options, solve

__all__ = [
    "LPBatch", "generate", "read_abc", "read_batch", "write_batch", "write_results", "solve", "Plan",
    "DeviceBatch", "Simplex", "SolveResult",
    "options", "WORKLOAD_COUNTS", "DEFAULT_SEED", "BlpgError", "shard",
]


def version() -> str:
    return _native.lib().blpg_version().decode()
