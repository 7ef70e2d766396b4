"""ctypes binding of the CPU oracle (oracle/cpu_ref.c).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA solver and the timed CPU
baseline.  Built by simplexprojects_gb300.build.build_oracle().
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from pathlib import Path
from typing import Optional

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libblpg_oracle.so"

OPT, UNBND, NOFEAS, UNDEF = 5, 6, 4, 1


class Opts(C.Structure):
    _fields_ = [
        ("precision", C.c_int), ("max_pivots", C.c_int), ("bland_after", C.c_int),
        ("refactor_period", C.c_int), ("opt_tol", C.c_double), ("piv_tol", C.c_double),
        ("phase1_tol", C.c_double), ("deg_tol", C.c_double), ("feas_tol", C.c_double),
        ("harris", C.c_int), ("ptol", C.c_double), ("composite", C.c_int),
        ("shift", C.c_double), ("pricing", C.c_int), ("weight", C.POINTER(C.c_float)),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} missing: run simplexprojects_gb300.build.build_oracle()")
        L = C.CDLL(str(LIB_PATH))
        L.oref_opts_init.argtypes = [C.POINTER(Opts), C.c_int]
        L.oref_opts_init.restype = None
        ip, lp, dp = C.POINTER(C.c_int), C.POINTER(C.c_int64), C.POINTER(C.c_double)
        L.oref_solve_batch.argtypes = [C.c_int, ip, ip, lp, lp, lp, dp, dp, dp, C.POINTER(Opts),
                                       C.c_int, ip, ip, dp, dp, ip, ip, ip,
                                       C.POINTER(C.c_float)]
        L.oref_solve_batch.restype = C.c_int
        L.oref_solve_one.argtypes = [C.c_int, C.c_int, dp, dp, dp, C.POINTER(Opts), ip, dp, dp, ip,
                                     ip, ip]
        L.oref_solve_one.restype = C.c_int
        _lib = L
    return _lib


PRICING = {"dantzig": 0, "steepest": 1}


def opts(precision: str = "fp64", **kw) -> Opts:
    o = Opts()
    lib().oref_opts_init(C.byref(o), 1 if precision == "fp32" else 0)
    for k, v in kw.items():
        if k == "pricing" and isinstance(v, str):
            v = PRICING[v]
        setattr(o, k, v)
    return o


@dataclass
class RefResult:
    status: np.ndarray
    objective: np.ndarray
    pivots: np.ndarray
    x: Optional[np.ndarray] = None
    basis: Optional[np.ndarray] = None
    info: Optional[np.ndarray] = None


def _p(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


def solve_batch(batch, precision: str = "fp64", threads: Optional[int] = None, want_x=False,
                want_basis=False, hint=None, weight=None, **kw) -> RefResult:
    """Solve a simplexprojects_gb300.LPBatch on the CPU with the oracle.
    `weight` (steepest-edge pricing only): n[k] + m[k] score factors per LP."""
    L = lib()
    k = batch.count
    m = batch.m.astype(np.int32)
    n = batch.n.astype(np.int32)
    oA, ob, oc = [np.ascontiguousarray(o, dtype=np.int64) for o in batch.offsets()]
    st = np.zeros(k, np.int32)
    obj = np.zeros(k)
    pv = np.zeros(k, np.int32)
    x = np.zeros(int((oc + n).max()) if k else 0) if want_x else None
    bs = np.zeros(int(m.sum()), np.int32) if want_basis else None
    info = np.zeros(k, np.int32)
    if hint is not None:
        hint = np.ascontiguousarray(hint, dtype=np.int32)
        assert hint.size == int(m.sum())
    if weight is not None:
        weight = np.ascontiguousarray(weight, dtype=np.float32)
        assert weight.size == int((m + n).sum())
    o = opts(precision, **kw)
    if threads is None:
        threads = os.cpu_count() or 1
    rc = L.oref_solve_batch(k, _p(m, C.c_int), _p(n, C.c_int), _p(oA, C.c_int64),
                            _p(ob, C.c_int64), _p(oc, C.c_int64), _p(batch.A, C.c_double),
                            _p(batch.b, C.c_double), _p(batch.c, C.c_double), C.byref(o),
                            int(threads), _p(hint, C.c_int), _p(st, C.c_int), _p(obj, C.c_double),
                            _p(x, C.c_double), _p(pv, C.c_int), _p(bs, C.c_int), _p(info, C.c_int),
                            _p(weight, C.c_float))
    if rc != 0:
        raise RuntimeError("oref_solve_batch failed")
    return RefResult(st, obj, pv, x, bs, info)
