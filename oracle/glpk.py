"""GLPK 4.45 harness — TEST INFRASTRUCTURE ONLY (fixture generation).

The reference judges its GPU results against GLPK 4.45 (ReadMe:26): each LP
becomes one problem object with rows ``GLP_UP`` (a_i x <= b_i), columns
``GLP_LO`` (x >= 0), the objective set per LP and ``glp_simplex`` run with
default parameters (glpk_lp_solver.cpp:243-286, :435-454, GPU_Tester.cu:154-164).
``glp_exact`` (GMP rationals, same library) is the exact arbiter.

GLPK is third-party and not in the reference's sources: only its prebuilt
x86-64 shared library ships (lib/libglpk.so.0.30.0, version string "4.45").
It is loaded with ctypes and called through its public API, declared here by
hand from GLPK's reference manual (no glpk.h is available).  The library is
x86-64 only, so this module runs in the x86 container: it generates the
committed fixtures in tests/golden/, and is never needed on the GPU host.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

REFERENCE = os.environ.get("BLPG_REFERENCE", "/root/reference")
DEFAULT_LIB = os.environ.get("BLPG_GLPK_LIB", os.path.join(REFERENCE, "lib", "libglpk.so.0.30.0"))

GLP_MAX = 2
GLP_LO, GLP_UP = 2, 3
GLP_OFF = 0
# glp_get_status codes
GLP_UNDEF, GLP_FEAS, GLP_INFEAS, GLP_NOFEAS, GLP_OPT, GLP_UNBND = 1, 2, 3, 4, 5, 6

_lib = None


def available(path: str = DEFAULT_LIB) -> bool:
    try:
        lib(path)
        return True
    except OSError:
        return False


def lib(path: str = DEFAULT_LIB):
    global _lib
    if _lib is None:
        L = C.CDLL(path)
        vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
        sig = {
            "glp_create_prob": (vp, []),
            "glp_delete_prob": (None, [vp]),
            "glp_set_obj_dir": (None, [vp, C.c_int]),
            "glp_add_rows": (C.c_int, [vp, C.c_int]),
            "glp_add_cols": (C.c_int, [vp, C.c_int]),
            "glp_set_row_bnds": (None, [vp, C.c_int, C.c_int, C.c_double, C.c_double]),
            "glp_set_col_bnds": (None, [vp, C.c_int, C.c_int, C.c_double, C.c_double]),
            "glp_set_obj_coef": (None, [vp, C.c_int, C.c_double]),
            "glp_load_matrix": (None, [vp, C.c_int, ip, ip, dp]),
            "glp_simplex": (C.c_int, [vp, vp]),
            "glp_exact": (C.c_int, [vp, vp]),
            "glp_get_status": (C.c_int, [vp]),
            "glp_get_obj_val": (C.c_double, [vp]),
            "glp_get_col_prim": (C.c_double, [vp, C.c_int]),
            "glp_get_row_stat": (C.c_int, [vp, C.c_int]),
            "glp_get_col_stat": (C.c_int, [vp, C.c_int]),
            "glp_term_out": (C.c_int, [C.c_int]),
            "glp_version": (C.c_char_p, []),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


GLP_BS = 1  # basic (glp_get_row_stat / glp_get_col_stat)


def solve(A, b, c, exact: bool = False, want_x: bool = False):
    """max c^T x, A x <= b, x >= 0 with glp_simplex (defaults) and, if
    `exact`, glp_exact from the final basis.  Returns a dict with status,
    objective, the final basis as column ids (0..n-1 structural, n+i for the
    slack of row i) and optionally x."""
    L = lib()
    L.glp_term_out(GLP_OFF)
    A = np.asarray(A, dtype=np.float64)
    m, n = A.shape
    P = L.glp_create_prob()
    try:
        L.glp_set_obj_dir(P, GLP_MAX)
        L.glp_add_rows(P, m)
        L.glp_add_cols(P, n)
        for i in range(m):
            L.glp_set_row_bnds(P, i + 1, GLP_UP, 0.0, float(b[i]))
        for j in range(n):
            L.glp_set_col_bnds(P, j + 1, GLP_LO, 0.0, 0.0)
            L.glp_set_obj_coef(P, j + 1, float(c[j]))
        rows, cols = np.nonzero(A)
        ne = len(rows)
        ia = (C.c_int * (ne + 1))(0, *(rows + 1).tolist())
        ja = (C.c_int * (ne + 1))(0, *(cols + 1).tolist())
        ar = (C.c_double * (ne + 1))(0.0, *A[rows, cols].tolist())
        L.glp_load_matrix(P, ne, ia, ja, ar)
        ret = L.glp_simplex(P, None)
        out = {"ret": ret, "status": L.glp_get_status(P), "objective": L.glp_get_obj_val(P)}
        basis = [j for j in range(n) if L.glp_get_col_stat(P, j + 1) == GLP_BS]
        basis += [n + i for i in range(m) if L.glp_get_row_stat(P, i + 1) == GLP_BS]
        out["basis"] = basis
        if exact:
            rete = L.glp_exact(P, None)
            out["exact_ret"] = rete
            out["exact_status"] = L.glp_get_status(P)
            out["exact_objective"] = L.glp_get_obj_val(P)
        if want_x:
            out["x"] = [L.glp_get_col_prim(P, j + 1) for j in range(n)]
        return out
    finally:
        L.glp_delete_prob(P)


def solve_batch(batch, exact: bool = False, limit: Optional[int] = None):
    out = []
    k = batch.count if limit is None else min(limit, batch.count)
    for i in range(k):
        A, b, c = batch.lp(i)
        out.append(solve(A, b, c, exact=exact))
    return out
