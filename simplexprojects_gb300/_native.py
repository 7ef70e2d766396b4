"""ctypes binding of libblpg.so (the C ABI declared in include/blpg.h).

The library is built in-tree by ``simplexprojects_gb300.build`` into
``simplexprojects_gb300/lib/libblpg.so``.  Loading fails loudly when it is
missing: there is no Python or CPU fallback for any solve entry point.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libblpg.so"

BLPG_UNDEF, BLPG_FEAS, BLPG_INFEAS, BLPG_NOFEAS, BLPG_OPT, BLPG_UNBND = 1, 2, 3, 4, 5, 6
BLPG_FP64, BLPG_FP32 = 0, 1
ERRORS = {
    -1: "BLPG_EINVAL", -2: "BLPG_ENODEV", -3: "BLPG_ECUDA", -4: "BLPG_ENOMEM",
    -5: "BLPG_ETOOBIG", -6: "BLPG_EIO", -7: "BLPG_ESTATE",
}

i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)
f64p = C.POINTER(C.c_double)


class Batch(C.Structure):
    _fields_ = [
        ("count", C.c_int32), ("m", i32p), ("n", i32p),
        ("off_A", i64p), ("off_b", i64p), ("off_c", i64p),
        ("A", f64p), ("b", f64p), ("c", f64p),
    ]


class Options(C.Structure):
    _fields_ = [
        ("precision", C.c_int32), ("max_pivots", C.c_int32), ("bland_after", C.c_int32),
        ("refactor_period", C.c_int32), ("opt_tol", C.c_double), ("piv_tol", C.c_double),
        ("basis_hint", i32p), ("device", C.c_int32), ("use_graph", C.c_int32),
        ("threads_per_cta", C.c_int32), ("max_cluster", C.c_int32), ("min_cluster", C.c_int32),
        ("cta_smem_budget", C.c_int32), ("ratio_rule", C.c_int32), ("feas_tol", C.c_double),
        ("warm_mode", C.c_int32), ("pricing", C.c_int32), ("price_weight", C.POINTER(C.c_float)),
    ]


class Result(C.Structure):
    _fields_ = [
        ("status", i32p), ("objective", f64p), ("x", f64p), ("pivots", i32p), ("basis", i32p),
        ("info", i32p),
    ]


# Every exported symbol of include/blpg.h with its signature.
SIGNATURES = {
    "blpg_options_init": (None, [C.POINTER(Options)]),
    "blpg_solve_batch": (C.c_int32, [C.POINTER(Batch), C.POINTER(Options), C.POINTER(Result)]),
    "blpg_solve_batch_chunks": (C.c_int32, []),
    "blpg_release_workspace": (C.c_int32, []),
    "blpg_plan_create": (C.c_int32, [C.POINTER(Batch), C.POINTER(Options), C.POINTER(C.c_void_p)]),
    "blpg_plan_execute": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.POINTER(Result), C.c_void_p]),
    "blpg_price_weights": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                       C.c_int32, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p]),
    "blpg_plan_execute_weighted": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                               C.c_void_p, C.c_void_p, C.POINTER(Result),
                                               C.c_void_p]),
    "blpg_plan_num_classes": (C.c_int32, [C.c_void_p]),
    "blpg_plan_class_info": (C.c_int32, [C.c_void_p, C.c_int32, i32p, i32p, i32p, i32p]),
    "blpg_plan_class_residency": (C.c_int32, [C.c_void_p, C.c_int32, i32p, i32p]),
    "blpg_plan_launches": (C.c_int32, [C.c_void_p]),
    "blpg_plan_class_key": (C.c_int32, [C.c_void_p, C.c_int32, i32p, i32p]),
    "blpg_plan_destroy": (None, [C.c_void_p]),
    "blpg_set_tuning": (C.c_int32, [C.c_char_p]),
    "blpg_last_error": (C.c_char_p, []),
    "blpg_version": (C.c_char_p, []),
    "blpg_measure_peaks": (C.c_int32, [C.c_int32, f64p, f64p, f64p]),
    "blpg_round_f32": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p]),
    "blpg_solve_noalloc": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32] + [C.c_void_p] * 8
                           + [C.c_int32] + [C.c_void_p] * 5),
    "blpg_mlp_create": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                    C.c_uint64, C.POINTER(C.c_void_p)]),
    "blpg_mlp_destroy": (None, [C.c_void_p]),
    "blpg_mlp_dims": (C.c_int32, [C.c_void_p, i32p, i32p]),
    "blpg_mlp_num_params": (C.c_int64, [C.c_void_p]),
    "blpg_mlp_get_params": (C.c_int32, [C.c_void_p, C.POINTER(C.c_float)]),
    "blpg_mlp_set_params": (C.c_int32, [C.c_void_p, C.POINTER(C.c_float)]),
    "blpg_mlp_train_step": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_float,
                                        C.POINTER(C.c_float), C.c_void_p]),
    "blpg_mlp_predict": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "blpg_mlp_gradients": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                       C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "blpg_features": (C.c_int32, [C.c_int32] * 4 + [C.c_void_p] * 8 + [C.c_int32, C.c_void_p]),
    "blpg_learned_create": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(C.c_float),
                                        C.POINTER(C.c_float), C.c_float, C.POINTER(Batch),
                                        C.POINTER(Options), C.POINTER(C.c_void_p)]),
    "blpg_learned_solve": (C.c_int32, [C.c_void_p, C.POINTER(Batch), C.POINTER(C.c_int32),
                                       C.POINTER(Result)]),
    "blpg_learned_destroy": (None, [C.c_void_p]),
    "blpg_topm_hint": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                   C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "blpg_read_abc": (C.c_int32, [C.c_char_p, C.c_char_p, C.c_char_p, i32p, i32p, f64p, f64p, f64p]),
    "blpg_write_batch": (C.c_int32, [C.c_char_p, C.POINTER(Batch)]),
    "blpg_read_batch": (C.c_int32, [C.c_char_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                    C.POINTER(C.c_int64), C.POINTER(C.c_int64), i32p, i32p,
                                    C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                    C.POINTER(C.c_int64), f64p, f64p, f64p]),
    "blpg_write_results": (C.c_int32, [C.c_char_p, C.POINTER(Batch), C.POINTER(Result)]),
    "blpg_gen_shapes": (C.c_int64, [C.c_int32, C.c_int64, C.c_int32, C.c_uint64, i32p, i32p, i32p]),
    "blpg_gen_fill": (C.c_int32, [C.c_int32, C.c_int64, C.c_int32, C.c_uint64, i32p, i32p, f64p,
                                  f64p, f64p, C.c_int32]),
}

_lib = None
_lock = threading.Lock()


class BlpgError(RuntimeError):
    def __init__(self, code: int, where: str):
        msg = lib().blpg_last_error().decode(errors="replace")
        super().__init__(f"{where}: {ERRORS.get(code, code)}: {msg}")
        self.code = code


def lib() -> C.CDLL:
    """Load libblpg.so once; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(
                    f"{LIB_PATH} is missing: build it with "
                    "`python -c 'import __graft_entry__ as g; g.build()'` "
                    "(no CPU fallback exists)")
            L = C.CDLL(str(LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(rc: int, where: str) -> None:
    if rc != 0:
        raise BlpgError(rc, where)


def ptr(a, ctype):
    """ctypes pointer to a numpy array's data (None for None)."""
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))
