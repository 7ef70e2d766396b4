"""Python front end of the GPU solver (calls the C ABI of libblpg.so).

``solve`` is the synchronous host-buffer path (blpg_solve_batch).  ``Plan``
wraps blpg_plan_create / blpg_plan_execute for device-resident data (torch
CUDA tensors): the size classes, queues and CUDA graph are built once and the
solve is enqueued on the current torch stream.  ``Simplex`` mirrors the
reference's host class (BLPG-Solver/src/simplex.cuh:37-83) name for name.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _native as N
from .lp import LPBatch

PRECISIONS = {"fp64": N.BLPG_FP64, "fp32": N.BLPG_FP32}


@dataclass
class SolveResult:
    status: np.ndarray
    objective: np.ndarray
    pivots: Optional[np.ndarray] = None
    x: Optional[np.ndarray] = None
    basis: Optional[np.ndarray] = None
    info: Optional[np.ndarray] = None


PRICING = {"dantzig": 0, "steepest": 1}


def options(precision: str = "fp64", **kw) -> N.Options:
    """blpg_options for `precision` ("fp64" | "fp32"); keyword arguments set
    fields by name (pricing also takes "dantzig" | "steepest")."""
    o = N.Options()
    N.lib().blpg_options_init(C.byref(o))
    o.precision = PRECISIONS[precision]
    for k, v in kw.items():
        if v is None:
            continue
        if k == "pricing" and isinstance(v, str):
            v = PRICING[v]
        if not hasattr(o, k):
            raise TypeError(f"unknown option {k}")
        setattr(o, k, v)
    return o


def solve(batch: LPBatch, precision: str = "fp64", want_x: bool = False,
          want_basis: bool = False, hint: Optional[np.ndarray] = None,
          weight: Optional[np.ndarray] = None, **opts) -> SolveResult:
    """Solve every LP of a host batch on the GPU (blocking).  `hint` (optional)
    is a packed array of m[k] basic column ids per LP (a warm-start basis);
    `weight` (optional, with pricing="steepest") n[k] + m[k] score factors
    per LP, packed."""
    L = N.lib()
    k = batch.count
    st = np.zeros(k, np.int32)
    ob = np.zeros(k, np.float64)
    pv = np.zeros(k, np.int32)
    info = np.zeros(k, np.int32)
    _, _, oc = batch.offsets()
    x = np.zeros(int(max((oc + batch.n).max(), 0)) if k else 0) if want_x else None
    bs = np.zeros(int(batch.m.sum()), np.int32) if want_basis else None
    res = N.Result(N.ptr(st, C.c_int32), N.ptr(ob, C.c_double), N.ptr(x, C.c_double),
                   N.ptr(pv, C.c_int32), N.ptr(bs, C.c_int32), N.ptr(info, C.c_int32))
    o = options(precision, **opts)
    if hint is not None:
        hint = np.ascontiguousarray(hint, dtype=np.int32)
        if hint.size != int(batch.m.sum()):
            raise ValueError("hint must hold m[k] column ids per LP")
        o.basis_hint = N.ptr(hint, C.c_int32)
    if weight is not None:
        weight = np.ascontiguousarray(weight, dtype=np.float32)
        if weight.size != int((batch.n + batch.m).sum()):
            raise ValueError("weight must hold n[k] + m[k] factors per LP")
        o.price_weight = N.ptr(weight, C.c_float)
    bst = batch.c_struct()
    N.check(L.blpg_solve_batch(C.byref(bst), C.byref(o), C.byref(res)), "blpg_solve_batch")
    return SolveResult(st, ob, pv, x, bs, info)


class Plan:
    """A reusable plan for one batch shape on device-resident data."""

    def __init__(self, batch: LPBatch, precision: str = "fp64", **opts):
        self._L = N.lib()
        self.batch = batch
        self.precision = precision
        self._opts = options(precision, **opts)
        h = C.c_void_p()
        # shapes, offsets and b (for the phase-I column counts) are read here
        bst = batch.c_struct()
        bst.A = None
        bst.c = None
        N.check(self._L.blpg_plan_create(C.byref(bst), C.byref(self._opts), C.byref(h)),
                "blpg_plan_create")
        self._h = h

    @property
    def handle(self):
        return self._h

    def classes(self):
        out = []
        for i in range(self._L.blpg_plan_num_classes(self._h)):
            K, nt, sm, cnt = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
            N.check(self._L.blpg_plan_class_info(self._h, i, C.byref(K), C.byref(nt),
                                                 C.byref(sm), C.byref(cnt)), "class_info")
            per_sm, grid = C.c_int32(), C.c_int32()
            N.check(self._L.blpg_plan_class_residency(self._h, i, C.byref(per_sm), C.byref(grid)),
                    "class_residency")
            key = C.c_int32()
            N.check(self._L.blpg_plan_class_key(self._h, i, C.byref(key), None), "class_key")
            out.append(dict(cluster=K.value, threads=nt.value, smem=sm.value, lps=cnt.value,
                            ctas_per_sm=per_sm.value, grid=grid.value, key=key.value))
        return out

    def launches(self) -> int:
        return int(self._L.blpg_plan_launches(self._h))

    def execute(self, dA: int, db: int, dc: int, status: int, objective: int, x: int = 0,
                pivots: int = 0, basis: int = 0, stream: int = 0, basis_hint: int = 0,
                info: int = 0, weight: int = 0) -> None:
        """Enqueue a solve on raw device pointers (ints) on `stream`."""
        res = N.Result(C.cast(status, N.i32p), C.cast(objective, N.f64p),
                       C.cast(x, N.f64p) if x else None, C.cast(pivots, N.i32p) if pivots else None,
                       C.cast(basis, N.i32p) if basis else None,
                       C.cast(info, N.i32p) if info else None)
        N.check(self._L.blpg_plan_execute_weighted(self._h, dA, db, dc, basis_hint or None,
                                                   weight or None, C.byref(res), stream or None),
                "blpg_plan_execute")

    def close(self):
        if self._h:
            self._L.blpg_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceBatch:
    """A batch's A, b, c and outputs resident in HBM (torch CUDA tensors),
    with a Plan; ``run()`` enqueues one solve on the current torch stream."""

    def __init__(self, batch: LPBatch, precision: str = "fp64", want_x=False, want_basis=False,
                 device: str = "cuda:0", **opts):
        import torch
        self.torch = torch
        self.batch = batch
        self.plan = Plan(batch, precision, **opts)
        dev = torch.device(device)
        self.A = torch.from_numpy(batch.A).to(dev)
        self.b = torch.from_numpy(batch.b).to(dev)
        self.c = torch.from_numpy(batch.c).to(dev)
        k = batch.count
        _, _, oc = batch.offsets()
        self.status = torch.zeros(k, dtype=torch.int32, device=dev)
        self.objective = torch.zeros(k, dtype=torch.float64, device=dev)
        self.pivots = torch.zeros(k, dtype=torch.int32, device=dev)
        self.x = (torch.zeros(int((oc + batch.n).max()), dtype=torch.float64, device=dev)
                  if want_x else None)
        self.basis = (torch.zeros(int(batch.m.sum()), dtype=torch.int32, device=dev)
                      if want_basis else None)
        self.info = torch.zeros(k, dtype=torch.int32, device=dev)

    def run(self, stream=None, hint=None, weight=None) -> None:
        """Enqueue one solve; `hint` is an optional int32 CUDA tensor of m[k]
        basic column ids per LP (a warm-start basis), `weight` an optional
        float32 CUDA tensor of n[k] + m[k] steepest-edge score factors per LP."""
        torch = self.torch
        s = stream if stream is not None else torch.cuda.current_stream()
        self.plan.execute(self.A.data_ptr(), self.b.data_ptr(), self.c.data_ptr(),
                          self.status.data_ptr(), self.objective.data_ptr(),
                          self.x.data_ptr() if self.x is not None else 0,
                          self.pivots.data_ptr(),
                          self.basis.data_ptr() if self.basis is not None else 0,
                          stream=s.cuda_stream,
                          basis_hint=hint.data_ptr() if hint is not None else 0,
                          info=self.info.data_ptr(),
                          weight=weight.data_ptr() if weight is not None else 0)

    def result(self) -> SolveResult:
        self.torch.cuda.synchronize()
        return SolveResult(self.status.cpu().numpy(), self.objective.cpu().numpy(),
                           self.pivots.cpu().numpy(),
                           self.x.cpu().numpy() if self.x is not None else None,
                           self.basis.cpu().numpy() if self.basis is not None else None,
                           self.info.cpu().numpy())


class Simplex:
    """Mirror of the reference's host class (simplex.cuh:37-83): one A, b for
    the batch, one objective per LP (max sense), results by LP, 1-based
    single-LP accessors.  Status codes: 5 optimal, 6 unbounded, 4 infeasible,
    1 pivot cap (the reference only reports 2 or 6, simplex.cu:451-461)."""

    def __init__(self, N_S: int, multipleBatch: int = 0):
        self.number_of_LPs = int(N_S)
        self.multipleBatchOn = int(multipleBatch)
        self._A = None
        self._b = None
        self._res: Optional[SolveResult] = None

    def setConstratint(self, A, B) -> None:  # (sic) the reference's spelling
        self._A = np.asarray(A, dtype=np.float64)
        self._b = np.asarray(B, dtype=np.float64)

    def ComputeLP(self, C_rows, number_of_streams: int = 1, precision: str = "fp64") -> None:
        # number_of_streams is accepted for signature parity; the plan's one
        # persistent launch per size class replaces the reference's stream split.
        C_rows = np.atleast_2d(np.asarray(C_rows, dtype=np.float64))
        if self._A is None:
            raise RuntimeError("setConstratint must be called before ComputeLP")
        batch = LPBatch.shared(self._A, self._b, C_rows)
        self._res = solve(batch, precision=precision)

    def getResultAll(self) -> np.ndarray:
        return self._res.objective.copy()

    def getStatusAll(self) -> np.ndarray:
        return self._res.status.copy()

    def getResult(self, n: int) -> float:
        return float(self._res.objective[n - 1])

    def getStatus(self, n: int) -> int:
        return int(self._res.status[n - 1])

    def getNo_OF_Simplx(self) -> int:
        return self.number_of_LPs
