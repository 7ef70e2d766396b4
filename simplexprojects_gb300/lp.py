"""LP batches: the host-side container, the synthetic workloads and the
reference's A/B/C text files.

A batch holds LP k as ``max c_k^T x  s.t.  A_k x <= b_k, x >= 0`` with A_k
row-major m_k x n_k.  Offsets let LPs share data: the reference's batch mode
(one A, b for the whole batch, one objective per LP; GPU_Tester.cu:119-127)
is ``off_A = off_b = 0`` for every LP, and the perturbed families of workload
3 share each family's A.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _native as N

# Workload sizes of the benchmark configurations (kind -> default count).
WORKLOAD_COUNTS = {0: 1024, 1: 10_000, 2: 2048, 3: 50_000, 4: 200_000}
DEFAULT_SEED = 20240611


@dataclass
class LPBatch:
    m: np.ndarray
    n: np.ndarray
    A: np.ndarray
    b: np.ndarray
    c: np.ndarray
    off_A: Optional[np.ndarray] = None
    off_b: Optional[np.ndarray] = None
    off_c: Optional[np.ndarray] = None
    family: Optional[np.ndarray] = None
    meta: dict = field(default_factory=dict)

    def __post_init__(self):
        self.m = np.ascontiguousarray(self.m, dtype=np.int32)
        self.n = np.ascontiguousarray(self.n, dtype=np.int32)
        self.A = np.ascontiguousarray(self.A, dtype=np.float64)
        self.b = np.ascontiguousarray(self.b, dtype=np.float64)
        self.c = np.ascontiguousarray(self.c, dtype=np.float64)
        for name in ("off_A", "off_b", "off_c"):
            v = getattr(self, name)
            if v is not None:
                setattr(self, name, np.ascontiguousarray(v, dtype=np.int64))

    @property
    def count(self) -> int:
        return int(self.m.shape[0])

    def offsets(self):
        """(off_A, off_b, off_c), computing packed offsets where absent."""
        def packed(sizes):
            out = np.zeros(sizes.size, np.int64)
            np.cumsum(sizes[:-1], out=out[1:])
            return out

        return (self.off_A if self.off_A is not None else
                packed(self.m.astype(np.int64) * self.n),
                self.off_b if self.off_b is not None else packed(self.m.astype(np.int64)),
                self.off_c if self.off_c is not None else packed(self.n.astype(np.int64)))

    def lp(self, k: int):
        """(A_k as an m x n array, b_k, c_k) for LP k."""
        oA, ob, oc = self.offsets()
        m, n = int(self.m[k]), int(self.n[k])
        A = self.A[oA[k]:oA[k] + m * n].reshape(m, n)
        return A, self.b[ob[k]:ob[k] + m], self.c[oc[k]:oc[k] + n]

    def head(self, k: int) -> "LPBatch":
        """The first k LPs, sharing this batch's arrays through offsets."""
        oA, ob, oc = self.offsets()
        fam = self.family[:k] if self.family is not None else None
        return LPBatch(self.m[:k], self.n[:k], self.A, self.b, self.c, off_A=oA[:k],
                       off_b=ob[:k], off_c=oc[:k], family=fam, meta=dict(self.meta, head=k))

    def subset(self, idx) -> "LPBatch":
        """A packed copy of the LPs listed in idx."""
        idx = np.asarray(idx, dtype=np.int64)
        As, bs, cs = [], [], []
        for k in idx:
            A, b, c = self.lp(int(k))
            As.append(A.ravel())
            bs.append(b)
            cs.append(c)
        fam = self.family[idx] if self.family is not None else None
        return LPBatch(self.m[idx], self.n[idx],
                       np.concatenate(As) if As else np.zeros(0),
                       np.concatenate(bs) if bs else np.zeros(0),
                       np.concatenate(cs) if cs else np.zeros(0), family=fam,
                       meta=dict(self.meta, subset=True))

    def __getstate__(self):
        """Pickled and deep-copied without the cached ctypes view."""
        state = dict(self.__dict__)
        state.pop("_c_struct", None)
        return state

    def c_struct(self) -> N.Batch:
        """ctypes view; the arrays must outlive the returned struct.  The view
        is kept with references to the arrays it points into and reused while
        the same array objects are in place (the references keep them alive,
        so a reused view never points at freed memory); each call returns its
        own copy of it, which the caller may change."""
        arrays = (self.m, self.n, self.off_A, self.off_b, self.off_c, self.A, self.b, self.c)
        cached = self.__dict__.get("_c_struct")
        if cached is not None and all(x is y for x, y in zip(cached[0], arrays)):
            return N.Batch.from_buffer_copy(cached[1])
        bst = N.Batch(self.count, N.ptr(self.m, C.c_int32), N.ptr(self.n, C.c_int32),
                      N.ptr(self.off_A, C.c_int64), N.ptr(self.off_b, C.c_int64),
                      N.ptr(self.off_c, C.c_int64), N.ptr(self.A, C.c_double),
                      N.ptr(self.b, C.c_double), N.ptr(self.c, C.c_double))
        self.__dict__["_c_struct"] = (arrays, bst)
        return N.Batch.from_buffer_copy(bst)

    def nbytes(self) -> int:
        return int(self.A.nbytes + self.b.nbytes + self.c.nbytes)

    @classmethod
    def from_lps(cls, lps) -> "LPBatch":
        """Packed batch from a list of (A, b, c)."""
        ms, ns, As, bs, cs = [], [], [], [], []
        for A, b, c in lps:
            A = np.asarray(A, dtype=np.float64)
            ms.append(A.shape[0])
            ns.append(A.shape[1])
            As.append(A.ravel())
            bs.append(np.asarray(b, dtype=np.float64))
            cs.append(np.asarray(c, dtype=np.float64))
        return cls(np.array(ms), np.array(ns), np.concatenate(As), np.concatenate(bs),
                   np.concatenate(cs))

    @classmethod
    def shared(cls, A, b, C_rows) -> "LPBatch":
        """The reference's batch mode: one A, b and one objective per LP
        (rows of C_rows), as Simplex::setConstratint + ComputeLP(C)."""
        A = np.asarray(A, dtype=np.float64)
        C_rows = np.asarray(C_rows, dtype=np.float64)
        k = C_rows.shape[0]
        m, n = A.shape
        return cls(np.full(k, m), np.full(k, n), A.ravel(), np.asarray(b, dtype=np.float64),
                   C_rows.ravel(), off_A=np.zeros(k, np.int64), off_b=np.zeros(k, np.int64),
                   off_c=np.arange(k, dtype=np.int64) * n)


def shard(count: int, first: int, rank: int, world: int):
    """(first LP index, LP count) of rank `rank` of `world` over LPs
    first .. first + count - 1: contiguous blocks of ceil(count / world), the
    last rank taking the remainder.  LPs are independent, so a multi-GPU run
    solves one shard per GPU and needs no collective on the data path."""
    per = (count + world - 1) // world
    lo = first + rank * per
    return lo, max(0, min(per, first + count - lo))


def generate(kind: int, count: Optional[int] = None, seed: int = DEFAULT_SEED, first: int = 0,
             threads: int = 0, share_family_A: bool = False) -> LPBatch:
    """Synthetic workload `kind` (0..4, see include/blpg.h): LPs first ..
    first+count-1 of the stream seeded with `seed`.  With share_family_A, LPs
    of the perturbed families (kinds 3 and 4) point at one copy of their
    family's A (they are identical by construction)."""
    L = N.lib()
    if count is None:
        count = WORKLOAD_COUNTS[kind]
    if share_family_A and kind in (3, 4) and count > 2048:
        # generate in chunks so that only one copy of each family's A exists
        parts = [generate(kind, min(2048, count - k0), seed, first + k0, threads, True)
                 for k0 in range(0, count, 2048)]
        return _concat_shared(parts, dict(kind=kind, seed=seed, first=first, count=count))
    m = np.zeros(count, np.int32)
    n = np.zeros(count, np.int32)
    fam = np.zeros(count, np.int32)
    total = L.blpg_gen_shapes(kind, first, count, seed, N.ptr(m, C.c_int32), N.ptr(n, C.c_int32),
                              N.ptr(fam, C.c_int32))
    if total < 0:
        N.check(int(total), "blpg_gen_shapes")
    A = np.empty(int(total), np.float64)
    b = np.empty(int(m.sum()), np.float64)
    c = np.empty(int(n.sum()), np.float64)
    rc = L.blpg_gen_fill(kind, first, count, seed, N.ptr(m, C.c_int32), N.ptr(n, C.c_int32),
                         N.ptr(A, C.c_double), N.ptr(b, C.c_double), N.ptr(c, C.c_double), threads)
    N.check(rc, "blpg_gen_fill")
    batch = LPBatch(m, n, A, b, c, family=fam,
                    meta=dict(kind=kind, seed=seed, first=first, count=count))
    if share_family_A and (fam >= 0).any():
        batch = _share_family_A(batch)
    return batch


def _concat_shared(parts, meta) -> LPBatch:
    """Concatenate family-shared batches, keeping one A per family."""
    As, fam_pos, pos = [], {}, 0
    oAs, bs, cs, obs, ocs = [], [], [], [], []
    bpos = cpos = 0
    for p in parts:
        oA, ob, oc = p.offsets()
        newA = np.empty(p.count, np.int64)
        local = {}
        for k in range(p.count):
            f = int(p.family[k])
            src = int(oA[k])
            if f >= 0 and f in fam_pos:
                newA[k] = fam_pos[f]
                continue
            if src in local:
                newA[k] = local[src]
                continue
            size = int(p.m[k]) * int(p.n[k])
            As.append(p.A[src:src + size])
            local[src] = pos
            if f >= 0:
                fam_pos[f] = pos
            newA[k] = pos
            pos += size
        oAs.append(newA)
        obs.append(ob + bpos)
        ocs.append(oc + cpos)
        bs.append(p.b)
        cs.append(p.c)
        bpos += p.b.size
        cpos += p.c.size
    return LPBatch(np.concatenate([p.m for p in parts]), np.concatenate([p.n for p in parts]),
                   np.concatenate(As), np.concatenate(bs), np.concatenate(cs),
                   off_A=np.concatenate(oAs), off_b=np.concatenate(obs), off_c=np.concatenate(ocs),
                   family=np.concatenate([p.family for p in parts]), meta=dict(meta, shared_A=True))


def _share_family_A(batch: LPBatch) -> LPBatch:
    oA, ob, oc = batch.offsets()
    fam = batch.family
    keep = {}
    pieces = []
    pos = 0
    new_oA = np.empty(batch.count, np.int64)
    for k in range(batch.count):
        f = int(fam[k])
        key = ("f", f) if f >= 0 else ("k", k)
        if key not in keep:
            size = int(batch.m[k]) * int(batch.n[k])
            pieces.append(batch.A[oA[k]:oA[k] + size])
            keep[key] = pos
            pos += size
        new_oA[k] = keep[key]
    return LPBatch(batch.m, batch.n, np.concatenate(pieces), batch.b, batch.c, off_A=new_oA,
                   off_b=ob, off_c=oc, family=batch.family, meta=dict(batch.meta, shared_A=True))


def read_abc(path_A: str, path_B: str, path_C: str):
    """Read the reference's dense A/B/C text files (parseBenchmark.cpp:59-126).
    Returns (A, b, c) as written (minimisation files: negate c for max form)."""
    L = N.lib()
    m = C.c_int32()
    n = C.c_int32()
    N.check(L.blpg_read_abc(path_A.encode(), path_B.encode(), path_C.encode(), C.byref(m),
                            C.byref(n), None, None, None), "blpg_read_abc")
    A = np.empty(m.value * n.value)
    b = np.empty(m.value)
    c = np.empty(n.value)
    N.check(L.blpg_read_abc(path_A.encode(), path_B.encode(), path_C.encode(), C.byref(m),
                            C.byref(n), N.ptr(A, C.c_double), N.ptr(b, C.c_double),
                            N.ptr(c, C.c_double)), "blpg_read_abc")
    return A.reshape(m.value, n.value), b, c


def write_batch(path: str, batch: LPBatch) -> None:
    """A batch in one binary file (blpg_write_batch: shapes, offsets, A, b, c;
    LPs that share A keep sharing it)."""
    bst = batch.c_struct()
    N.check(N.lib().blpg_write_batch(str(path).encode(), C.byref(bst)), "blpg_write_batch")


def read_batch(path: str) -> LPBatch:
    """The batch a batch file holds (blpg_read_batch), offsets included."""
    L = N.lib()
    cnt, na, nb, nc = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
    p = str(path).encode()
    N.check(L.blpg_read_batch(p, C.byref(cnt), C.byref(na), C.byref(nb), C.byref(nc), None, None,
                              None, None, None, None, None, None), "blpg_read_batch")
    k = cnt.value
    m, n = np.empty(k, np.int32), np.empty(k, np.int32)
    oA, ob, oc = np.empty(k, np.int64), np.empty(k, np.int64), np.empty(k, np.int64)
    A, b, c = np.empty(na.value), np.empty(nb.value), np.empty(nc.value)
    if k == 0:
        return LPBatch(m, n, A, b, c, off_A=oA, off_b=ob, off_c=oc)
    N.check(L.blpg_read_batch(p, C.byref(cnt), C.byref(na), C.byref(nb), C.byref(nc),
                              N.ptr(m, C.c_int32), N.ptr(n, C.c_int32), N.ptr(oA, C.c_int64),
                              N.ptr(ob, C.c_int64), N.ptr(oc, C.c_int64), N.ptr(A, C.c_double),
                              N.ptr(b, C.c_double), N.ptr(c, C.c_double)), "blpg_read_batch")
    return LPBatch(m, n, A, b, c, off_A=oA, off_b=ob, off_c=oc)


def write_results(path: str, batch: LPBatch, status, objective, x=None) -> None:
    """One text line per LP (blpg_write_results): the status, the objective
    and, when x is given, x in the batch's c layout, every double printed with
    17 significant digits so it reads back bit for bit. path "-" is stdout."""
    st = np.ascontiguousarray(status, dtype=np.int32)
    ob = np.ascontiguousarray(objective, dtype=np.float64)
    xs = None if x is None else np.ascontiguousarray(x, dtype=np.float64)
    res = N.Result(N.ptr(st, C.c_int32), N.ptr(ob, C.c_double),
                   None if xs is None else N.ptr(xs, C.c_double), None, None, None)
    bst = batch.c_struct()
    N.check(N.lib().blpg_write_results(str(path).encode(), C.byref(bst), C.byref(res)),
            "blpg_write_results")
