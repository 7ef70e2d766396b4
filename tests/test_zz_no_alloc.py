"""The allocation-free entry point, blpg_solve_noalloc, against the normal
entry point (blpg_solve_batch).

blpg_solve_noalloc serves callers that cannot call cudaMalloc (code running
inside a memory pool it does not own, or a framework that has handed all
device memory to its own allocator): it takes only caller-provided device
buffers and keeps its work-queue scratch in a fixed array inside the library.
It runs the same pivot kernel with the same rules, so FP64 results are
bit-identical to blpg_solve_batch's.  In FP32 they are bit-identical on every
LP that blpg_solve_batch verified by iterative refinement alone; where a plan
factorised a basis in FP64 (BLPG_INFO_FACTOR: its LU scratch is plan
memory, which this entry point does not have) the allocation-free call
reports the same status or BLPG_UNDEF.  Two calls in a row check that the
shared scratch is reset between calls.  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

import simplexprojects_gb300 as sp
from simplexprojects_gb300 import _native as N
from oracle import ref as oracle

pytestmark = pytest.mark.gpu


def _device(batch):
    import torch
    oA, ob, oc = batch.offsets()
    d = dict(
        m=torch.from_numpy(batch.m).cuda(), n=torch.from_numpy(batch.n).cuda(),
        oA=torch.from_numpy(np.ascontiguousarray(oA)).cuda(),
        ob=torch.from_numpy(np.ascontiguousarray(ob)).cuda(),
        oc=torch.from_numpy(np.ascontiguousarray(oc)).cuda(),
        A=torch.from_numpy(batch.A).cuda(), b=torch.from_numpy(batch.b).cuda(),
        c=torch.from_numpy(batch.c).cuda(),
        status=torch.full((batch.count,), -9, dtype=torch.int32, device="cuda"),
        obj=torch.full((batch.count,), float("nan"), dtype=torch.float64, device="cuda"),
        piv=torch.full((batch.count,), -9, dtype=torch.int32, device="cuda"),
        x=torch.full((int((oc + batch.n).max()),), float("nan"), dtype=torch.float64,
                     device="cuda"),
    )
    return d


def _call(batch, d, precision, max_m=None, max_n=None):
    import torch
    p = lambda t: C.c_void_p(t.data_ptr())
    max_m = int(batch.m.max()) if max_m is None else max_m
    max_n = int(batch.n.max()) if max_n is None else max_n
    rc = N.lib().blpg_solve_noalloc(
        batch.count, max_m, max_n, p(d["m"]), p(d["n"]), p(d["oA"]),
        p(d["ob"]), p(d["oc"]), p(d["A"]), p(d["b"]), p(d["c"]), precision, p(d["status"]),
        p(d["obj"]), p(d["x"]), p(d["piv"]), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    N.check(rc, "blpg_solve_noalloc")
    torch.cuda.synchronize()
    return (d["status"].cpu().numpy(), d["obj"].cpu().numpy(), d["piv"].cpu().numpy(),
            d["x"].cpu().numpy())


FACTOR = 512 | 256  # BLPG_INFO_FACTOR | BLPG_INFO_REINVERT


def _same(got, want, call=None, batch=None):
    """Bit-identical results, except (FP32 plans) on LPs the plan verified by
    an FP64 factorisation: there the same status or BLPG_UNDEF."""
    st, obj, piv, x = got
    plain = np.ones(st.size, bool) if want.info is None else (want.info & FACTOR) == 0
    assert plain.mean() > 0.9, call
    assert np.array_equal(st[plain], want.status[plain]), call
    assert np.array_equal(piv[plain], want.pivots[plain]), call
    assert np.array_equal(obj[plain].view(np.uint64), want.objective[plain].view(np.uint64)), call
    if batch is not None:
        _, _, oc = batch.offsets()
        for k in np.nonzero(plain)[0]:
            sl = slice(int(oc[k]), int(oc[k] + batch.n[k]))
            assert np.array_equal(x[sl].view(np.uint64), want.x[sl].view(np.uint64)), (call, k)
    else:
        assert np.array_equal(x.view(np.uint64), want.x.view(np.uint64)), call
    rest = ~plain
    assert ((st[rest] == want.status[rest]) | (st[rest] == 1)).all(), call


@pytest.mark.parametrize("kind,count", [(1, 400), (4, 160)])
@pytest.mark.parametrize("precision,name", [(0, "fp64"), (1, "fp32")])
def test_noalloc_matches_solve_batch(built, kind, count, precision, name):
    """Two calls in a row give blpg_solve_batch's bits.  Kind 4 mixes shapes
    from m=16 to m=256: here every LP runs with the cluster size and thread
    count of the largest, where blpg_solve_batch gives each its own size
    class; the pivot rules do not depend on either."""
    batch = sp.generate(kind, count, seed=4242 + kind)
    want = sp.solve(batch, name, want_x=True)
    d = _device(batch)
    for call in range(2):
        d["status"].fill_(-9)
        d["obj"].fill_(float("nan"))
        _same(_call(batch, d, precision), want, call, batch)
    if precision == 0:  # and the FP64 oracle's, bit for bit
        _same(_call(batch, d, precision), oracle.solve_batch(batch, "fp64", want_x=True))


@pytest.mark.parametrize("precision,name", [(0, "fp64"), (1, "fp32")])
def test_noalloc_large_tableaux_use_clusters(built, precision, name):
    """Shapes that need a multi-CTA cluster give the same results too."""
    batch = sp.generate(2, 24, seed=99)
    want = sp.solve(batch, name, want_x=True)
    d = _device(batch)
    _same(_call(batch, d, precision), want, batch=batch)


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_refuses_phase_one_and_oversized_lps(built, precision):
    """An LP with some b_i < 0 (phase I is not part of this entry point) and
    an LP larger than the max_m / max_n passed get BLPG_UNDEF with pivots -1;
    the other LPs of the call are solved as usual."""
    base = sp.generate(0, 6, seed=7)
    big = sp.generate(1, 1, seed=8)
    lps = [base.lp(k) for k in range(6)]
    A, b, c = base.lp(0)
    b = b.copy()
    b[3] = -1.0
    lps.append((A, b, c))
    lps.append(big.lp(0))
    batch = sp.LPBatch.from_lps(lps)
    d = _device(batch)
    st, obj, piv, x = _call(batch, d, precision, max_m=28, max_n=32)
    assert st[6] == 1 and piv[6] == -1
    assert st[7] == 1 and piv[7] == -1
    want = sp.solve(base, "fp32" if precision else "fp64")
    plain = (want.info & FACTOR) == 0
    assert np.array_equal(st[:6][plain], want.status[plain])
    assert np.array_equal(piv[:6][plain], want.pivots[plain])
    assert np.array_equal(obj[:6][plain].view(np.uint64), want.objective[plain].view(np.uint64))


def test_noalloc_rejects_oversized_batches(built):
    rc = N.lib().blpg_solve_noalloc(1 << 20, 10, 10, *([None] * 8), 0, None, None, None, None,
                                    None)
    assert rc == -1
    assert b"outside" in N.lib().blpg_last_error()
