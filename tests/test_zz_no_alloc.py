"""The allocation-free entry point, blpg_solve_noalloc, against the normal
entry point (blpg_solve_batch).

blpg_solve_noalloc serves callers that cannot call cudaMalloc (code running
inside a memory pool it does not own, or a framework that has handed all
device memory to its own allocator): it takes only caller-provided device
buffers and keeps its work-queue scratch in a fixed array inside the library.
It runs the same pivot kernel with the same rules, so its results must be
bit-identical to blpg_solve_batch's (the FP64 tolerance of the parity tests)
and, in FP32, equal to the FP32 path's.  Two calls in a row check that the
shared scratch is reset between calls.  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

import simplexprojects_gb300 as sp
from simplexprojects_gb300 import _native as N

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


def _call(batch, d, precision):
    import torch
    p = lambda t: C.c_void_p(t.data_ptr())
    rc = N.lib().blpg_solve_noalloc(
        batch.count, int(batch.m.max()), int(batch.n.max()), p(d["m"]), p(d["n"]), p(d["oA"]),
        p(d["ob"]), p(d["oc"]), p(d["A"]), p(d["b"]), p(d["c"]), precision, p(d["status"]),
        p(d["obj"]), p(d["x"]), p(d["piv"]), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    N.check(rc, "blpg_solve_noalloc")
    torch.cuda.synchronize()
    return (d["status"].cpu().numpy(), d["obj"].cpu().numpy(), d["piv"].cpu().numpy(),
            d["x"].cpu().numpy())


@pytest.mark.parametrize("precision,name", [(0, "fp64"), (1, "fp32")])
def test_noalloc_matches_solve_batch(built, precision, name):
    batch = sp.generate(1, 400, seed=4242)
    ref = sp.solve(batch, name, want_x=True)
    d = _device(batch)
    for call in range(2):
        d["status"].fill_(-9)
        d["obj"].fill_(float("nan"))
        st, obj, piv, x = _call(batch, d, precision)
        assert np.array_equal(st, ref.status), call
        assert np.array_equal(piv, ref.pivots), call
        assert np.array_equal(obj.view(np.uint64), ref.objective.view(np.uint64)), call
        assert np.array_equal(x.view(np.uint64), ref.x.view(np.uint64)), call


def test_noalloc_large_tableaux_use_clusters(built):
    """Shapes that need a multi-CTA cluster give the same results too."""
    batch = sp.generate(2, 24, seed=99)
    ref = sp.solve(batch, "fp64", want_x=True)
    d = _device(batch)
    st, obj, piv, x = _call(batch, d, 0)
    assert np.array_equal(st, ref.status) and np.array_equal(piv, ref.pivots)
    assert np.array_equal(obj.view(np.uint64), ref.objective.view(np.uint64))


def test_noalloc_rejects_oversized_batches(built):
    rc = N.lib().blpg_solve_noalloc(1 << 20, 10, 10, *([None] * 8), 0, None, None, None, None,
                                    None)
    assert rc == -1
    assert b"outside" in N.lib().blpg_last_error()
