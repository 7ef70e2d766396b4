"""blpg_solve_batch's chunked path (include/blpg.h): a packed batch whose
uploads are large is solved in eight chunks whose uploads overlap the
previous chunks' solves, and one that does not fit the device budget in as many chunks
as the budget needs, taking turns in two device regions.  Either way the
results are the one-plan results: FP64 status, pivots, objective, x and basis
bit for bit the oracle's; FP32 statuses the oracle's, objectives within 1e-6.
The thresholds are lowered through the tuning table so that a batch of a few
hundred MB takes each path."""
import numpy as np
import pytest

import simplexprojects_gb300 as sp
from simplexprojects_gb300 import _native as N
from simplexprojects_gb300.autotune import override as _tuning
from oracle import ref

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("knobs,chunks", [({}, 8), ({"overlap_chunks": 3}, 3), ({"overlap_mb": 100_000}, 1),
                                          ({"device_budget_mb": 40}, None)])
def test_chunked_solve(built, knobs, chunks):
    batch = sp.generate(1, 3000, seed=sp.DEFAULT_SEED)  # uneven sizes, packed, 183 MB
    assert batch.off_A is None
    cpu = ref.solve_batch(batch, "fp64", want_x=True, want_basis=True)
    try:
        _tuning(knobs)
        g = sp.solve(batch, "fp64", want_x=True, want_basis=True)
        used = N.lib().blpg_solve_batch_chunks()
        again = sp.solve(batch, "fp64", want_x=True, want_basis=True)  # cached plans
        f = sp.solve(batch, "fp32", pricing="steepest")
    finally:
        N.check(N.lib().blpg_set_tuning(None), "blpg_set_tuning")
    if chunks is None:
        assert used > 8  # 183 MB of inputs against a 40 MB budget: two regions of 20 MB
    else:
        assert used == chunks
    for r in (g, again):
        assert np.array_equal(r.status, cpu.status)
        assert np.array_equal(r.pivots, cpu.pivots)
        assert np.array_equal(r.basis, cpu.basis)
        assert np.array_equal(r.objective.view(np.uint64), cpu.objective.view(np.uint64))
        assert np.array_equal(r.x.view(np.uint64), cpu.x.view(np.uint64))
    opt = cpu.status == 5
    assert np.array_equal(f.status, cpu.status)
    rel = np.abs(f.objective - cpu.objective) / np.maximum(np.abs(cpu.objective), 1.0)
    assert rel[opt].max() <= 1e-6


@pytest.mark.parametrize("knobs", [{}, {"device_budget_mb": 40}])
def test_chunked_warm_start_inputs(built, knobs):
    """Basis hints and pricing weights are split with the LPs (in the device
    copy of the batch, and relocated into the two regions of the budget
    split): a chunked solve given the FP64 bases as hints ends where a
    one-plan solve does."""
    batch = sp.generate(1, 3000, seed=sp.DEFAULT_SEED)
    base = sp.solve(batch, "fp64", want_basis=True)
    w = np.random.default_rng(3).uniform(0.5, 2.0, int((batch.m + batch.n).sum())).astype(np.float32)
    try:
        _tuning({"overlap_mb": 100_000})
        one = sp.solve(batch, "fp64", hint=base.basis)
        assert N.lib().blpg_solve_batch_chunks() == 1
        one_w = sp.solve(batch, "fp32", pricing="steepest", weight=w)
        _tuning(knobs)
        eight = sp.solve(batch, "fp64", hint=base.basis)
        assert N.lib().blpg_solve_batch_chunks() >= 8
        eight_w = sp.solve(batch, "fp32", pricing="steepest", weight=w)
        assert N.lib().blpg_solve_batch_chunks() >= 8
    finally:
        N.check(N.lib().blpg_set_tuning(None), "blpg_set_tuning")
    assert np.array_equal(one_w.status, eight_w.status)
    opt = one_w.status == 5
    rel = np.abs(one_w.objective - eight_w.objective) / np.maximum(np.abs(one_w.objective), 1.0)
    assert rel[opt].max() <= 1e-6
    assert np.array_equal(one.status, eight.status)
    assert np.array_equal(one.pivots, eight.pivots)
    assert np.array_equal(one.info, eight.info)
    assert np.array_equal(one.objective.view(np.uint64), eight.objective.view(np.uint64))


@pytest.mark.parametrize("knobs,chunks", [({"overlap_mb": 8}, 8), ({"overlap_mb": 8, "overlap_chunks": 5}, 5),
                                          ({"device_budget_mb": 4}, 8)])
def test_chunked_solve_with_offsets(built, knobs, chunks):
    """A batch given by offset arrays (LPs of a family share one A) is solved
    in chunks on one device copy of the caller's arrays, each chunk uploading
    what its LPs read beyond what earlier chunks uploaded.  It is never
    relocated (its LPs may read any part of A), so a device budget does not
    split it further."""
    batch = sp.generate(4, 3000, seed=sp.DEFAULT_SEED, share_family_A=True)
    assert batch.off_A is not None
    cpu = ref.solve_batch(batch, "fp64", want_x=True, want_basis=True)
    try:
        _tuning(knobs)
        g = sp.solve(batch, "fp64", want_x=True, want_basis=True)
        used = N.lib().blpg_solve_batch_chunks()
        f = sp.solve(batch, "fp32", pricing="steepest", want_x=True)
    finally:
        N.check(N.lib().blpg_set_tuning(None), "blpg_set_tuning")
    assert used == chunks
    assert np.array_equal(g.status, cpu.status)
    assert np.array_equal(g.pivots, cpu.pivots)
    assert np.array_equal(g.basis, cpu.basis)
    assert np.array_equal(g.objective.view(np.uint64), cpu.objective.view(np.uint64))
    assert np.array_equal(g.x.view(np.uint64), cpu.x.view(np.uint64))
    opt = cpu.status == 5
    assert np.array_equal(f.status, cpu.status)
    rel = np.abs(f.objective - cpu.objective) / np.maximum(np.abs(cpu.objective), 1.0)
    assert rel[opt].max() <= 1e-6


def test_release_workspace(built):
    """blpg_release_workspace frees the cached plans and device buffers of
    blpg_solve_batch (one-plan and chunked); the next call rebuilds them and
    gives the same results."""
    import torch
    big = sp.generate(1, 3000, seed=sp.DEFAULT_SEED)     # chunked
    small = sp.generate(0, 200, seed=sp.DEFAULT_SEED)    # one plan
    a = sp.solve(big, "fp64", want_x=True)
    s1 = sp.solve(small, "fp64")
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    N.check(N.lib().blpg_release_workspace(), "blpg_release_workspace")
    free1, _ = torch.cuda.mem_get_info()
    assert free1 - free0 >= 150 << 20  # at least the chunked batch's 183 MB device copy
    b = sp.solve(big, "fp64", want_x=True)
    s2 = sp.solve(small, "fp64")
    assert np.array_equal(a.objective.view(np.uint64), b.objective.view(np.uint64))
    assert np.array_equal(a.x.view(np.uint64), b.x.view(np.uint64))
    assert np.array_equal(s1.objective.view(np.uint64), s2.objective.view(np.uint64))
    N.check(N.lib().blpg_release_workspace(), "blpg_release_workspace")
