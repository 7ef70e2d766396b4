"""Steepest-edge pricing (BLPG_PRICE_STEEPEST): the CUDA solver against the
CPU oracle's steepest-edge mode and against the Dantzig optimum.

The GPU sums column norms as fixed-point integers and scores in FP32, the
oracle sums in FP64, so near-tied scores can pick different columns: this
mode is checked on statuses (identical), objectives (1e-9 relative in FP64,
1e-6 in the FP32 form, against the FP64 Dantzig oracle) and pivot counts
(mean within 5% of the oracle's), not bit for bit.  Across cluster splits
the GPU itself is deterministic: norms are integer sums, so results with the
tableau over 1, 2 or 4 CTAs are identical.
"""
import numpy as np
import pytest

import simplexprojects_gb300 as sp
from oracle import ref

pytestmark = pytest.mark.gpu

FP32_REL = 1e-6


def _rel(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1.0)


@pytest.mark.parametrize("kind,count", [(0, 512), (1, 512), (2, 16), (3, 128), (4, 384)])
def test_fp64_steepest_against_oracle(built, kind, count):
    batch = sp.generate(kind, count, seed=sp.DEFAULT_SEED + 31 * kind)
    gpu = sp.solve(batch, "fp64", pricing="steepest", want_x=True)
    cpu = ref.solve_batch(batch, "fp64", pricing="steepest")
    dz = ref.solve_batch(batch, "fp64")
    assert np.array_equal(gpu.status, dz.status)
    assert np.array_equal(cpu.status, dz.status)
    opt = dz.status == 5
    assert _rel(gpu.objective[opt], dz.objective[opt]).max() <= 1e-9
    assert abs(gpu.pivots.mean() - cpu.pivots.mean()) <= 0.05 * cpu.pivots.mean() + 0.5
    # fewer pivots than Dantzig on every workload with real work
    if dz.pivots.mean() > 20:
        assert gpu.pivots.mean() < dz.pivots.mean()


@pytest.mark.parametrize("kind,count", [(1, 512), (2, 16), (3, 128)])
def test_fp32_steepest(built, kind, count):
    batch = sp.generate(kind, count, seed=sp.DEFAULT_SEED + 7 * kind)
    g = sp.solve(batch, "fp32", pricing="steepest")
    dz = ref.solve_batch(batch, "fp64")
    assert np.array_equal(g.status, dz.status)
    opt = dz.status == 5
    assert (g.info[opt] & (16 | 1024)).all()  # verified in FP64, or re-solved in FP64
    assert _rel(g.objective[opt], dz.objective[opt]).max() <= FP32_REL


def test_steepest_cluster_split_deterministic(built):
    batch = sp.generate(4, 64, seed=11)
    for prec in ("fp64", "fp32"):
        a = sp.solve(batch, prec, pricing="steepest", want_x=True)
        for K in (2, 4):
            b = sp.solve(batch, prec, pricing="steepest", min_cluster=K, want_x=True)
            assert np.array_equal(a.status, b.status)
            assert np.array_equal(a.pivots, b.pivots)
            assert np.array_equal(a.objective, b.objective)
            assert np.array_equal(a.x, b.x)


def test_steepest_periodic_refresh(built):
    """FP32 with FP64 refreshes every k pivots: the refresh reuses the norms'
    shared memory, which the next pricing recomputes."""
    batch = sp.generate(2, 24, seed=21)
    dz = ref.solve_batch(batch, "fp64")
    for period in (16, 32):
        g = sp.solve(batch, "fp32", pricing="steepest", refactor_period=period)
        assert np.array_equal(g.status, dz.status)
        opt = dz.status == 5
        assert _rel(g.objective[opt], dz.objective[opt]).max() <= FP32_REL


def test_weighted_steepest_against_oracle(built):
    """Per-variable score factors (the learned warm start's channel)."""
    batch = sp.generate(3, 128, seed=9)
    rng = np.random.default_rng(4)
    w = (1.0 + rng.random(int((batch.n + batch.m).sum()))).astype(np.float32)
    gpu = sp.solve(batch, "fp64", pricing="steepest", weight=w)
    cpu = ref.solve_batch(batch, "fp64", pricing="steepest", weight=w)
    dz = ref.solve_batch(batch, "fp64")
    assert np.array_equal(gpu.status, dz.status)
    opt = dz.status == 5
    assert _rel(gpu.objective[opt], dz.objective[opt]).max() <= 1e-9
    assert abs(gpu.pivots.mean() - cpu.pivots.mean()) <= 0.05 * cpu.pivots.mean() + 0.5


def test_two_phase_steepest(built, known_golden):
    lps = list(known_golden["hand"].items())
    batch = sp.LPBatch.from_lps([(v["A"], v["b"], v["c"]) for _, v in lps])
    gpu = sp.solve(batch, "fp64", pricing="steepest")
    for k, (name, v) in enumerate(lps):
        assert gpu.status[k] == v["exact_status"], name
        if v["exact_status"] == 5:
            assert abs(gpu.objective[k] - v["exact_objective"]) <= 1e-9 * max(1, abs(v["exact_objective"])), name


def test_weights_need_steepest(built):
    batch = sp.generate(0, 4, seed=1)
    w = np.ones(int((batch.n + batch.m).sum()), np.float32)
    with pytest.raises(sp.BlpgError):
        sp.solve(batch, "fp64", weight=w)


@pytest.mark.parametrize("kind,count", [(1, 512), (2, 16), (3, 256)])
def test_fp32_steepest_repeatable(built, kind, count):
    """Repeated FP32 steepest-edge solves give the same bits: every value a
    pivot's threads share (ratios, multipliers, norms) is published by a
    barrier before it is overwritten."""
    batch = sp.generate(kind, count, seed=sp.DEFAULT_SEED + 13 * kind)
    a = sp.solve(batch, "fp32", pricing="steepest", want_x=True)
    for _ in range(3):
        b = sp.solve(batch, "fp32", pricing="steepest", want_x=True)
        assert np.array_equal(a.status, b.status)
        assert np.array_equal(a.pivots, b.pivots)
        assert np.array_equal(a.objective, b.objective)
        assert np.array_equal(a.x, b.x)
