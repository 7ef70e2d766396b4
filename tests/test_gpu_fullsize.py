"""GPU parity at the benchmark configurations' full sizes and on the
reference's own Netlib LPs, through the C ABI.

Configurations (the seeded generator of include/blpg.h):
  kind 0   1,024 LPs, m=28, n=32
  kind 1   10,000 LPs of uneven sizes, 10% unbounded, 5% zero-b rows
  kind 2   2,048 LPs, m=205, n=203
  kind 3   the 10,000 held-out perturbed LPs (indices 40,000-49,999)
  kind 4   200,000 LPs, m log-uniform on [16, 256]

FP64 (the reference's method): status, pivot count and objective bits
identical to the CPU oracle on every LP.  FP32 (Dantzig, steepest edge, and
the learned warm start on kind 3): statuses identical to the FP64 oracle,
objectives within 1e-6 relative of it.

Netlib (tests/golden/netlib, the reference's benchmarks/*.txt, minimisation
files negated into max form as GPU_Tester.cu:119-127 does): FP64 bit-identical
to the oracle and within 1e-9 of the exact optimum; FP32 within 1e-6; three
of the eight need phase I.
"""
import numpy as np
import pytest

import simplexprojects_gb300 as sp
from oracle import ref
from conftest import NETLIB

pytestmark = pytest.mark.gpu

FP32_REL = 1e-6
FULL = {0: (1024, 0), 1: (10_000, 0), 2: (2048, 0), 3: (10_000, 40_000), 4: (200_000, 0)}


def _rel(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1.0)


def _full(kind):
    """A configuration at its full size (perturbed families share A)."""
    count, first = FULL[kind]
    return sp.generate(kind, count, seed=sp.DEFAULT_SEED, first=first,
                       share_family_A=kind in (3, 4))


@pytest.mark.parametrize("kind", [0, 1, 2, 3, 4])
def test_full_config(built, kind):
    """FP64 bit-identical to the oracle; FP32 (both pricing rules) statuses
    identical and objectives within 1e-6, every optimum FP64-verified."""
    batch = _full(kind)
    cpu = ref.solve_batch(batch, "fp64")
    gpu = sp.solve(batch, "fp64")
    assert gpu.status.size == FULL[kind][0]
    assert np.array_equal(gpu.status, cpu.status)
    assert np.array_equal(gpu.pivots, cpu.pivots)
    assert np.array_equal(gpu.objective.view(np.uint64), cpu.objective.view(np.uint64))
    opt = cpu.status == 5
    for pricing in ("dantzig", "steepest"):
        g = sp.solve(batch, "fp32", pricing=pricing)
        assert np.array_equal(g.status, cpu.status), pricing
        assert (g.info[opt] & (16 | 1024)).all(), pricing  # verified in FP64, or re-solved in FP64
        assert _rel(g.objective[opt], cpu.objective[opt]).max() <= FP32_REL, pricing


def test_full_config_learned_warm_start(built):
    """Kind 3 as the benchmark runs it: a network trained on the plain FP64
    solver's bases of LPs 0-39,999 guides the FP32 steepest-edge solve of the
    10,000 held-out LPs; the crash mode (predicted basis, primal / dual finish,
    cold fallback) is checked too."""
    from simplexprojects_gb300.warmstart import WarmStart, LearnedSolver
    batch = _full(3)
    cpu = ref.solve_batch(batch, "fp64")
    train = sp.generate(3, 40_000, seed=sp.DEFAULT_SEED, share_family_A=True)
    tb = sp.solve(train, "fp64", want_basis=True)
    ws = WarmStart(174, 142, 64, seed=7, max_batch=10_048)
    ws.train(train, tb.basis, epochs=4, lr=1e-3, batch_size=512)
    opt = cpu.status == 5
    for mode in ("guided", "crash"):
        ls = LearnedSolver(ws, batch, "fp32", mode=mode)
        ls.run()
        r = ls.result()
        assert np.array_equal(r.status, cpu.status), mode
        assert _rel(r.objective[opt], cpu.objective[opt]).max() <= FP32_REL, mode


def _netlib(known):
    names = list(known["netlib"])
    lps = []
    for nm in names:
        A, b, c = sp.read_abc(*(str(NETLIB / f"{nm}_{s}.txt") for s in "ABC"))
        lps.append((A, b, -c))  # max form (GPU_Tester.cu:119-127)
    return names, sp.LPBatch.from_lps(lps)


def test_netlib_fp64(built, known_golden):
    names, batch = _netlib(known_golden)
    assert len(names) == 8
    gpu = sp.solve(batch, "fp64", want_x=True, want_basis=True)
    cpu = ref.solve_batch(batch, "fp64", want_x=True, want_basis=True)
    assert np.array_equal(gpu.status, cpu.status)
    assert np.array_equal(gpu.pivots, cpu.pivots)
    assert np.array_equal(gpu.basis, cpu.basis)
    assert np.array_equal(gpu.objective.view(np.uint64), cpu.objective.view(np.uint64))
    assert np.array_equal(gpu.x.view(np.uint64), cpu.x.view(np.uint64))
    for k, nm in enumerate(names):
        v = known_golden["netlib"][nm]
        assert gpu.status[k] == v["exact_status"], nm
        ex = v["exact_objective"]
        assert abs(gpu.objective[k] - ex) <= 1e-9 * max(1.0, abs(ex)), nm
        assert abs(-gpu.objective[k] - v["listed_min"]) <= 1e-5 * abs(v["listed_min"]), nm


@pytest.mark.parametrize("prec,pricing,tol", [("fp64", "steepest", 1e-9),
                                              ("fp32", "dantzig", FP32_REL),
                                              ("fp32", "steepest", FP32_REL)])
def test_netlib_other_modes(built, known_golden, prec, pricing, tol):
    names, batch = _netlib(known_golden)
    g = sp.solve(batch, prec, pricing=pricing)
    for k, nm in enumerate(names):
        v = known_golden["netlib"][nm]
        assert g.status[k] == v["exact_status"], (nm, prec, pricing)
        ex = v["exact_objective"]
        assert abs(g.objective[k] - ex) <= tol * max(1.0, abs(ex)), (nm, prec, pricing,
                                                                     g.objective[k], ex)


def test_fp64_pass_of_fp32_plans(built, known_golden):
    """LPs the FP32 tableau cannot settle (Netlib's BLEND, ADLITTLE, SC205 in
    some pricing modes: unverified, stalled at the FP32 pivot cap) are handed
    to the plan's FP64 pass, which solves them from scratch with the FP64
    Dantzig method: their results are bit for bit the FP64 solve's, flagged
    BLPG_INFO_FP64.  A pivot cap the FP64 pass shares leaves them UNDEF."""
    names, batch = _netlib(known_golden)
    f64 = sp.solve(batch, "fp64", want_x=True)
    handed = 0
    for pricing in ("dantzig", "steepest"):
        g = sp.solve(batch, "fp32", pricing=pricing, want_x=True)
        fb = (g.info & 1024) != 0
        handed += int(fb.sum())
        _, _, oc = batch.offsets()
        for k in np.nonzero(fb)[0]:
            assert g.status[k] == f64.status[k] and g.pivots[k] == f64.pivots[k], names[k]
            assert g.objective[k] == f64.objective[k], names[k]
            sl = slice(int(oc[k]), int(oc[k] + batch.n[k]))
            assert np.array_equal(g.x[sl], f64.x[sl]), names[k]
    assert handed > 0
    capped = sp.solve(batch, "fp32", max_pivots=5)
    assert (capped.status == 1).all() and (capped.pivots == 5).all()
    assert ((capped.info & 1024) != 0).all()
