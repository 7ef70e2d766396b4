"""GPU warm start from a basis hint, through the C ABI, against the oracle.

The hinted structural columns are pivoted in (largest-magnitude pivot among
rows whose slack the hint does not keep); the LP is then finished by primal
simplex (hinted basis primal feasible), dual simplex (dual feasible), a
cost-shifted dual phase (infeasible both ways, warm_mode 1, the default) or a
cold solve (warm_mode 2).  FP64: bit-identical to the oracle's same path.
"""
import numpy as np
import pytest

import simplexprojects_gb300 as sp
from oracle import ref

pytestmark = pytest.mark.gpu


def _hints(batch, cold_basis):
    m = batch.m
    B = np.split(cold_basis, np.cumsum(m)[:-1])
    k = batch.count
    rng = np.random.default_rng(7)
    perfect = cold_basis.copy()
    sibling = np.concatenate([B[(i + 64) % k] for i in range(k)])  # same family
    rand = np.concatenate([rng.permutation(int(m[i]) + int(batch.n[i]))[: int(m[i])]
                           for i in range(k)]).astype(np.int32)
    return {"perfect": perfect, "sibling": sibling, "random": rand}


@pytest.fixture(scope="module")
def fam_batch():
    return sp.generate(3, 192, seed=sp.DEFAULT_SEED + 1, share_family_A=True)


@pytest.mark.parametrize("mode,oracle_composite", [(1, 1), (2, 0)])
def test_warm_fp64_bit_identical(built, fam_batch, mode, oracle_composite):
    cold = ref.solve_batch(fam_batch, "fp64", want_basis=True)
    for name, hint in _hints(fam_batch, cold.basis).items():
        g = sp.solve(fam_batch, "fp64", want_x=True, want_basis=True, hint=hint, warm_mode=mode)
        c = ref.solve_batch(fam_batch, "fp64", want_x=True, want_basis=True, hint=hint,
                            composite=oracle_composite)
        assert np.array_equal(g.status, c.status), name
        assert np.array_equal(g.pivots, c.pivots), name
        assert np.array_equal(g.info, c.info), name
        assert np.array_equal(g.basis, c.basis), name
        assert np.array_equal(g.objective.view(np.uint64), c.objective.view(np.uint64)), name
        assert np.array_equal(g.status, cold.status), name
    # a perfect hint needs only the crash pivots (one per structural basic)
    g = sp.solve(fam_batch, "fp64", hint=cold.basis)
    nstruct = np.array([(b < n).sum() for b, n in
                        zip(np.split(cold.basis, np.cumsum(fam_batch.m)[:-1]), fam_batch.n)])
    assert np.array_equal(g.pivots, nstruct)


def test_warm_fp32_matches_exact(built, fam_batch):
    cold = ref.solve_batch(fam_batch, "fp64", want_basis=True)
    for name, hint in _hints(fam_batch, cold.basis).items():
        g = sp.solve(fam_batch, "fp32", hint=hint)
        assert np.array_equal(g.status, cold.status), name
        opt = cold.status == 5
        rel = np.abs(g.objective[opt] - cold.objective[opt]) / np.abs(cold.objective[opt])
        assert rel.max() <= 1e-6, (name, rel.max())  # the FP32 form's bar
        assert (g.info[opt] & (16 | 1024)).all()  # refreshed in FP64, or re-solved in FP64


def test_warm_cluster_split_fp64(built):
    """Warm start on LPs split across a cluster (the crash and dual phases
    exchange pivot rows and columns through distributed shared memory)."""
    batch = sp.generate(3, 24, seed=11, share_family_A=True)
    cold = ref.solve_batch(batch, "fp64", want_basis=True)
    hint = _hints(batch, cold.basis)["random"]
    for K in (2, 4):
        g = sp.solve(batch, "fp64", want_basis=True, hint=hint, min_cluster=K)
        c = ref.solve_batch(batch, "fp64", want_basis=True, hint=hint)
        assert np.array_equal(g.pivots, c.pivots) and np.array_equal(g.basis, c.basis)
        assert np.array_equal(g.objective.view(np.uint64), c.objective.view(np.uint64))


def test_hint_ignored_for_two_phase_lps(built, known_golden):
    lps = [(v["A"], v["b"], v["c"]) for v in known_golden["hand"].values()]
    batch = sp.LPBatch.from_lps(lps)
    hint = np.concatenate([np.arange(len(v["b"])) for v in known_golden["hand"].values()])
    g = sp.solve(batch, "fp64", hint=hint.astype(np.int32))
    c = ref.solve_batch(batch, "fp64", hint=hint.astype(np.int32))
    assert np.array_equal(g.status, c.status) and np.array_equal(g.pivots, c.pivots)
    assert np.array_equal(g.objective.view(np.uint64), c.objective.view(np.uint64))


def test_learned_warm_start_end_to_end(built):
    """Train the network on plain-solver bases of 4,096 perturbed LPs, then
    solve 512 held-out LPs with its hints: fewer pivots than the cold solve
    (what the network gains over the method without it), identical statuses,
    FP64 results bit-identical to the oracle given the same hints, FP32
    objectives within 1e-6."""
    from simplexprojects_gb300.warmstart import WarmStart, LearnedSolver, basis_accuracy
    train = sp.generate(3, 16384, seed=sp.DEFAULT_SEED, first=0, share_family_A=True)
    held = sp.generate(3, 512, seed=sp.DEFAULT_SEED, first=45_000, share_family_A=True)
    tb = sp.solve(train, "fp64", want_basis=True)
    ws = WarmStart(174, 142, 64, seed=3)
    rep = ws.train(train, tb.basis, epochs=16, lr=1e-3)
    assert rep.losses[-1] < rep.losses[0]
    cold = sp.solve(held, "fp64", want_basis=True)
    ls = LearnedSolver(ws, held, "fp64", mode="crash")
    ls.run()
    res = ls.result()
    hint = ls.hint.cpu().numpy()
    acc, _ = basis_accuracy(hint, cold.basis, 174)
    assert acc > 0.85  # (an all-slack guess scores about 0.8)
    assert (hint < 142).sum() > 20 * held.count  # structural columns are predicted
    assert np.array_equal(res.status, cold.status)
    assert res.pivots.mean() < 0.9 * cold.pivots.mean()
    orc = ref.solve_batch(held, "fp64", hint=hint)
    assert np.array_equal(res.pivots, orc.pivots) and np.array_equal(res.info, orc.info)
    assert np.array_equal(res.objective.view(np.uint64), orc.objective.view(np.uint64))
    l32 = LearnedSolver(ws, held, "fp32", mode="crash")
    r32 = l32.solve(held)
    assert np.array_equal(r32.status, cold.status)
    opt = cold.status == 5
    rel = np.abs(r32.objective[opt] - cold.objective[opt]) / np.abs(cold.objective[opt])
    assert rel.max() <= 1e-6
    # guided mode: the network's probabilities weight steepest-edge pricing.
    # Against the same pricing without the network: fewer pivots.
    cold_se = sp.solve(held, "fp64", pricing="steepest")
    lg = LearnedSolver(ws, held, "fp64", mode="guided")
    lg.run()
    rg = lg.result()
    assert np.array_equal(rg.status, cold.status)
    assert _relerr(rg.objective[opt], cold.objective[opt]) <= 1e-9
    assert rg.pivots.mean() < 0.95 * cold_se.pivots.mean()
    w = lg.weight.cpu().numpy()
    assert w.min() >= 1.0 and w.max() <= 2.0
    orc = ref.solve_batch(held, "fp64", pricing="steepest", weight=w)
    assert np.array_equal(orc.status, cold.status)
    assert abs(rg.pivots.mean() - orc.pivots.mean()) <= 0.05 * orc.pivots.mean()
    g32 = LearnedSolver(ws, held, "fp32", mode="guided").solve(held)
    assert np.array_equal(g32.status, cold.status)
    assert _relerr(g32.objective[opt], cold.objective[opt]) <= 1e-6


def _relerr(a, b):
    return float((np.abs(a - b) / np.maximum(np.abs(b), 1.0)).max()) if a.size else 0.0


def test_warm_start_checkpoint_roundtrip(built, tmp_path):
    from simplexprojects_gb300.warmstart import WarmStart
    train = sp.generate(3, 256, seed=5, share_family_A=True)
    tb = sp.solve(train, "fp64", want_basis=True)
    ws = WarmStart(174, 142, 64, hidden=128, layers=2, seed=1)
    ws.train(train, tb.basis, epochs=1)
    ws.save(str(tmp_path / "model"))
    ws2 = WarmStart.load(str(tmp_path / "model"))
    assert np.array_equal(ws.mlp.get_params(), ws2.mlp.get_params())
    d = ws.device_inputs(train)
    import torch
    assert torch.equal(ws.features(d), ws2.features(d))


@pytest.mark.parametrize("pricing", ["dantzig", "steepest"])
def test_fp32_warm_start_is_verified(built, pricing):
    """FP32 warm starts on the uneven workload (unbounded columns, zero-b
    rows): crash and dual simplex in FP32 can end on a tableau too inaccurate
    to trust.  The FP64 refresh must then fail to converge, and the LP is
    re-solved cold: every optimal objective within 1e-6, statuses as FP64."""
    batch = sp.generate(1, 2048, seed=sp.DEFAULT_SEED)
    exact = ref.solve_batch(batch, "fp64", want_basis=True)
    g = sp.solve(batch, "fp32", pricing=pricing, hint=exact.basis)
    assert np.array_equal(g.status, exact.status)
    opt = exact.status == 5
    rel = np.abs(g.objective[opt] - exact.objective[opt]) / np.maximum(np.abs(exact.objective[opt]), 1.0)
    assert rel.max() <= 1e-6
    assert ((g.info & 128) == 0).all()  # nothing left unverified
    # warm starts whose final basis the FP64 refresh shows not optimal after
    # all (FP32 dual simplex stopped on inaccurate values) are re-run cold
    # (BLPG_INFO_RETRY): 11 of these 2,048 LPs under both pricing rules
    retries = int(((g.info & 2048) != 0).sum())
    print(f"kind-1 FP32 warm starts ({pricing}): {retries} re-run cold, "
          f"{int(((g.info & 2) != 0).sum())} hints infeasible both ways or re-run, "
          f"{int(((g.info & 512) != 0).sum())} factorised, "
          f"{int(((g.info & 256) != 0).sum())} rebuilt, {int(((g.info & 1024) != 0).sum())} FP64")
    assert retries <= 2048 // 100  # at most 1% re-run cold


def test_learned_solve_through_the_c_abi(built):
    """blpg_learned_create / blpg_learned_solve called through ctypes from
    host arrays: the same kernels in the same order as the device-resident
    path (features -> network -> weights -> FP32 steepest-edge plan), so the
    same bits; statuses and objectives as the FP64 oracle's (1e-6)."""
    import ctypes as C
    import torch
    from simplexprojects_gb300 import _native as N
    from simplexprojects_gb300.warmstart import WarmStart, LearnedSolver
    train = sp.generate(3, 4096, seed=sp.DEFAULT_SEED, first=0, share_family_A=True)
    held = sp.generate(3, 640, seed=sp.DEFAULT_SEED, first=47_000, share_family_A=True)
    tb = sp.solve(train, "fp64", want_basis=True)
    ws = WarmStart(174, 142, 64, seed=5)
    ws.train(train, tb.basis, epochs=4, lr=1e-3)
    L = N.lib()
    mean = np.ascontiguousarray(ws.mean.cpu().numpy(), np.float32)
    std = np.ascontiguousarray(ws.std.cpu().numpy(), np.float32)
    o = sp.options("fp32")
    bst = held.c_struct()
    h = C.c_void_p()
    N.check(L.blpg_learned_create(ws.mlp.h, 64, mean.ctypes.data_as(C.POINTER(C.c_float)),
                                  std.ctypes.data_as(C.POINTER(C.c_float)), 1.0, C.byref(bst),
                                  C.byref(o), C.byref(h)), "blpg_learned_create")
    k = held.count
    st, ob, pv, info = (np.zeros(k, np.int32), np.zeros(k), np.zeros(k, np.int32),
                        np.zeros(k, np.int32))
    res = N.Result(N.ptr(st, C.c_int32), N.ptr(ob, C.c_double), None, N.ptr(pv, C.c_int32), None,
                   N.ptr(info, C.c_int32))
    fam = np.ascontiguousarray(held.family, np.int32)
    for _ in range(2):  # twice: the solver object is reusable
        N.check(L.blpg_learned_solve(h, C.byref(bst), N.ptr(fam, C.c_int32), C.byref(res)),
                "blpg_learned_solve")
    L.blpg_learned_destroy(h)
    dev = LearnedSolver(ws, held, "fp32", mode="guided")
    dev.run()
    torch.cuda.synchronize()
    want = dev.result()
    assert np.array_equal(st, want.status) and np.array_equal(pv, want.pivots)
    assert np.array_equal(ob.view(np.uint64), want.objective.view(np.uint64))
    cpu = ref.solve_batch(held, "fp64")
    assert np.array_equal(st, cpu.status)
    opt = cpu.status == 5
    assert _relerr(ob[opt], cpu.objective[opt]) <= 1e-6
    # LearnedSolver.solve is this call
    r = dev.solve(held)
    assert np.array_equal(r.status, st) and np.array_equal(r.objective, ob)
    dev.close()
