"""GPU parity: the CUDA solver against the CPU oracle, through the C ABI.

FP64: the kernels apply the oracle's pivot rules with the same IEEE
operations (fused eliminations, divided pivot row), so statuses, pivot
counts, final bases, x and objectives must be BIT-IDENTICAL.
FP32: statuses and pivot counts identical to the FP32 oracle; objectives
within 1e-6 relative of the FP64 oracle (the FP32 form's tolerance).
"""
import numpy as np
import pytest

import simplexprojects_gb300 as sp
from oracle import ref

pytestmark = pytest.mark.gpu

FP32_REL = 1e-6


def _rel(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1.0)


def assert_bit_identical(gpu, cpu):
    assert np.array_equal(gpu.status, cpu.status)
    assert np.array_equal(gpu.pivots, cpu.pivots)
    assert np.array_equal(gpu.objective.view(np.uint64), cpu.objective.view(np.uint64))
    if gpu.basis is not None:
        assert np.array_equal(gpu.basis, cpu.basis)
    if gpu.x is not None:
        assert np.array_equal(gpu.x.view(np.uint64), cpu.x.view(np.uint64))


@pytest.mark.parametrize("kind,count", [(0, 512), (1, 512), (2, 16), (3, 64), (4, 384)])
def test_fp64_bit_identical(built, kind, count):
    batch = sp.generate(kind, count, seed=sp.DEFAULT_SEED + 17 * kind)
    gpu = sp.solve(batch, "fp64", want_x=True, want_basis=True)
    cpu = ref.solve_batch(batch, "fp64", want_x=True, want_basis=True)
    assert_bit_identical(gpu, cpu)


@pytest.mark.parametrize("min_cluster", [2, 4, 8])
def test_fp64_cluster_split_bit_identical(built, min_cluster):
    """Tableaux split across 2/4/8 CTAs (DSMEM exchange) give the same bits."""
    batch = sp.generate(1, 96, seed=99)
    gpu = sp.solve(batch, "fp64", want_x=True, want_basis=True, min_cluster=min_cluster)
    cpu = ref.solve_batch(batch, "fp64", want_x=True, want_basis=True)
    assert_bit_identical(gpu, cpu)


@pytest.mark.parametrize("kind,count", [(0, 256), (1, 256), (3, 32), (4, 256)])
def test_fp32_against_oracle(built, kind, count):
    batch = sp.generate(kind, count, seed=5 + kind)
    g32 = sp.solve(batch, "fp32", want_basis=True)
    c32 = ref.solve_batch(batch, "fp32", want_basis=True)
    c64 = ref.solve_batch(batch, "fp64")
    assert np.array_equal(g32.status, c32.status)
    assert np.array_equal(g32.status, c64.status)
    # same FP32 pivot sequence unless the final FP64 check sent the LP back
    # for repair pivots (BLPG_INFO_REPAIR) or the FP64 pass re-solved it
    clean = (g32.info & (32 | 1024)) == 0
    assert np.array_equal(g32.pivots[clean], c32.pivots[clean])
    opt = c64.status == 5
    assert (g32.info[opt] & (16 | 1024)).all()  # FP64-refreshed, or re-solved in FP64
    assert _rel(g32.objective[opt], c64.objective[opt]).max() <= FP32_REL


def test_fp32_cluster_split(built):
    """The FP64 refresh reads and writes other CTAs' columns through DSMEM:
    the same results with the tableau split over 1, 2 or 4 CTAs."""
    batch = sp.generate(4, 64, seed=3)
    a = sp.solve(batch, "fp32", want_x=True)
    for K in (2, 4):
        b = sp.solve(batch, "fp32", min_cluster=K, want_x=True)
        assert np.array_equal(a.status, b.status)
        assert np.array_equal(a.pivots, b.pivots)
        assert np.array_equal(a.objective, b.objective)
        assert np.array_equal(a.x, b.x)


@pytest.mark.parametrize("period", [16, 32, 64])
def test_fp32_periodic_refresh(built, period):
    """FP64 refresh every k pivots (and at termination): statuses exact,
    objectives within 1e-6 of the exact optimum."""
    batch = sp.generate(2, 24, seed=21)
    c64 = ref.solve_batch(batch, "fp64")
    g = sp.solve(batch, "fp32", refactor_period=period)
    assert np.array_equal(g.status, c64.status)
    opt = c64.status == 5
    assert _rel(g.objective[opt], c64.objective[opt]).max() <= FP32_REL


def test_golden_statuses_and_exact_objectives(built, workloads_golden):
    """GLPK's statuses exactly; objectives within 1e-9 (FP64) / 1e-6 (FP32)
    of glp_exact's rational optimum."""
    for kind, w in workloads_golden["workloads"].items():
        batch = sp.generate(int(kind), w["count"], seed=workloads_golden["seed"], first=w["first"])
        st = np.array([r["exact_status"] for r in w["lps"]])
        ex = np.array([r["exact_objective"] for r in w["lps"]])
        for prec, tol in (("fp64", 1e-9), ("fp32", FP32_REL)):
            g = sp.solve(batch, prec)
            assert np.array_equal(g.status, st), (kind, prec)
            opt = st == 5
            assert _rel(g.objective[opt], ex[opt]).max() <= tol, (kind, prec)


def test_two_phase_known_answers(built, known_golden):
    """The reference's hand LPs (several need phase I): GLPK's status and
    objective, and bit-identical to the oracle."""
    lps = list(known_golden["hand"].items())
    batch = sp.LPBatch.from_lps([(v["A"], v["b"], v["c"]) for _, v in lps])
    gpu = sp.solve(batch, "fp64", want_x=True, want_basis=True)
    cpu = ref.solve_batch(batch, "fp64", want_x=True, want_basis=True)
    assert_bit_identical(gpu, cpu)
    for k, (name, v) in enumerate(lps):
        assert gpu.status[k] == v["exact_status"], name
        if v["exact_status"] == 5:
            assert abs(gpu.objective[k] - v["exact_objective"]) <= 1e-9 * max(1, abs(v["exact_objective"])), name


def test_reference_batch_mode_shared_A_b(built):
    """One A, b and one objective per LP (Simplex::setConstratint + ComputeLP)."""
    base = sp.generate(1, 1, seed=1234)
    A, b, _ = base.lp(0)
    rng = np.random.default_rng(0)
    C = rng.uniform(-1, 5, size=(300, A.shape[1]))
    s = sp.Simplex(300, 0)
    s.setConstratint(A, b)
    s.ComputeLP(C, 10)
    batch = sp.LPBatch.shared(A, b, C)
    cpu = ref.solve_batch(batch, "fp64")
    assert np.array_equal(s.getStatusAll(), cpu.status)
    assert np.array_equal(s.getResultAll().view(np.uint64), cpu.objective.view(np.uint64))
    assert s.getResult(3) == cpu.objective[2] and s.getStatus(3) == cpu.status[2]


def test_device_plan_graph_replay(built):
    """Device-resident plan: graph replays give identical results."""
    import torch
    batch = sp.generate(1, 256, seed=77)
    db = sp.DeviceBatch(batch, "fp64", want_x=True, want_basis=True)
    outs = []
    for _ in range(3):
        db.status.zero_()
        db.objective.zero_()
        db.run()
        outs.append(db.result())
    torch.cuda.synchronize()
    cpu = ref.solve_batch(batch, "fp64", want_x=True, want_basis=True)
    for o in outs:
        assert_bit_identical(o, cpu)
    assert db.plan.launches() == len(db.plan.classes())


def test_edge_cases(built):
    lps = [
        (np.array([[1.0]]), np.array([2.0]), np.array([3.0])),          # m = n = 1
        (np.ones((3, 4)), np.ones(3), np.zeros(4)),                      # c = 0: optimal at start
        (np.array([[-1.0, 1.0]]), np.array([1.0]), np.array([1.0, 0.0])),  # unbounded
        (np.array([[1.0, 1.0], [1.0, -1.0]]), np.array([0.0, 0.0]), np.array([1.0, 1.0])),  # degenerate
        (np.zeros((2, 2)), np.array([1.0, 1.0]), np.array([-1.0, -2.0])),  # all-zero A
    ]
    batch = sp.LPBatch.from_lps(lps)
    gpu = sp.solve(batch, "fp64", want_x=True, want_basis=True)
    cpu = ref.solve_batch(batch, "fp64", want_x=True, want_basis=True)
    assert_bit_identical(gpu, cpu)
    assert gpu.status.tolist() == [5, 5, 6, 5, 5]
    assert gpu.objective[0] == 6.0 and gpu.pivots[1] == 0 and gpu.objective[3] == 0.0


def test_largest_workload_shape(built):
    """m = 256, n = 512 (the largest kind-4 shape): FP64 needs an 8-CTA cluster."""
    rng = np.random.default_rng(3)
    A = rng.uniform(0, 1, (256, 512)) * (rng.uniform(size=(256, 512)) < 0.3)
    b = rng.uniform(1, 10, 256)
    c = rng.uniform(1, 5, 512)
    batch = sp.LPBatch.from_lps([(A, b, c)])
    plan = sp.Plan(batch, "fp64")
    assert plan.classes()[0]["cluster"] == 8
    plan.close()
    gpu = sp.solve(batch, "fp64", want_x=True, want_basis=True)
    cpu = ref.solve_batch(batch, "fp64", want_x=True, want_basis=True)
    assert_bit_identical(gpu, cpu)


def test_empty_batch_and_errors(built):
    empty = sp.LPBatch(np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0))
    r = sp.solve(empty)
    assert r.status.size == 0
    bad = sp.LPBatch(np.array([0]), np.array([2]), np.zeros(0), np.zeros(0), np.zeros(2))
    with pytest.raises(sp._native.BlpgError) as e:
        sp.solve(bad)
    assert e.value.code == -1
    big = sp.LPBatch.from_lps([(np.ones((900, 900)), np.ones(900), np.ones(900))])
    with pytest.raises(sp._native.BlpgError) as e:
        sp.solve(big)
    assert e.value.code == -5


@pytest.mark.parametrize("kind,period", [(1, 0), (1, 16), (4, 16)])
def test_fp32_solutions_are_feasible(built, kind, period):
    """The x reported in FP32 mode belongs to the final basis: FP64-refreshed,
    so Ax <= b and x >= 0 hold to rounding for optimal LPs and for the basic
    solution where unboundedness was found (with periodic refreshes the last
    refresh may precede later pivots, and its x must not be reported)."""
    batch = sp.generate(kind, 512, seed=41 + kind)
    g = sp.solve(batch, "fp32", refactor_period=period, want_x=True)
    _, _, oc = batch.offsets()
    for k in range(batch.count):
        if g.status[k] not in (5, 6):
            continue
        A, b, _ = batch.lp(k)
        xk = g.x[oc[k]:oc[k] + A.shape[1]]
        # the FP64 check accepts x_B >= -1e-7 (the FP32 mode's primal tolerance)
        scale = max(1.0, float(np.abs(b).max()), float(np.abs(xk).max()))
        assert (A @ xk - b).max() <= 1e-7 * scale, (k, g.status[k])
        assert xk.min() >= -1e-7 * scale, (k, g.status[k])


def _shared_A(kind, count):
    """A batch whose LPs share A: workload 3's families, or workload 0 in the
    reference's batch mode (every LP on LP 0's A)."""
    if kind == 3:
        return sp.generate(3, count, seed=80, share_family_A=True)
    g = sp.generate(0, count, seed=77)
    m, n = int(g.m[0]), int(g.n[0])
    assert (g.m == m).all() and (g.n == n).all()
    return sp.LPBatch(g.m, g.n, g.A[:m * n].copy(), g.b, g.c,
                      off_A=np.zeros(count, np.int64), off_b=g.off_b, off_c=g.off_c)


@pytest.mark.parametrize("kind,count", [(0, 256), (3, 256)])
def test_fp32_shared_A_copy_matches_private_A(built, kind, count):
    """LPs that share A (each element read by two LPs or more) are loaded from
    the plan's FP32 copy of A; the same LPs with a private copy of A each are
    converted by the loaders.  Both give the same FP32 tableau, hence the same
    bits."""
    shared = _shared_A(kind, count)
    oA, _, _ = shared.offsets()
    reads = int((shared.m.astype(np.int64) * shared.n).sum())
    assert reads >= 2 * len(shared.A)  # the plan makes the copy
    parts = [shared.A[oA[k]:oA[k] + int(shared.m[k]) * int(shared.n[k])] for k in range(count)]
    private = sp.LPBatch(shared.m, shared.n, np.concatenate(parts), shared.b, shared.c,
                         off_b=shared.off_b, off_c=shared.off_c)
    for pricing in ("dantzig", "steepest"):
        a = sp.solve(shared, "fp32", pricing=pricing, want_x=True)
        b = sp.solve(private, "fp32", pricing=pricing, want_x=True)
        assert np.array_equal(a.status, b.status)
        assert np.array_equal(a.pivots, b.pivots)
        assert np.array_equal(a.objective, b.objective)
        assert np.array_equal(a.x, b.x)


def test_fp32_shared_A_copy_phase_one(built):
    """Phase-I LPs (some b_i < 0: negated rows, a zero objective row until
    phase II) loaded from the FP32 copy of a shared A give the bits of the
    in-kernel conversion and the oracle's statuses.  A has mixed signs and
    b = A x0 + slack for x0 >= 0, so every LP is feasible."""
    base = _shared_A(0, 256)
    m, n = int(base.m[0]), int(base.n[0])
    rng = np.random.default_rng(5)
    A = base.A.copy().reshape(m, n)
    A[rng.random((m, n)) < 0.3] *= -1
    x0 = rng.random((256, n)) * (rng.random((256, n)) < 0.3)
    b = (x0 @ A.T + rng.random((256, m)) * 0.5).reshape(-1)
    shared = sp.LPBatch(base.m, base.n, A.reshape(-1), b, base.c, off_A=base.off_A,
                        off_c=base.off_c)
    assert (b.reshape(256, m) < 0).any(1).sum() > 200  # most LPs need phase I
    private = sp.LPBatch(base.m, base.n, np.tile(A.reshape(-1), 256), b, base.c,
                         off_c=base.off_c)
    c64 = ref.solve_batch(shared, "fp64")
    for pricing in ("dantzig", "steepest"):
        a = sp.solve(shared, "fp32", pricing=pricing, want_x=True)
        p = sp.solve(private, "fp32", pricing=pricing, want_x=True)
        assert np.array_equal(a.status, p.status)
        assert np.array_equal(a.pivots, p.pivots)
        assert np.array_equal(a.objective, p.objective)
        assert np.array_equal(a.x, p.x)
        assert np.array_equal(a.status, c64.status)
        # every phase-I optimum verified in FP64 by the factorised refresh
        # (or re-solved by the plan's FP64 pass): objectives within 1e-6
        opt = c64.status == 5
        assert (a.info[opt] & (16 | 1024)).all(), pricing
        assert _rel(a.objective[opt], c64.objective[opt]).max() <= FP32_REL, pricing
