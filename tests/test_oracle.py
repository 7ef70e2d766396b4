"""CPU tests: the oracle pinned against GLPK / glp_exact fixtures, the
reference's known answers, and the generator's determinism."""
import hashlib
import math

import numpy as np
import pytest

import simplexprojects_gb300 as sp
from oracle import ref, exact
from conftest import NETLIB, REFERENCE


def _fp(batch):
    h = hashlib.sha256()
    for a in (batch.m, batch.n, batch.A, batch.b, batch.c):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def test_generator_matches_fixture_fingerprints(built, workloads_golden):
    for kind, w in workloads_golden["workloads"].items():
        batch = sp.generate(int(kind), w["count"], seed=workloads_golden["seed"], first=w["first"])
        assert batch.m.tolist() == w["m"] and batch.n.tolist() == w["n"]
        assert _fp(batch) == w["sha256"], f"generator drift in kind {kind}"


def test_oracle_against_glpk_and_exact(built, workloads_golden):
    """Oracle statuses equal GLPK's and glp_exact's; FP64 objectives within
    1e-9 relative of the exact rational optimum."""
    for kind, w in workloads_golden["workloads"].items():
        batch = sp.generate(int(kind), w["count"], seed=workloads_golden["seed"], first=w["first"])
        r = ref.solve_batch(batch, "fp64")
        st = np.array([x["status"] for x in w["lps"]])
        est = np.array([x["exact_status"] for x in w["lps"]])
        ex = np.array([x["exact_objective"] for x in w["lps"]])
        assert np.array_equal(r.status, st), kind
        assert np.array_equal(r.status, est), kind
        opt = est == 5
        rel = np.abs(r.objective[opt] - ex[opt]) / np.maximum(np.abs(ex[opt]), 1.0)
        assert rel.max() <= 1e-9, (kind, rel.max())


def test_oracle_fp32_within_1e6(built, workloads_golden):
    for kind, w in workloads_golden["workloads"].items():
        batch = sp.generate(int(kind), w["count"], seed=workloads_golden["seed"], first=w["first"])
        r = ref.solve_batch(batch, "fp32")
        est = np.array([x["exact_status"] for x in w["lps"]])
        ex = np.array([x["exact_objective"] for x in w["lps"]])
        assert np.array_equal(r.status, est), kind
        opt = est == 5
        rel = np.abs(r.objective[opt] - ex[opt]) / np.maximum(np.abs(ex[opt]), 1.0)
        assert rel.max() <= 1e-6, (kind, rel.max())


def test_oracle_hand_lps(built, known_golden):
    """The reference's hand LPs: GLPK's verdicts, and the answers the
    reference's comments state (parseBenchmark.cpp:151-221) where correct."""
    for name, v in known_golden["hand"].items():
        batch = sp.LPBatch.from_lps([(v["A"], v["b"], v["c"])])
        r = ref.solve_batch(batch, "fp64")
        assert r.status[0] == v["exact_status"], name
        if v["exact_status"] == 5:
            assert math.isclose(r.objective[0], v["exact_objective"], rel_tol=1e-12, abs_tol=1e-12), name
        if v["stated"] is not None:
            assert abs(r.objective[0] - v["stated"]) < 1e-4, name


def test_exact_fraction_simplex_agrees(built, known_golden):
    """The pure-Python rational simplex (travels to any host) reproduces
    glp_exact on the hand LPs and on small seeded LPs."""
    for name, v in known_golden["hand"].items():
        if len(v["A"]) > 12:
            continue
        st, obj = exact.solve(v["A"], v["b"], v["c"])
        assert st == v["exact_status"], name
        if st == 5:
            assert float(obj) == pytest.approx(v["exact_objective"], rel=1e-15, abs=1e-15)


def test_oracle_pivot_rules_deterministic(built):
    batch = sp.generate(4, 64, seed=5)
    a = ref.solve_batch(batch, "fp64", threads=1, want_basis=True)
    b = ref.solve_batch(batch, "fp64", threads=8, want_basis=True)
    assert np.array_equal(a.pivots, b.pivots) and np.array_equal(a.basis, b.basis)
    assert np.array_equal(a.objective.view(np.uint64), b.objective.view(np.uint64))


def test_oracle_netlib(built, known_golden):
    """The 8 Netlib LPs the reference ships (benchmarks/*.txt, committed copies
    in tests/golden/netlib): GLPK's verdict and its objective; listed Netlib
    optima to 1e-5."""
    assert len(known_golden["netlib"]) == 8
    for name, v in known_golden["netlib"].items():
        A, b, c = sp.read_abc(*(str(NETLIB / f"{name}_{s}.txt") for s in "ABC"))
        batch = sp.LPBatch.from_lps([(A, b, -c)])
        r = ref.solve_batch(batch, "fp64")
        assert r.status[0] == v["exact_status"], name
        if v["exact_status"] == 5:
            assert abs(r.objective[0] - v["exact_objective"]) <= 1e-7 * max(1, abs(v["exact_objective"])), name
            assert abs(-r.objective[0] - v["listed_min"]) <= 1e-5 * abs(v["listed_min"]), name


def test_generator_properties(built):
    b = sp.generate(1, 200, seed=3)
    assert set(np.unique(b.m)) <= {50, 56, 74, 105}
    assert (b.n >= b.m).all() and (b.n <= np.floor(1.8 * b.m)).all()
    assert (b.b >= 0).all() and (b.c > 0).all()
    b4 = sp.generate(4, 400, seed=3)
    assert b4.m.min() >= 16 and b4.m.max() <= 256
    assert ((b4.family >= 0).mean() > 0.2) and ((b4.family >= 0).mean() < 0.4)
    # independent per-LP streams: a sub-range regenerates identically
    sub = sp.generate(4, 10, seed=3, first=100)
    whole = b4.subset(range(100, 110))
    assert np.array_equal(sub.A, whole.A) and np.array_equal(sub.c, whole.c)


def test_family_sharing(built):
    b = sp.generate(3, 130, seed=9, share_family_A=True)
    assert b.A.size == 64 * 174 * 142
    full = sp.generate(3, 130, seed=9)
    for k in (0, 64, 129):
        assert np.array_equal(b.lp(k)[0], full.lp(k)[0])


@pytest.mark.skipif(not (REFERENCE / "benchmarks").exists(), reason="reference checkout absent")
def test_netlib_copies_match_reference():
    """The committed Netlib files are byte-for-byte the reference's."""
    for p in sorted(NETLIB.glob("*.txt")):
        assert p.read_bytes() == (REFERENCE / "benchmarks" / p.name).read_bytes(), p.name
    assert len(list(NETLIB.glob("*.txt"))) == 24
