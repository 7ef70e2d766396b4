"""The size-class tuning table: per-class entries change the plan's classes
(threads per CTA, CTAs per SM) and leave results bit-identical (the pivot
rules do not depend on the launch shape); a null table restores the table
compiled into the library (tuning/gb300.json, written by autotune.py)."""
import numpy as np
import pytest

import simplexprojects_gb300 as sp
from simplexprojects_gb300 import autotune
from conftest import ROOT

pytestmark = pytest.mark.gpu


def _classes(batch, prec, **kw):
    plan = sp.Plan(batch, prec, **kw)
    c = plan.classes()
    plan.close()
    return c


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_class_entries_change_the_plan_not_the_results(built, prec):
    batch = sp.generate(4, 600, seed=12)
    try:
        autotune.reset()
        base = _classes(batch, prec)
        want = sp.solve(batch, prec, want_x=True)
        one = max(base, key=lambda c: c["lps"])  # the largest class
        key = one["key"]
        nt = 64 if one["threads"] > 64 else 128
        autotune.override({f"{prec}_c{key}": nt})  # the compiled-in table, one entry changed
        tuned = _classes(batch, prec)
        changed = [c for c in tuned if c["key"] == key]
        assert changed and changed[0]["threads"] != one["threads"]
        others = {c["key"]: c["threads"] for c in tuned if c["key"] != key}
        assert others == {c["key"]: c["threads"] for c in base if c["key"] != key}
        got = sp.solve(batch, prec, want_x=True)  # the cached plan is rebuilt
        assert np.array_equal(got.status, want.status)
        assert np.array_equal(got.pivots, want.pivots)
        assert np.array_equal(got.objective.view(np.uint64), want.objective.view(np.uint64))
        assert np.array_equal(got.x.view(np.uint64), want.x.view(np.uint64))
    finally:
        autotune.reset()
    assert _classes(batch, prec) == base


def test_compiled_in_table_is_the_committed_one(built):
    """Loading tuning/gb300.json gives the classes of the default table."""
    path = ROOT / "simplexprojects_gb300" / "tuning" / "gb300.json"
    if not path.exists():
        pytest.skip("no committed tuning table")
    batch = sp.generate(4, 400, seed=13, share_family_A=True)
    try:
        autotune.reset()
        default = _classes(batch, "fp32", pricing="steepest")
        autotune.load(str(path))
        assert _classes(batch, "fp32", pricing="steepest") == default
    finally:
        autotune.reset()
