"""CPU tests of the C-ABI library: it loads, exports every function that
include/blpg.h declares, and its host-only entry points work without a GPU."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import simplexprojects_gb300 as sp
from simplexprojects_gb300 import _native as N
from conftest import ROOT, has_gpu


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(blpg_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol(built):
    L = C.CDLL(str(N.LIB_PATH))
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) <= set(N.SIGNATURES), set(names) - set(N.SIGNATURES)


def test_version_and_options(built):
    assert "sm_103a" in sp.version()
    o = sp.options("fp32", max_pivots=7)
    assert o.precision == 1 and o.use_graph == 1 and o.max_cluster == 8 and o.max_pivots == 7


@pytest.mark.skipif(has_gpu(), reason="checks the no-GPU error path")
def test_solve_without_gpu_fails_loudly(built):
    batch = sp.generate(0, 4, seed=1)
    with pytest.raises(N.BlpgError) as e:
        sp.solve(batch)
    assert e.value.code == -2  # BLPG_ENODEV: no CPU fallback


def test_read_abc(tmp_path, built):
    (tmp_path / "A.txt").write_text("2 3\n1 0 -0\n0.5 2 3\n")
    (tmp_path / "B.txt").write_text("4\n5\n")
    (tmp_path / "C.txt").write_text("1\n2\n3\n")
    A, b, c = sp.read_abc(*(str(tmp_path / f) for f in ("A.txt", "B.txt", "C.txt")))
    assert A.tolist() == [[1, 0, 0], [0.5, 2, 3]] and b.tolist() == [4, 5] and c.tolist() == [1, 2, 3]
    with pytest.raises(N.BlpgError):
        sp.read_abc(str(tmp_path / "nope"), str(tmp_path / "B.txt"), str(tmp_path / "C.txt"))


def test_set_tuning_parses(built):
    assert N.lib().blpg_set_tuning(b'{"fp64_k1": 256, "fp32_k2": 384}') == 0
    assert N.lib().blpg_set_tuning(None) == 0


def test_shared_batch_layout(built):
    A = np.arange(6.0).reshape(2, 3)
    bt = sp.LPBatch.shared(A, [1, 2], np.ones((4, 3)))
    assert bt.count == 4 and bt.off_A.tolist() == [0, 0, 0, 0]
    assert np.array_equal(bt.lp(3)[0], A)


def test_batch_view_copies_are_independent(built):
    """LPBatch.c_struct reuses one ctypes view while the arrays stay the same
    objects, hands out copies (a caller nulling a field does not change the
    next view) and rebuilds the view when an array is replaced."""
    b = sp.generate(1, 20, seed=3)
    first = b.c_struct()
    first.A = None
    first.c = None
    again = b.c_struct()
    assert C.addressof(again.A.contents) == b.A.ctypes.data
    assert C.addressof(again.c.contents) == b.c.ctypes.data
    b.c = b.c.copy()
    assert C.addressof(b.c_struct().c.contents) == b.c.ctypes.data


def test_batch_offsets_packed_and_given(built):
    """LPBatch.offsets(): offsets a batch carries come back as they are;
    missing ones are the packed layout (each LP right after the previous)."""
    b = sp.generate(1, 30, seed=5)
    oA, ob, oc = b.offsets()
    m, n = b.m.astype(np.int64), b.n.astype(np.int64)
    assert np.array_equal(oA, np.concatenate([[0], np.cumsum(m * n)[:-1]]))
    assert np.array_equal(ob, np.concatenate([[0], np.cumsum(m)[:-1]]))
    assert np.array_equal(oc, np.concatenate([[0], np.cumsum(n)[:-1]]))
    assert oA.dtype == ob.dtype == oc.dtype == np.int64
    shared = sp.generate(4, 40, seed=6, share_family_A=True)
    sA, sb, sc = shared.offsets()
    assert sA is shared.off_A
    e = np.empty(0)
    empty = sp.LPBatch(np.empty(0, np.int32), np.empty(0, np.int32), e, e, e)
    assert all(o.size == 0 for o in empty.offsets())
