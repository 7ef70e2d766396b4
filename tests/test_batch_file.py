"""The binary batch container (blpg_write_batch / blpg_read_batch) and the
per-LP results text (blpg_write_results): round trips keep every value and
every offset bit for bit, shared A stays shared, damaged files are refused."""
import subprocess

import numpy as np
import pytest

import simplexprojects_gb300 as sp
from simplexprojects_gb300 import build as B

KIND1 = dict(kind=1, count=40, seed=31)


def _packed_offsets(sizes):
    return np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)


def _same(a, b):
    return np.array_equal(np.atleast_1d(a).view(np.uint8), np.atleast_1d(b).view(np.uint8))


def test_packed_batch_round_trip(built, tmp_path):
    batch = sp.generate(KIND1["kind"], KIND1["count"], seed=KIND1["seed"])
    path = tmp_path / "k1.blpg"
    sp.write_batch(path, batch)
    got = sp.read_batch(path)
    assert got.count == batch.count
    for f in ("m", "n", "A", "b", "c"):
        assert _same(getattr(got, f), getattr(batch, f)), f
    mn = batch.m.astype(np.int64) * batch.n
    assert np.array_equal(got.off_A, _packed_offsets(mn))
    assert np.array_equal(got.off_b, _packed_offsets(batch.m))
    assert np.array_equal(got.off_c, _packed_offsets(batch.n))


def test_shared_A_stays_shared(built, tmp_path):
    batch = sp.generate(4, 60, seed=32, share_family_A=True)
    assert batch.off_A is not None
    path = tmp_path / "k4.blpg"
    sp.write_batch(path, batch)
    got = sp.read_batch(path)
    for f in ("m", "n", "off_A", "off_b", "off_c"):
        assert np.array_equal(getattr(got, f), getattr(batch, f)), f
    need = int((batch.off_A + batch.m.astype(np.int64) * batch.n).max())
    assert got.A.size == need < int((batch.m.astype(np.int64) * batch.n).sum())
    assert _same(got.A, batch.A[:need])
    assert _same(got.b, batch.b[:got.b.size]) and _same(got.c, batch.c[:got.c.size])
    header = 8 + 8 + 32
    per_lp = 2 * 4 + 3 * 8
    body = 8 * (got.A.size + got.b.size + got.c.size)
    assert path.stat().st_size == header + per_lp * batch.count + body


def test_empty_batch_round_trip(built, tmp_path):
    e = np.empty(0)
    empty = sp.LPBatch(np.empty(0, np.int32), np.empty(0, np.int32), e, e, e)
    path = tmp_path / "empty.blpg"
    sp.write_batch(path, empty)
    got = sp.read_batch(path)
    assert got.count == 0 and got.A.size == got.b.size == got.c.size == 0


def test_damaged_files_are_refused(built, tmp_path):
    batch = sp.generate(1, 5, seed=33)
    path = tmp_path / "ok.blpg"
    sp.write_batch(path, batch)
    raw = path.read_bytes()
    bad = tmp_path / "bad.blpg"
    bad.write_bytes(b"NOTABATC" + raw[8:])
    with pytest.raises(sp.BlpgError) as e:
        sp.read_batch(bad)
    assert e.value.code == -6 and "not a batch file" in str(e.value)
    bad.write_bytes(raw[:-8])                       # one double short
    with pytest.raises(sp.BlpgError) as e:
        sp.read_batch(bad)
    assert e.value.code == -6 and "truncated" in str(e.value)
    off = bytearray(raw)                            # LP 0's off_A beyond the stored A
    pos = 48 + 2 * 4 * batch.count
    off[pos:pos + 8] = np.int64(batch.A.size).tobytes()
    bad.write_bytes(bytes(off))
    with pytest.raises(sp.BlpgError) as e:
        sp.read_batch(bad)
    assert e.value.code == -6 and "outside" in str(e.value)
    with pytest.raises(sp.BlpgError):
        sp.read_batch(tmp_path / "missing.blpg")


def test_results_text_reads_back_bit_for_bit(built, tmp_path):
    batch = sp.generate(1, 6, seed=34)
    rng = np.random.default_rng(0)
    status = rng.integers(1, 7, batch.count).astype(np.int32)
    obj = rng.standard_normal(batch.count) * 1e3
    obj[0] = -0.0
    x = rng.standard_normal(int(batch.n.sum())) / 3.0
    path = tmp_path / "res.txt"
    sp.write_results(path, batch, status, obj, x)
    lines = path.read_text().splitlines()
    assert len(lines) == batch.count
    oc = _packed_offsets(batch.n)
    for k, line in enumerate(lines):
        f = line.split()
        assert int(f[0]) == status[k]
        assert _same(np.float64(f[1]), obj[k])
        xs = np.array([float(v) for v in f[2:]])
        assert xs.size == batch.n[k] and _same(xs, x[oc[k]:oc[k] + batch.n[k]])
    sp.write_results(path, batch, status, obj)      # without x: two fields a line
    assert all(len(l.split()) == 2 for l in path.read_text().splitlines())


def test_cli_batch_mode_rejects_a_bad_precision(built, tmp_path):
    r = subprocess.run([str(B.CLI), str(tmp_path / "x.blpg"), "1", "-", "16", "3"],
                       capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stdout


def test_cli_batch_mode_reports_a_missing_file(built, tmp_path):
    r = subprocess.run([str(B.CLI), str(tmp_path / "missing.blpg"), "1", "-", "64", "3"],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("bits", [64, 32])
def test_cli_batch_mode_matches_the_library(built, tmp_path, bits):
    """blpg_cli mode 3 on a batch file: the results file holds what
    sp.solve returns for the same batch (FP64 bit for bit; FP32 statuses and
    verified optima)."""
    batch = sp.generate(4, 300, seed=35, share_family_A=True)
    path, out = tmp_path / "k4.blpg", tmp_path / "res.txt"
    sp.write_batch(path, batch)
    r = subprocess.run([str(B.CLI), str(path), "1", str(out), str(bits), "3"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    want = sp.solve(batch, f"fp{bits}", want_x=True)
    lines = out.read_text().splitlines()
    assert len(lines) == batch.count
    st = np.array([int(l.split()[0]) for l in lines], np.int32)
    ob = np.array([float(l.split()[1]) for l in lines])
    assert np.array_equal(st, want.status)
    if bits == 64:
        assert _same(ob, want.objective)
        for k, l in enumerate(lines):
            xs = np.array([float(v) for v in l.split()[2:]])
            o = batch.off_c[k] if batch.off_c is not None else int(batch.n[:k].sum())
            assert _same(xs, want.x[o:o + batch.n[k]])
    else:
        ok = want.status == 5
        assert np.allclose(ob[ok], want.objective[ok], rtol=1e-9, atol=1e-9)


def test_unsupported_version_and_bad_header(built, tmp_path):
    batch = sp.generate(1, 3, seed=36)
    path = tmp_path / "ok.blpg"
    sp.write_batch(path, batch)
    raw = bytearray(path.read_bytes())
    bad = tmp_path / "bad.blpg"
    v2 = bytearray(raw)
    v2[8:12] = np.uint32(2).tobytes()               # version 2
    bad.write_bytes(bytes(v2))
    with pytest.raises(sp.BlpgError) as e:
        sp.read_batch(bad)
    assert e.value.code == -6 and "version" in str(e.value)
    neg = bytearray(raw)
    neg[16:24] = np.int64(-1).tobytes()             # count
    bad.write_bytes(bytes(neg))
    with pytest.raises(sp.BlpgError) as e:
        sp.read_batch(bad)
    assert e.value.code == -6 and "header" in str(e.value)
    bad.write_bytes(bytes(raw[:20]))                # cut inside the sizes
    with pytest.raises(sp.BlpgError):
        sp.read_batch(bad)


def test_header_claiming_more_data_than_the_file_holds(built, tmp_path):
    """A damaged size in the header is refused before any buffer is sized
    from it (the first call of the two already fails)."""
    batch = sp.generate(1, 4, seed=37)
    path = tmp_path / "ok.blpg"
    sp.write_batch(path, batch)
    raw = bytearray(path.read_bytes())
    for field, value in ((24, 10**15), (32, 2**62), (40, 3)):   # nA, nb, nc
        bad = bytearray(raw)
        bad[field:field + 8] = np.int64(value).tobytes()
        p = tmp_path / f"bad{field}.blpg"
        p.write_bytes(bytes(bad))
        with pytest.raises(sp.BlpgError) as e:
            sp.read_batch(p)
        assert e.value.code == -6 and ("damaged" in str(e.value) or "header" in str(e.value))
    longer = tmp_path / "longer.blpg"
    longer.write_bytes(bytes(raw) + b"\0" * 8)      # trailing bytes: not this batch's file
    with pytest.raises(sp.BlpgError):
        sp.read_batch(longer)
