"""Seeded generators (benchmark/src/generators.rs) and the datafile format
(benchmark/src/datafile.rs), host only.  The size/selectivity/density checks
follow the reference's dataset validator (benchmark/src/bin/datatest.rs:109-238)."""
from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import GOLDEN
from simd_set_operations_gb300 import datasets as ds


def strictly_increasing(a):
    return a.size < 2 or bool(np.all(a[1:] > a[:-1]))


@pytest.mark.parametrize("small,large,dens,sel", [
    (1 << 12, 1 << 12, 0.1, 0.1), (1 << 10, 1 << 16, 0.05, 0.01),
    (100, 100, 0.9, 1.0), (1000, 5000, 0.5, 0.0)])
def test_twoset_shape(small, large, dens, sel):
    s, l = ds.gen_twoset(7, dens, sel, small, large)
    assert s.size == small and l.size == large
    assert strictly_increasing(s) and strictly_increasing(l)
    m = int(large / dens)
    assert int(max(s.max(), l.max())) < m
    shared = np.intersect1d(s, l).size
    want = int(sel * small)
    if small + large - want <= m:
        assert shared == want
    s2, l2 = ds.gen_twoset(7, dens, sel, small, large)
    assert np.array_equal(s, s2) and np.array_equal(l, l2)
    s3, _ = ds.gen_twoset(8, dens, sel, small, large)
    assert not np.array_equal(s, s3)


def test_twoset_density_cap():
    # generators.rs:46-50: selectivity is raised when the domain is too small
    s, l = ds.gen_twoset(1, 1.0, 0.0, 100, 100)
    assert s.size == 100 and l.size == 100
    assert np.intersect1d(s, l).size == 100


def test_kset_shape():
    lens = ds.kset_lens(1 << 14, 1.0, 5)
    assert lens == sorted(lens) and lens[-1] == 1 << 14 and lens[0] == (1 << 14) // 5
    sets = ds.gen_kset(3, 0.2, 0.05, 1 << 14, 1.0, 5)
    core = sets[0]
    for s, n in zip(sets, lens):
        assert s.size == n and strictly_increasing(s)
        core = np.intersect1d(core, s)
    assert core.size >= int(0.05 * lens[0])


def test_batch_and_index():
    b = ds.gen_batch(11, 200, 16, 1 << 12, nthreads=3)
    b2 = ds.gen_batch(11, 200, 16, 1 << 12, nthreads=1)
    assert np.array_equal(b.pool, b2.pool)
    assert len(b) == 200
    assert b.a_len.min() >= 16 and b.a_len.max() <= 1 << 12
    for p in range(0, 200, 17):
        a, c = b.pair(p)
        assert strictly_increasing(a) and strictly_increasing(c)
    idx = ds.gen_index(5, 1000, max_len=1 << 12, s=1.1, doc_space=1 << 20, nthreads=2)
    assert idx.lens[0] == 1 << 12 and idx.lens[-1] >= 1
    assert np.all(np.diff(idx.lens.astype(np.int64)) <= 0)
    for i in (0, 1, 10, 999):
        v = idx.list(i)
        assert v.size == idx.lens[i] and strictly_increasing(v) and int(v.max()) < 1 << 20


def test_datafile_golden_roundtrip(tmp_path):
    g = json.loads((GOLDEN / "datafile_roundtrip.json").read_text())
    cases = dict(g["cases"])
    for name, ranges in g["range_cases"].items():
        cases[name] = [list(range(lo, hi)) for lo, hi in ranges]
    for name, sets in cases.items():
        p = tmp_path / f"{name}.dat"
        ds.datafile_write(p, sets)
        raw = p.read_bytes()
        assert list(raw[:3]) == g["magic"]
        assert int.from_bytes(raw[4:8], "little") == len(sets)
        back = ds.datafile_read(p)
        assert [x.tolist() for x in back] == sets, name


def test_datafile_errors(tmp_path):
    with pytest.raises(ds.DatafileError) as e:
        ds.datafile_write(tmp_path / "x.dat", [[1, 2]])
    assert e.value.code == -3
    p = tmp_path / "bad.dat"
    p.write_bytes(b"\x00\x01\x02\x01\x02\x00\x00\x00")
    with pytest.raises(ds.DatafileError) as e:
        ds.datafile_read(p)
    assert e.value.code == -4
    p.write_bytes(bytes([0xE9, 0xAA, 0x05, 0x00, 2, 0, 0, 0]))
    with pytest.raises(ds.DatafileError) as e:
        ds.datafile_read(p)
    assert e.value.code == -5
    with pytest.raises(ds.DatafileError):
        ds.datafile_read(tmp_path / "missing.dat")


def test_bsr_encode_batch_matches_oracle(orc):
    """The bench's host BSR encoder equals BsrVec::from_sorted
    (setops/src/bsr.rs:140-163) as the oracle restates it, set by set."""
    b = ds.gen_batch(5, 200, 1, 1 << 12, density=(0.5, 0.5))
    e = ds.bsr_encode_batch(b)
    assert len(e) == len(b)
    for p in range(len(b)):
        a, bb = b.pair(p)
        ba, sa, bb_, sb = e.pair(p)
        for (wb, ws), x in (((ba, sa), a), ((bb_, sb), bb)):
            ob, os_ = orc.bsr_from_sorted(x)
            assert np.array_equal(wb, ob) and np.array_equal(ws, os_), p
    # empty and one-element sets
    pool = np.array([7, 0, 31, 32, 0xFFFFFFFF], np.uint32)
    u = lambda x: np.array(x, np.uint64)  # noqa: E731
    e = ds.bsr_encode_batch(ds.PairBatch(pool, u([0, 1]), u([0, 1]), u([1, 2]), u([4, 3])))
    # pair 0: {} and {0, 31, 32, 2^32-1}; pair 1: {0} and {31, 32, 2^32-1}
    assert [int(x) for x in e.a_len] == [0, 1] and [int(x) for x in e.b_len] == [3, 3]
    ba, sa, bb, sb = e.pair(1)
    assert list(ba) == [0] and list(sa) == [1]
    assert list(bb) == [0, 1, 0x7FFFFFF] and list(sb) == [0x80000000, 1, 0x80000000]


def test_oracle_copy_of_the_generators_makes_the_same_inputs():
    """The timed CPU reference path generates its inputs with the oracle's
    build of the generator source (so that it maps no GPU library); those
    inputs must be the GPU path's."""
    import bench
    from simd_set_operations_gb300 import datasets as ds
    cds = bench.cpu_datasets()
    for args in ((7, 0.05, 0.01, 1 << 10, 1 << 16), (8, 0.1, 0.1, 5000, 5000)):
        for x, y in zip(ds.gen_twoset(*args), cds.gen_twoset(*args)):
            assert np.array_equal(x, y)
    b1, b2 = ds.gen_batch(3, 50, 16, 1 << 10), cds.gen_batch(3, 50, 16, 1 << 10)
    assert np.array_equal(b1.pool, b2.pool) and np.array_equal(b1.a_len, b2.a_len)
    k1, k2 = ds.gen_kset(5, 0.2, 0.05, 1 << 12, 1.0, 3), cds.gen_kset(5, 0.2, 0.05, 1 << 12, 1.0, 3)
    assert all(np.array_equal(x, y) for x, y in zip(k1, k2))
