"""The CPU oracle, pinned against the reference's golden vectors.

* known-answer tests of setops/tests/unit_tests.rs (fixture unit_tests.json);
* outputs of the reference's own C++ kernels (qfilter.cpp) on seeded inputs
  (fixture ref_kernels.npz, made by tests/golden/make_golden.py);
* the reference's property definitions (setops/tests/testlib/properties.rs)
  and its BSR round trip (setops/tests/property_tests.rs:728-730).
"""
from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import GOLDEN, pair_with_overlap, rand_set


def props_intersection_correct(result, sets):
    """prop_intersection_correct (testlib/properties.rs:2-50)."""
    r = np.asarray(result)
    if r.size > 1 and not np.all(r[1:] > r[:-1]):
        return False
    common = sets[0]
    for s in sets[1:]:
        common = np.intersect1d(common, s)
    return np.array_equal(np.sort(r), common)


def test_unit_test_kats(orc):
    kat = json.loads((GOLDEN / "unit_tests.json").read_text())
    fns = [orc.naive_merge, orc.branchless_merge, orc.shuffling_w8,
           orc.simd_galloping_w16, orc.bmiss_w4]
    for case in kat["twoset"]:
        for f in fns:
            assert f(case["a"], case["b"]).tolist() == case["expected"], (case["name"], f)
        s, l = sorted([case["a"], case["b"]], key=len)
        assert orc.galloping(s, l).tolist() == case["expected"]
    g = kat["galloping"]
    large = np.arange(*g["large_range"], dtype=np.uint32)
    for f in (orc.galloping, orc.simd_galloping_w16, orc.branchless_merge):
        assert f(g["small"], large).tolist() == g["expected"]


def test_pinned_to_reference_kernels(orc):
    z = np.load(GOLDEN / "ref_kernels.npz")
    n = len(z["kinds"])
    assert n >= 20
    for i in range(n):
        a, b = z[f"a{i}"], z[f"b{i}"]
        want = orc.naive_merge(a, b)
        assert np.array_equal(z[f"bmiss{i}"], want)
        assert np.array_equal(z[f"qfilter{i}"], want)
        ba, sa = orc.bsr_from_sorted(a)
        bb, sb = orc.bsr_from_sorted(b)
        ob, os_ = orc.branchless_merge_bsr(ba, sa, bb, sb)
        assert np.array_equal(ob, z[f"qbsr_bases{i}"])
        assert np.array_equal(os_, z[f"qbsr_states{i}"])


def test_reference_kernels_live_if_built(orc):
    """On x86 hosts with the reference tree, re-run its C++ kernels."""
    if orc.ref_lib() is None:
        pytest.skip("reference kernels not built on this host")
    rng = np.random.default_rng(5)
    for n in (0, 1, 7, 64, 1000):
        a, b = pair_with_overlap(rng, n + 3, 2 * n + 5, n // 2, hi=1 << 31)
        assert np.array_equal(orc.ref_two("intersect_bmiss_uint_b4", a, b), orc.naive_merge(a, b))


@pytest.mark.parametrize("seed", range(6))
def test_baselines_equal_naive_merge(orc, seed):
    rng = np.random.default_rng(seed)
    for na, nb, sh in [(0, 10, 0), (5, 0, 0), (1, 1, 1), (17, 33, 9), (1000, 1000, 300),
                       (64, 5000, 40), (3000, 129, 100), (4096, 4096, 4096)]:
        a, b = pair_with_overlap(rng, na, nb, sh)
        want = orc.naive_merge(a, b)
        assert orc.naive_merge_count(a, b) == want.size
        for f in (orc.branchless_merge, orc.shuffling_w8, orc.simd_galloping_w16, orc.bmiss_w4):
            assert np.array_equal(f(a, b), want), f
        s, l = (a, b) if a.size <= b.size else (b, a)
        assert np.array_equal(orc.galloping(s, l), want)
        assert np.array_equal(orc.binary_search_intersect(s, l), want)
        assert props_intersection_correct(want, [a, b])


def test_high_values_unsigned_order(orc):
    a = np.array([0, 5, 2**31 - 1, 2**31, 2**31 + 7, 2**32 - 2, 2**32 - 1], np.uint32)
    b = np.array([5, 2**31, 2**31 + 8, 2**32 - 1], np.uint32)
    assert orc.naive_merge(a, b).tolist() == [5, 2**31, 2**32 - 1]
    assert orc.shuffling_w8(a, b).tolist() == [5, 2**31, 2**32 - 1]


def test_binary_search_semantics(orc):
    """galloping.rs:110-131: match index, else the final lo."""
    arr = np.array([1, 3, 5, 7], np.uint32)
    assert orc.binary_search(arr, 5, 0, 3) == 2
    assert orc.binary_search(arr, 4, 0, 3) == 2
    assert orc.binary_search(arr, 9, 0, 3) == 4
    assert orc.binary_search(arr, 0, 0, 3) == 0


@pytest.mark.parametrize("seed", range(4))
def test_bsr_roundtrip_and_merge(orc, seed):
    rng = np.random.default_rng(100 + seed)
    for n, hi in [(0, 10), (1, 10), (50, 64), (1000, 3000), (5000, 1 << 32)]:
        s = rand_set(rng, n, hi)
        b, st = orc.bsr_from_sorted(s)
        assert np.all(st != 0)
        assert b.size == 0 or np.all(b[1:] > b[:-1])
        assert np.array_equal(orc.bsr_to_sorted(b, st), s)
    for n in (10, 500, 4000):
        a, c = pair_with_overlap(rng, n, 2 * n, n // 3, hi=8 * n)
        ba, sa = orc.bsr_from_sorted(a)
        bc, sc = orc.bsr_from_sorted(c)
        ob, os_ = orc.branchless_merge_bsr(ba, sa, bc, sc)
        # property_tests.rs:82-96: decoded BSR intersection == naive_merge
        assert np.array_equal(orc.bsr_to_sorted(ob, os_), orc.naive_merge(a, c))
        # property_tests.rs:539-550: Counter on BSR == Counter on arrays
        assert orc.branchless_merge_bsr_count(ba, sa, bc, sc) == orc.naive_merge_count(a, c)
        gb, gs = orc.galloping_bsr(ba, sa, bc, sc)
        assert np.array_equal(gb, ob) and np.array_equal(gs, os_)
        # broadcast_{sse,avx2,avx512}_bsr (broadcast.rs:163-357), the scheme of
        # the GPU's block-broadcast kernel: the same words for every width
        for w in (4, 8, 16):
            for x, y in (((ba, sa), (bc, sc)), ((bc, sc), (ba, sa))):
                bb_, bs_ = orc.broadcast_bsr(*x, *y, w=w)
                mb, ms = orc.branchless_merge_bsr(*x, *y)
                assert np.array_equal(bb_, mb) and np.array_equal(bs_, ms), (w, n)


@pytest.mark.parametrize("seed", range(4))
def test_svs_generic_properties(orc, seed):
    """SetCollection (testlib/mod.rs:169-212) + prop_intersection_correct."""
    rng = np.random.default_rng(200 + seed)
    for k in range(2, 7):
        mutual = rand_set(rng, int(rng.integers(0, 50)), 5000)
        sets = [np.union1d(rand_set(rng, int(rng.integers(0, 400)), 5000), mutual).astype(np.uint32)
                for _ in range(k)]
        res = orc.svs_generic(sets)
        assert props_intersection_correct(res, sets)
        assert np.array_equal(orc.svs_generic(sorted(sets, key=len)), res)


def test_run_pairs_threads(orc):
    rng = np.random.default_rng(9)
    pairs = [pair_with_overlap(rng, int(rng.integers(1, 500)), int(rng.integers(1, 500)), 0)
             for _ in range(40)]
    want = np.array([orc.naive_merge_count(a, b) for a, b in pairs], np.uint64)
    for algo in (orc.NAIVE_MERGE, orc.SHUFFLING_W8, orc.SIMD_GALLOPING_W16, orc.BMISS_W4,
                 orc.GALLOPING):
        for nt in (1, 4):
            assert np.array_equal(orc.run_pairs(algo, pairs, nt), want)
    groups = [[rand_set(rng, 300, 2000) for _ in range(3)] for _ in range(10)]
    wantk = np.array([orc.svs_generic(g).size for g in groups], np.uint64)
    assert np.array_equal(orc.run_svs_groups(groups, 3), wantk)


def test_svs_with_each_baseline_equals_svs_generic(orc):
    """svs_generic run with each timed CPU baseline as its 2-set function
    gives svs_generic's (naive_merge) result."""
    rng = np.random.default_rng(33)
    core = np.sort(rng.choice(1 << 20, 300, replace=False)).astype(np.uint32)
    groups = []
    for k in (2, 3, 5):
        g = []
        for i in range(k):
            extra = rng.choice(1 << 20, 4000 // (i + 1), replace=False).astype(np.uint32)
            g.append(np.unique(np.concatenate([core, extra])))
        groups.append(sorted(g, key=len))
    want = [orc.svs_generic(g) for g in groups]
    for algo in (orc.SHUFFLING_W8, orc.SIMD_GALLOPING_W16, orc.BMISS_W4, orc.BRANCHLESS_MERGE):
        outs = [np.empty(min(s.size for s in g), np.uint32) for g in groups]
        counts = orc.run_svs_groups(groups, 2, outs=outs, algo=algo)
        for w, o, c in zip(want, outs, counts):
            assert np.array_equal(o[:int(c)], w), orc.ALGO_NAMES[algo]


def test_bsr_pair_runner_equals_single_calls(orc):
    rng = np.random.default_rng(44)
    pairs, want = [], []
    for n in (0, 1, 50, 3000):
        a = np.unique(rng.integers(0, 1 << 14, n)).astype(np.uint32)
        b = np.unique(rng.integers(0, 1 << 14, 2 * n + 1)).astype(np.uint32)
        ba, sa = orc.bsr_from_sorted(a)
        bb, sb = orc.bsr_from_sorted(b)
        pairs.append((ba, sa, bb, sb))
        want.append(orc.branchless_merge_bsr(ba, sa, bb, sb))
    for algo in (0, 1):
        outs = [(np.empty(max(p[0].size, 1), np.uint32), np.empty(max(p[0].size, 1), np.uint32))
                for p in pairs]
        words = orc.run_bsr_pairs(pairs, 3, outs=outs, algo=algo)
        for (wb, ws), (ob, os_), w in zip(want, outs, words):
            assert np.array_equal(ob[:int(w)], wb) and np.array_equal(os_[:int(w)], ws)


def test_small_adaptive_equals_svs_generic(orc):
    """small_adaptive and svs_generic give the same k-set intersection (the
    reference's property tests hold every k-set algorithm to one answer)."""
    rng = np.random.default_rng(55)
    for k in (2, 3, 5, 8):
        core = rng.choice(1 << 18, 200, replace=False).astype(np.uint32)
        sets = []
        for i in range(k):
            extra = rng.choice(1 << 18, 20000 // (i + 1), replace=False).astype(np.uint32)
            sets.append(np.unique(np.concatenate([core, extra])))
        sets.sort(key=len)
        assert np.array_equal(orc.small_adaptive(sets), orc.svs_generic(sets)), k
    # edges: an empty set, disjoint sets, identical sets, values near 2^32
    e = np.empty(0, np.uint32)
    x = np.array([1, 5, 0xFFFFFFFF], np.uint32)
    assert orc.small_adaptive([e, x]).size == 0
    assert orc.small_adaptive([x, e, x]).size == 0
    assert orc.small_adaptive([x, np.array([2, 6], np.uint32)]).size == 0
    assert np.array_equal(orc.small_adaptive([x, x.copy(), x.copy()]), x)
