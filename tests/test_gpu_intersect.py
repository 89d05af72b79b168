"""GPU 2-set intersection vs the oracle (naive_merge), bit-exact: same
elements, same ascending order, same count.  Every kernel variant of both
algorithms is exercised, through host and device pointers."""
from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import GOLDEN, pair_with_overlap, rand_set

pytestmark = pytest.mark.gpu

so = pytest.importorskip("simd_set_operations_gb300")
from simd_set_operations_gb300 import datasets as ds  # noqa: E402


def all_algos():
    algos = [so.ALGO_AUTO]
    algos += [so.ALGO_MERGE | so.VARIANT(v) for v in range(so.num_variants(so.ALGO_MERGE))]
    algos += [so.ALGO_GALLOP | so.VARIANT(v) for v in range(so.num_variants(so.ALGO_GALLOP))]
    algos += [so.ALGO_BITMAP | so.VARIANT(v) for v in range(so.num_variants(so.ALGO_BITMAP))]
    return algos


def check_pair(ctx, orc, a, b, algos=None):
    want = orc.naive_merge(a, b)
    for algo in (algos or all_algos()):
        out, n = so.intersect(a, b, algo=algo, ctx=ctx)
        assert np.array_equal(out[:n], want), (hex(algo), a.size, b.size)
        assert so.intersect_count(a, b, algo=algo, ctx=ctx) == want.size, hex(algo)
    return want


def test_unit_test_kats(ctx, orc):
    kat = json.loads((GOLDEN / "unit_tests.json").read_text())
    for case in kat["twoset"]:
        a = np.array(case["a"], np.uint32)
        b = np.array(case["b"], np.uint32)
        for algo in all_algos():
            out, n = so.intersect(a, b, algo=algo, ctx=ctx)
            assert out[:n].tolist() == case["expected"], (case["name"], hex(algo))
    g = kat["galloping"]
    large = np.arange(*g["large_range"], dtype=np.uint32)
    for algo in all_algos():
        out, n = so.intersect(np.array(g["small"], np.uint32), large, algo=algo, ctx=ctx)
        assert out[:n].tolist() == g["expected"]


def test_reference_kernel_fixtures(ctx, orc):
    z = np.load(GOLDEN / "ref_kernels.npz")
    for i in range(len(z["kinds"])):
        a, b = z[f"a{i}"], z[f"b{i}"]
        for algo in all_algos():
            out, n = so.intersect(a, b, algo=algo, ctx=ctx)
            assert np.array_equal(out[:n], z[f"bmiss{i}"]), (i, hex(algo))


def test_edge_cases(ctx, orc):
    E = np.empty(0, np.uint32)
    one = np.array([7], np.uint32)
    rng = np.random.default_rng(1)
    big = rand_set(rng, 5000)
    cases = [(E, E), (E, big), (big, E), (one, one), (one, big), (big, big),
             (np.arange(0, 20000, 2, dtype=np.uint32), np.arange(1, 20000, 2, dtype=np.uint32)),
             (np.array([0, 2**31 - 1, 2**31, 2**32 - 2, 2**32 - 1], np.uint32),
              np.array([0, 2**31, 2**32 - 1], np.uint32)),
             (np.arange(2**32 - 3000, 2**32, dtype=np.uint64).astype(np.uint32),
              np.arange(2**32 - 6000, 2**32, 3, dtype=np.uint64).astype(np.uint32))]
    for a, b in cases:
        check_pair(ctx, orc, a, b)


@pytest.mark.parametrize("n", [1, 3, 4, 5, 15, 16, 17, 255, 256, 257, 1023, 1024, 1025,
                               2047, 2048, 2049, 4095, 4097, 6143, 8193, 16385])
def test_tile_boundaries(ctx, orc, n):
    """Sizes around tile (NV = 1024, 2048), ring and 16-byte chunk edges;
    identical sets put a match on every boundary."""
    a = np.arange(n, dtype=np.uint32) * 3
    check_pair(ctx, orc, a, a)
    b = np.arange(n + 1, dtype=np.uint32) * 3 + 1
    check_pair(ctx, orc, a, b[: max(n - 1, 0)])


@pytest.mark.parametrize("seed", range(8))
def test_random_pairs(ctx, orc, seed):
    rng = np.random.default_rng(1000 + seed)
    for _ in range(6):
        na = int(rng.integers(0, 200_000))
        nb = int(rng.integers(0, 200_000))
        sh = int(rng.integers(0, min(na, nb) + 1))
        hi = int(rng.choice([max(na + nb, 1) * 2, 1 << 32]))
        a, b = pair_with_overlap(rng, na, nb, sh, hi)
        check_pair(ctx, orc, a, b)


@pytest.mark.parametrize("ratio", [2, 16, 64, 256, 1024, 16384])
def test_skewed_pairs(ctx, orc, ratio):
    rng = np.random.default_rng(ratio)
    nl = 1 << 20
    ns = max(nl // ratio, 1)
    s, l = ds.gen_twoset(ratio, 0.05, 0.1, ns, nl)
    check_pair(ctx, orc, s, l)
    check_pair(ctx, orc, l, s)


def test_device_pointers_and_misalignment(ctx, orc):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    a, b = pair_with_overlap(rng, 100_003, 77_777, 20_000)
    want = orc.naive_merge(a, b)
    for off_a in range(4):
        for off_b in range(4):
            ta = torch.zeros(a.size + 4, dtype=torch.int32, device="cuda")
            tb = torch.zeros(b.size + 4, dtype=torch.int32, device="cuda")
            ta[off_a:off_a + a.size] = torch.from_numpy(a.view(np.int32))
            tb[off_b:off_b + b.size] = torch.from_numpy(b.view(np.int32))
            va, vb = ta[off_a:off_a + a.size], tb[off_b:off_b + b.size]
            for algo in (so.ALGO_MERGE, so.ALGO_GALLOP, so.ALGO_MERGE | so.VARIANT(2),
                         so.ALGO_BITMAP, so.ALGO_BITMAP | so.VARIANT(1)):
                out, n = so.intersect(va, vb, algo=algo, ctx=ctx)
                got = out[:n].cpu().numpy().view(np.uint32)
                assert np.array_equal(got, want), (off_a, off_b, hex(algo))
                assert so.intersect_count(va, vb, algo=algo, ctx=ctx) == want.size


def test_async_and_capacity(ctx, orc):
    torch = pytest.importorskip("torch")
    import ctypes as C
    from simd_set_operations_gb300 import _lib
    rng = np.random.default_rng(4)
    a, b = pair_with_overlap(rng, 50_000, 60_000, 1234)
    ta = torch.from_numpy(a.view(np.int32)).cuda()
    tb = torch.from_numpy(b.view(np.int32)).cuda()
    out = torch.empty(50_000, dtype=torch.int32, device="cuda")
    ln = torch.zeros(2, dtype=torch.int64, device="cuda")
    rc = _lib.lib.setops_gpu_intersect_async(ctx.handle, ta.data_ptr(), a.size, tb.data_ptr(),
                                             b.size, out.data_ptr(), 50_000, ln.data_ptr(), 0)
    assert rc == 0
    rc = _lib.lib.setops_gpu_intersect_async(ctx.handle, ta.data_ptr(), a.size, tb.data_ptr(),
                                             b.size, None, 0, ln.data_ptr() + 8, 0)
    assert rc == 0
    ctx.synchronize()
    assert int(ln[0]) == 1234 and int(ln[1]) == 1234
    assert np.array_equal(out[:1234].cpu().numpy().view(np.uint32), orc.naive_merge(a, b))
    small = np.empty(10, np.uint32)
    n = C.c_size_t()
    rc = _lib.lib.setops_gpu_intersect(ctx.handle, a.ctypes.data, a.size, b.ctypes.data, b.size,
                                       small.ctypes.data, 10, C.byref(n), _lib.HOST)
    assert rc == _lib.ERR_CAPACITY
    # the context is still usable after an error
    assert so.intersect_count(a, b, ctx=ctx) == 1234


def test_many_launches_epoch_wrap(ctx, orc):
    """More than 2^16 launches on one context: look-back tags wrap."""
    torch = pytest.importorskip("torch")
    from simd_set_operations_gb300 import _lib
    a = np.arange(0, 6000, 3, dtype=np.uint32)
    b = np.arange(0, 6000, 2, dtype=np.uint32)
    want = orc.naive_merge(a, b)
    ta = torch.from_numpy(a.view(np.int32)).cuda()
    tb = torch.from_numpy(b.view(np.int32)).cuda()
    out = torch.empty(a.size, dtype=torch.int32, device="cuda")
    ln = torch.zeros(1, dtype=torch.int64, device="cuda")
    for i in range(66_000):
        algo = so.ALGO_MERGE if i % 2 else so.ALGO_GALLOP
        rc = _lib.lib.setops_gpu_intersect_async(ctx.handle, ta.data_ptr(), a.size,
                                                 tb.data_ptr(), b.size, out.data_ptr(), a.size,
                                                 ln.data_ptr(), algo)
        assert rc == 0
    ctx.synchronize()
    assert int(ln[0]) == want.size
    assert np.array_equal(out[:want.size].cpu().numpy().view(np.uint32), want)


def test_full_size_skewed_sweep(ctx, orc):
    """The 2^24-element sweep: |large| = 2^24, |small| in {2^10, 2^14, 2^18,
    2^24}, density 0.05, selectivity 0.01; exact vs naive_merge."""
    for k, e in enumerate((10, 14, 18, 24)):
        s, l = ds.gen_twoset(100 + k, 0.05, 0.01, 1 << e, 1 << 24)
        want = orc.naive_merge(s, l)
        assert want.size == int(0.01 * (1 << e))
        for algo in (so.ALGO_AUTO, so.ALGO_MERGE, so.ALGO_GALLOP):
            out, n = so.intersect(s, l, algo=algo, ctx=ctx)
            assert np.array_equal(out[:n], want), (e, hex(algo))


def test_validate_sorted(ctx):
    assert so.validate_sorted(np.arange(100000, dtype=np.uint32), ctx=ctx)
    x = np.arange(100000, dtype=np.uint32)
    x[77777] = x[77776]
    assert not so.validate_sorted(x, ctx=ctx)
    assert so.validate_sorted(np.empty(0, np.uint32), ctx=ctx)


def test_visitor_api(ctx, orc):
    rng = np.random.default_rng(8)
    a, b = pair_with_overlap(rng, 3000, 4000, 500)
    want = orc.naive_merge(a, b)
    assert np.array_equal(so.run_2set(a, b, so.gpu_auto), want)
    assert np.array_equal(so.run_2set(a, b, so.gpu_merge), want)
    assert np.array_equal(so.run_2set(a, b, so.gpu_galloping), want)
    assert np.array_equal(so.run_2set_c(a, b, so.gpu_auto_c), want)
    c = so.Counter()
    so.gpu_auto(a, b, c)
    assert c.count() == want.size
    w = so.UnsafeWriter.with_capacity(min(a.size, b.size))
    so.gpu_auto(a, b, w)
    assert np.array_equal(w.into(), want)


def test_default_policy_bands(ctx, orc):
    """The default policy per floor(log2(max/min)) band: arrays take the
    window kernel with staged inputs (8) below ratio 2, its coarse-bitmap
    variant (7) for 2-31, then
    the search kernel (sampled, 8-lane, warp per element); BSR pairs take the
    block-broadcast variant of the merge family (3) below 32.  Each band's
    choice gives the oracle's result on a pair of that ratio."""
    def algo_var(flags):
        return flags & 0xFF00, (flags >> 16) & 0xFF  # (algorithm bits, variant)
    want_arr = {0: (so.ALGO_BITMAP, 8), 1: (so.ALGO_BITMAP, 7), 4: (so.ALGO_BITMAP, 7),
                5: (so.ALGO_GALLOP, 0), 8: (so.ALGO_GALLOP, 0), 9: (so.ALGO_GALLOP, 3),
                12: (so.ALGO_GALLOP, 3), 13: (so.ALGO_GALLOP, 2), 20: (so.ALGO_GALLOP, 2)}
    for band, (algo, var) in want_arr.items():
        got = algo_var(ctx.get_policy(False, band))
        assert got == (algo, var), (band, got)
    for band in (0, 4):
        assert algo_var(ctx.get_policy(True, band)) == (so.ALGO_MERGE, 3)
    # ratios 32-511 with a smaller set of 2^16 to 2^22 elements: the sampled
    # search with 512-element tiles (variant 8)
    for band in (5, 8):
        assert algo_var(ctx.get_policy_class(False, band, 2)) == (so.ALGO_GALLOP, 8)
    rng = np.random.default_rng(21)
    for ratio in (1, 2, 3, 5, 16, 31, 32, 600, 9000):
        na = 2000 if ratio < 600 else 200
        a, b = pair_with_overlap(rng, na, na * ratio, na // 5, 1 << 32)
        want = orc.naive_merge(a, b)
        out, n = so.intersect(a, b, ctx=ctx)
        assert np.array_equal(out[:n], want), ratio


def test_config0_plain_pair(ctx, orc):
    """The plain 2-set configuration at its exact shape: |A| = |B| = 2^20,
    element space 2^20 / 0.1, selectivity 0.1 (the reference's gen_twoset,
    benchmark/src/generators.rs:30-68).  Count and materialised output of the
    default policy and of every merge and bitmap variant, through host and
    device pointers, equal naive_merge (setops/src/intersect/merge.rs:7-33)."""
    import torch
    a, b = ds.gen_twoset(20240620, 0.1, 0.1, 1 << 20, 1 << 20)
    want = orc.naive_merge(a, b)
    assert want.size == int(0.1 * (1 << 20))
    algos = [so.ALGO_AUTO]
    algos += [so.ALGO_MERGE | so.VARIANT(v) for v in range(so.num_variants(so.ALGO_MERGE))]
    algos += [so.ALGO_BITMAP | so.VARIANT(v) for v in range(so.num_variants(so.ALGO_BITMAP))]
    check_pair(ctx, orc, a, b, algos)
    ta = torch.from_numpy(a.view(np.int32)).cuda()
    tb = torch.from_numpy(b.view(np.int32)).cuda()
    for algo in algos:
        out, n = so.intersect(ta, tb, algo=algo, ctx=ctx)
        got = out[:n].cpu().numpy().view(np.uint32)
        assert np.array_equal(got, want), hex(algo)
        out, n = so.intersect(tb, ta, algo=algo, ctx=ctx)  # operands swapped
        assert np.array_equal(out[:n].cpu().numpy().view(np.uint32), want), hex(algo)


def _pinned(x: np.ndarray) -> np.ndarray:
    import torch
    t = torch.empty(max(x.size, 1), dtype=torch.int32).pin_memory()
    v = t.numpy().view(np.uint32)[:x.size]
    v[:] = x
    return v  # (the view's base holds the pinned tensor)


def test_intersect_pairs_host(ctx, orc):
    """One setops_gpu_intersect_pairs call over mixed host pairs -- search-band
    pairs with pinned inputs and outputs (read in place on the second stream),
    balanced pairs (copied; more than three, so copy slots are reused), pairs
    with pageable inputs or outputs, empty pairs, operands swapped -- gives
    every pair exactly naive_merge; so does a second call on the same context
    with other sizes, and a call whose pairs are all of one kind."""
    rng = np.random.default_rng(41)
    shapes = [(1 << 10, 1 << 22, 10, "pp"), (200_000, 190_000, 2_000, "pp"),
              (1 << 14, 1 << 22, 160, "pp"), (0, 1000, 0, "pp"), (70_000, 210_000, 700, "pp"),
              (1 << 18, 1 << 22, 2_600, "pp"), (3000, 3000, 300, "ph"), (150_000, 150_000, 0, "pp"),
              (1 << 12, 1 << 20, 40, "hp"), (5, 3, 1, "pp"), (1 << 20, 1 << 16, 600, "pp"),
              (40_000, 45_000, 4_000, "pp")]
    pairs, outs, wants = [], [], []
    for na, nb, shared, kind in shapes:
        a, b = pair_with_overlap(rng, na, nb, shared)
        wants.append(orc.naive_merge(a, b))
        pin_in, pin_out = kind[0] == "p", kind[1] == "p"
        pairs.append((_pinned(a), _pinned(b)) if pin_in else (a, b))
        cap = max(min(na, nb), 1)
        outs.append(_pinned(np.zeros(cap, np.uint32)) if pin_out else np.zeros(cap, np.uint32))
    for rep in range(2):
        res = so.intersect_pairs(pairs, outs, ctx=ctx)
        for i, ((got, n), want) in enumerate(zip(res, wants)):
            assert n == want.size and np.array_equal(got[:n], want), (rep, i, shapes[i])
        pairs = [(y, x) for x, y in pairs]  # swapped operands, same results
    # only search-band pairs, then only balanced ones
    for sel in ([0, 2, 5, 8], [1, 4, 7, 11]):
        res = so.intersect_pairs([pairs[i] for i in sel], [outs[i] for i in sel], ctx=ctx)
        for (got, n), i in zip(res, sel):
            assert np.array_equal(got[:n], wants[i]), i
    with pytest.raises(so.SetopsError):
        so.intersect_pairs([pairs[1]], [np.zeros(1, np.uint32)], ctx=ctx)  # capacity


def test_pinned_host_inputs_read_in_place(ctx, orc):
    """Host-pointer calls on pinned host memory: the kernels read the inputs
    in place (and write the result straight into a pinned output) where the
    chosen kernel allows it, else copy them first.  Every shape, count and
    materialised, pinned or pageable output, equals naive_merge."""
    rng = np.random.default_rng(31)
    shapes = [(200_000, 200_000, 2_000), (70_000, 210_000, 700), (1_000, 1 << 18, 10),
              (1 << 14, 1 << 22, 160), (1 << 18, 1 << 22, 2_600), (5, 3, 1)]
    for na, nb, shared in shapes:
        a, b = pair_with_overlap(rng, na, nb, shared)
        want = orc.naive_merge(a, b)
        pa, pb = _pinned(a), _pinned(b)
        for algo in (so.ALGO_AUTO, so.ALGO_BITMAP, so.ALGO_GALLOP, so.ALGO_MERGE):
            for pinned_out in (True, False):
                cap = min(na, nb)
                out = _pinned(np.zeros(cap, np.uint32)) if pinned_out else np.zeros(cap, np.uint32)
                got, n = so.intersect(pa, pb, out, algo=algo, ctx=ctx)
                assert np.array_equal(got[:n], want), (na, nb, hex(algo), pinned_out)
            assert so.intersect_count(pa, pb, algo=algo, ctx=ctx) == want.size
