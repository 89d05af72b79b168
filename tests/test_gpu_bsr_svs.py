"""GPU BSR intersection (vs branchless_merge_bsr), device BSR encode/decode
(vs BsrVec::from_sorted / to_sorted_set), and device k-set SvS (vs
svs_generic with naive_merge) -- all bit-exact."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import pair_with_overlap, rand_set

pytestmark = pytest.mark.gpu

so = pytest.importorskip("simd_set_operations_gb300")
from simd_set_operations_gb300 import datasets as ds  # noqa: E402


def bsr_algos():
    algos = [so.ALGO_AUTO]
    algos += [so.ALGO_MERGE | so.VARIANT(v) for v in range(so.num_variants(so.ALGO_MERGE, True))]
    algos += [so.ALGO_GALLOP | so.VARIANT(v) for v in range(so.num_variants(so.ALGO_GALLOP, True))]
    return algos


def check_bsr(ctx, orc, a, b):
    ba, sa = orc.bsr_from_sorted(a)
    bb, sb = orc.bsr_from_sorted(b)
    wb, ws = orc.branchless_merge_bsr(ba, sa, bb, sb)
    wc = orc.branchless_merge_bsr_count(ba, sa, bb, sb)
    assert wc == orc.naive_merge_count(a, b)
    A, B = so.BsrRef(ba, sa), so.BsrRef(bb, sb)
    for algo in bsr_algos():
        v = so.BsrVec()
        so.gpu_bsr(A, B, v, algo=algo, ctx=ctx)
        assert np.array_equal(v.bases, wb) and np.array_equal(v.states, ws), hex(algo)
        c = so.Counter()
        so.gpu_bsr(A, B, c, algo=algo, ctx=ctx)
        assert c.count() == wc, hex(algo)


def test_bsr_edges(ctx, orc):
    E = np.empty(0, np.uint32)
    check_bsr(ctx, orc, E, E)
    check_bsr(ctx, orc, E, np.arange(100, dtype=np.uint32))
    x = np.arange(0, 64, dtype=np.uint32)
    check_bsr(ctx, orc, x, x)
    check_bsr(ctx, orc, np.arange(0, 64, 2, dtype=np.uint32), np.arange(1, 64, 2, dtype=np.uint32))
    hi = np.array([2**32 - 33, 2**32 - 32, 2**32 - 2, 2**32 - 1], np.uint32)
    check_bsr(ctx, orc, hi, hi[1:])


@pytest.mark.parametrize("seed", range(6))
def test_bsr_random(ctx, orc, seed):
    rng = np.random.default_rng(300 + seed)
    for n, dens in [(100, 0.5), (5000, 0.5), (50_000, 0.3), (200_000, 0.05), (30_000, 0.9)]:
        nb = int(n * rng.uniform(0.3, 3))
        hi = max(int(n / dens) * 3, 2 * (n + nb))
        a, b = pair_with_overlap(rng, n, nb, n // 4, hi=hi)
        check_bsr(ctx, orc, a, b)


def _bsr_decode(bases, states):
    """The sorted set whose BSR words these are (BsrVec::to_sorted_set)."""
    bits = np.unpackbits(states.astype('<u4').view(np.uint8).reshape(-1, 4), axis=1,
                         bitorder='little')
    rows, cols = np.nonzero(bits)
    return (bases[rows].astype(np.uint64) * 32 + cols).astype(np.uint32)


@pytest.mark.parametrize("nw", [1, 31, 32, 33, 63, 64, 65, 1023, 1025, 4097, 70_001])
def test_bsr_block_boundaries(ctx, orc, nw):
    """Word counts around the 32-word blocks of the block-broadcast kernel
    (and the merge kernels' chunks); half of the shared bases carry states
    whose AND is zero, so those words are dropped."""
    rng = np.random.default_rng(nw)
    ab = np.arange(nw, dtype=np.uint32) * 2
    ast = rng.integers(1, 2**32, size=nw, dtype=np.uint64).astype(np.uint32)
    nbw = 2 * nw + 5
    bbase = np.arange(nbw, dtype=np.uint32)
    bst = rng.integers(1, 2**32, size=nbw, dtype=np.uint64).astype(np.uint32)
    shared = np.arange(0, 2 * nw, 2)
    zero = shared[rng.random(shared.size) < 0.5]
    bst[zero] = ~ast[zero // 2]
    bst[bst == 0] = 1
    a, b = _bsr_decode(ab, ast), _bsr_decode(bbase, bst)
    check_bsr(ctx, orc, a, b)
    check_bsr(ctx, orc, b, a)


def test_bsr_skewed(ctx, orc):
    rng = np.random.default_rng(11)
    s, l = ds.gen_twoset(11, 0.5, 0.1, 2000, 1 << 20)
    check_bsr(ctx, orc, s, l)


@pytest.mark.parametrize("n,hi", [(0, 10), (1, 10), (31, 32), (1000, 2000), (300_000, 400_000),
                                  (100_000, 1 << 32), (2049, 4096), (70_000, 70_001)])
def test_bsr_encode_decode(ctx, orc, n, hi):
    rng = np.random.default_rng(n)
    s = rand_set(rng, n, hi)
    wb, ws = orc.bsr_from_sorted(s)
    v = so.BsrVec.from_sorted(s, ctx=ctx)
    assert np.array_equal(v.bases, wb) and np.array_equal(v.states, ws)
    assert np.array_equal(v.to_sorted_set(ctx=ctx), s)


def test_run_2set_bsr_property(ctx, orc):
    """property_tests.rs:82-96: decoded BSR intersection == naive_merge."""
    rng = np.random.default_rng(12)
    a, b = pair_with_overlap(rng, 40_000, 50_000, 9000, hi=300_000)
    A = so.BsrVec.from_sorted(a, ctx=ctx)
    B = so.BsrVec.from_sorted(b, ctx=ctx)
    r = so.run_2set_bsr(A.bsr_ref(), B.bsr_ref())
    assert np.array_equal(r.to_sorted_set(ctx=ctx), orc.naive_merge(a, b))


# ---- k-set ----------------------------------------------------------------

def check_svs(ctx, orc, sets):
    want = orc.svs_generic(sorted(sets, key=len))
    assert np.array_equal(orc.svs_generic(sets), want)
    for fn in (so.gpu_auto, so.gpu_merge, so.gpu_galloping):
        assert np.array_equal(so.run_svs(sets, fn), want), fn
    assert np.array_equal(so.run_kset(sets, so.gpu_svs), want)
    c = so.Counter()
    so.gpu_svs(sets, c)
    assert c.count() == want.size
    return want


@pytest.mark.parametrize("k", [2, 3, 4, 5, 8, 12])
def test_svs_random(ctx, orc, k):
    rng = np.random.default_rng(400 + k)
    for trial in range(3):
        mutual = rand_set(rng, int(rng.integers(0, 2000)), 1 << 22)
        sets = [np.union1d(rand_set(rng, int(rng.integers(1, 300_000)), 1 << 22), mutual)
                .astype(np.uint32) for _ in range(k)]
        check_svs(ctx, orc, sets)


def test_svs_edges(ctx, orc):
    E = np.empty(0, np.uint32)
    x = np.arange(1000, dtype=np.uint32)
    check_svs(ctx, orc, [x, x, x])
    check_svs(ctx, orc, [x, E, x])
    check_svs(ctx, orc, [x, x[::2], x[::3], x[::5]])
    check_svs(ctx, orc, [np.arange(0, 10**6, 7, dtype=np.uint32), np.array([7, 14, 999_999], np.uint32)])
    with pytest.raises(so.SetopsError):
        so.run_svs([x])


@pytest.mark.parametrize("k", [3, 5, 8])
def test_svs_config_shape(ctx, orc, k):
    """k-set sets of sizes 2^22 / i, density 0.2, 5% core of the smallest."""
    sets = ds.gen_kset(500 + k, 0.2, 0.05, 1 << 22, 1.0, k)
    want = check_svs(ctx, orc, sets)
    assert want.size >= int(0.05 * sets[0].size)


def test_svs_device_pointers(ctx, orc):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(21)
    sets = [rand_set(rng, n, 1 << 20) for n in (50_000, 120_000, 300_000, 80_000)]
    want = orc.svs_generic(sorted(sets, key=len))
    tsets = [torch.from_numpy(s.view(np.int32)).cuda() for s in sets]
    w = so.VecWriter()
    so.gpu_svs(tsets, w, ctx=ctx)
    assert np.array_equal(w.into(), want)


@pytest.mark.parametrize("k,dens", [(3, 0.001), (6, 0.3), (16, 0.05), (4, 0.9)])
def test_svs_fused_shapes(ctx, orc, k, dens):
    """Sets within 16x of the smallest take the fused k-set kernel: sparse
    tiles (density 0.001), dense ones, the most sets it takes (16)."""
    sets = ds.gen_kset(600 + k, dens, 0.1, 1 << 18, 0.5, k)
    want = check_svs(ctx, orc, sets)
    assert want.size >= int(0.1 * min(s.size for s in sets))


def test_kset_kernel_shapes(ctx, orc):
    """The fused k-set kernel, count and materialise, equals svs_generic: the
    k-set configuration's shape, sparse and dense tiles, the most sets (16),
    identical sets, a set holding only a few far values, and tile edges
    (smallest sets of 4095-4097 elements, its 4096-element tiles)."""
    from simd_set_operations_gb300 import _svs
    flags = so.ALGO_AUTO
    rng = np.random.default_rng(701)
    x = np.arange(50_000, dtype=np.uint32) * 3
    groups = [ds.gen_kset(800 + k, 0.2, 0.05, 1 << 21, 1.0, k) for k in (3, 5, 8)]
    groups += [ds.gen_kset(810 + k, dens, 0.1, 1 << 17, 0.5, k)
               for k, dens in ((3, 0.001), (6, 0.3), (16, 0.05), (4, 0.9))]
    groups += [[x, x, x], [x, x[::2], x[::3], x[1::5]],
               [x, np.array([0, 3, 149_997, 4_000_000_000], np.uint32), x[::7]]]
    for n in (4095, 4096, 4097, 8191, 12_289):
        base = rand_set(rng, n, 1 << 24)
        groups.append([base, np.union1d(base[::2], rand_set(rng, n, 1 << 24)).astype(np.uint32),
                       np.union1d(base[::3], rand_set(rng, 2 * n, 1 << 24)).astype(np.uint32)])
    for sets in groups:
        sets = sorted(sets, key=len)
        want = orc.svs_generic(sets)
        out, n = _svs(sets, algo=flags, ctx=ctx)
        assert np.array_equal(np.asarray(out[:n]), want), [s.size for s in sets]
        assert _svs(sets, count_only=True, algo=flags, ctx=ctx) == want.size


def test_svs_async(ctx, orc):
    """setops_gpu_svs_async: the result (or the count) on the device, no
    synchronisation; the fused path and the step-wise path (a set over 16x
    the smallest)."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    from simd_set_operations_gb300 import _lib
    rng = np.random.default_rng(33)
    for sizes in ((40_000, 90_000, 120_000, 60_000), (10_000, 400_000, 30_000)):
        sets = sorted([rand_set(rng, n, 1 << 21) for n in sizes], key=len)
        want = orc.svs_generic(sets)
        ts = [torch.from_numpy(s.view(np.int32)).cuda() for s in sets]
        ptrs = (C.c_void_p * len(ts))(*[x.data_ptr() for x in ts])
        lens = (C.c_size_t * len(ts))(*[s.size for s in sets])
        out = torch.full((sets[0].size,), -1, dtype=torch.int32, device="cuda")
        dlen = torch.zeros(1, dtype=torch.int64, device="cuda")
        for _ in range(2):
            ctx.check(_lib.lib.setops_gpu_svs_async(ctx.handle, ptrs, lens, len(ts), out.data_ptr(),
                                                    out.numel(), dlen.data_ptr(), 0))
        ctx.check(_lib.lib.setops_gpu_synchronize(ctx.handle))
        n = int(dlen.item())
        assert n == want.size and np.array_equal(out[:n].cpu().numpy().view(np.uint32), want)
        ctx.check(_lib.lib.setops_gpu_svs_async(ctx.handle, ptrs, lens, len(ts), None, 0,
                                                dlen.data_ptr(), 0))
        ctx.check(_lib.lib.setops_gpu_synchronize(ctx.handle))
        assert int(dlen.item()) == want.size
