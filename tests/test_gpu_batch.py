"""Batched pairs (setops_gpu_batch_intersect / _count): every pair of a batch
in one launch must equal naive_merge of that pair (the reference's oracle,
setops/src/intersect/merge.rs:7-33), for every kernel shape and search ratio
of the batch policy, through host and device arrays."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import rand_set

pytestmark = pytest.mark.gpu

import simd_set_operations_gb300 as so  # noqa: E402
from simd_set_operations_gb300 import _lib, datasets as ds  # noqa: E402


def expected(orc, batch):
    pairs = [batch.pair(p) for p in range(len(batch))]
    outs = [np.empty(max(min(a.size, b.size), 1), np.uint32) for a, b in pairs]
    counts = orc.run_pairs(orc.NAIVE_MERGE, pairs, 8, outs=outs)
    return [o[:int(c)] for o, c in zip(outs, counts)]


def check_batch(ctx, orc, batch, want=None):
    want = want or expected(orc, batch)
    out, out_off, lens = so.batch_intersect(batch.pool, batch.a_off, batch.a_len, batch.b_off,
                                            batch.b_len, ctx=ctx)
    for p, w in enumerate(want):
        got = out[int(out_off[p]):int(out_off[p]) + int(lens[p])]
        assert int(lens[p]) == w.size and np.array_equal(got, w), (p, batch.a_len[p], batch.b_len[p])
    counts = so.batch_count(batch.pool, batch.a_off, batch.a_len, batch.b_off, batch.b_len, ctx=ctx)
    assert [int(c) for c in counts] == [w.size for w in want]
    return want


def handmade_batch():
    """Edge cases: empty sides, identical sets, disjoint, one element, values
    near 2^32, a pair longer than one tile, and a strongly skewed pair."""
    rng = np.random.default_rng(7)
    big = rand_set(rng, 20000, 1 << 20)
    sets = [
        (np.empty(0, np.uint32), rand_set(rng, 50, 1000)),
        (rand_set(rng, 50, 1000), np.empty(0, np.uint32)),
        (big, big.copy()),
        (np.arange(0, 1000, 2, dtype=np.uint32), np.arange(1, 1000, 2, dtype=np.uint32)),
        (np.array([5], np.uint32), np.array([5], np.uint32)),
        (np.array([0xFFFFFFFF], np.uint32), np.array([0, 7, 0xFFFFFFFE, 0xFFFFFFFF], np.uint32)),
        (rand_set(rng, 9000, 1 << 16), rand_set(rng, 30000, 1 << 16)),
        (rand_set(rng, 40, 1 << 30), rand_set(rng, 60000, 1 << 30)),
    ]
    pool = np.concatenate([np.concatenate([a, b]) for a, b in sets]).astype(np.uint32)
    a_off, a_len, b_off, b_len = [], [], [], []
    off = 0
    for a, b in sets:
        a_off.append(off); a_len.append(a.size); off += a.size
        b_off.append(off); b_len.append(b.size); off += b.size
    u = lambda x: np.array(x, np.uint64)  # noqa: E731
    return ds.PairBatch(pool, u(a_off), u(a_len), u(b_off), u(b_len))


@pytest.fixture(scope="module")
def generated():
    # the reference shape (log-uniform sizes, density and selectivity drawn
    # per pair), scaled down: 3000 pairs of up to 2^14 elements
    return ds.gen_batch(20240611, 3000, 16, 1 << 14)


def test_batch_generated_every_policy(ctx, orc, generated):
    want = expected(orc, generated)
    v0, r0 = C.c_int(), C.c_uint32()
    ctx.check(_lib.lib.setops_gpu_batch_get_policy(ctx.handle, C.byref(v0), C.byref(r0)))
    try:
        for v in range(_lib.lib.setops_gpu_batch_num_variants()):
            for ratio in (0, 1, 8, 64):  # never / always / sometimes the search path
                ctx.check(_lib.lib.setops_gpu_batch_set_policy(ctx.handle, v, ratio))
                check_batch(ctx, orc, generated, want)
    finally:
        ctx.check(_lib.lib.setops_gpu_batch_set_policy(ctx.handle, v0.value, r0.value))


def test_batch_edge_cases(ctx, orc):
    b = handmade_batch()
    for ratio in (0, 1, 64):
        ctx.check(_lib.lib.setops_gpu_batch_set_policy(ctx.handle, 0, ratio))
        check_batch(ctx, orc, b)
    ctx.check(_lib.lib.setops_gpu_batch_set_policy(ctx.handle, 0, 16))


def test_batch_device_arrays_and_offsets(ctx, orc, generated):
    """Device arrays with the output offsets from the device scan, twice in a
    row; then a capacity error."""
    import torch
    want = expected(orc, generated)
    t = lambda x, dt: torch.from_numpy(np.ascontiguousarray(x).view(dt)).cuda()  # noqa: E731
    pool = t(generated.pool, np.int32)
    arrs = [t(x, np.int64) for x in (generated.a_off, generated.a_len, generated.b_off,
                                     generated.b_len)]
    n = len(generated)
    cap = int(np.minimum(generated.a_len, generated.b_len).sum())
    caps = np.minimum(generated.a_len, generated.b_len)
    offs = np.zeros(n, np.uint64)
    offs[1:] = np.cumsum(caps[:-1])
    for _ in range(2):
        out = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
        lens = torch.zeros(n, dtype=torch.int64, device="cuda")
        ctx.check(_lib.lib.setops_gpu_batch_intersect(
            ctx.handle, pool.data_ptr(), pool.numel(), *[a.data_ptr() for a in arrs], n,
            out.data_ptr(), cap, None, lens.data_ptr(), 0))
        o = out.cpu().numpy().view(np.uint32)
        ln = lens.cpu().numpy()
        for p, w in enumerate(want):
            lo, n_p = int(offs[p]), int(ln[p])
            assert n_p == w.size and np.array_equal(o[lo:lo + n_p], w), p
    rc = _lib.lib.setops_gpu_batch_intersect(
        ctx.handle, pool.data_ptr(), pool.numel(), *[a.data_ptr() for a in arrs], n,
        out.data_ptr(), cap - 1, None, lens.data_ptr(), 0)
    assert rc == _lib.ERR_CAPACITY


def test_batch_autotune_keeps_results_exact(ctx, orc, generated):
    want = expected(orc, generated)
    v0, r0 = C.c_int(), C.c_uint32()
    ctx.check(_lib.lib.setops_gpu_batch_get_policy(ctx.handle, C.byref(v0), C.byref(r0)))
    try:
        v, r = so.batch_autotune(generated.pool, generated.a_off, generated.a_len,
                                 generated.b_off, generated.b_len, reps=1, ctx=ctx)
        assert 0 <= v < _lib.lib.setops_gpu_batch_num_variants()
        check_batch(ctx, orc, generated, want)
    finally:
        ctx.check(_lib.lib.setops_gpu_batch_set_policy(ctx.handle, v0.value, r0.value))


def long_pairs_batch():
    """Pairs whose smaller set spans several units of 16384 elements (split
    over CTAs), at the unit boundary, identical (every element moves when the
    units are packed), skewed, and mixed with small pairs."""
    rng = np.random.default_rng(11)
    same = rand_set(rng, 100000, 1 << 24)
    sets = [
        (rand_set(rng, 200000, 1 << 22), rand_set(rng, 300000, 1 << 22)),
        (same, same.copy()),
        (rand_set(rng, 16384, 1 << 16), rand_set(rng, 40000, 1 << 16)),
        (rand_set(rng, 16385, 1 << 16), rand_set(rng, 40000, 1 << 16)),
        (rand_set(rng, 3, 100), rand_set(rng, 50, 100)),
        (rand_set(rng, 50000, 1 << 28), rand_set(rng, 2000000, 1 << 28)),
        (np.empty(0, np.uint32), rand_set(rng, 70000, 1 << 20)),
        (rand_set(rng, 70000, 1 << 18), rand_set(rng, 65536, 1 << 18)),
    ]
    pool = np.concatenate([np.concatenate([a, b]) for a, b in sets]).astype(np.uint32)
    a_off, a_len, b_off, b_len = [], [], [], []
    off = 0
    for a, b in sets:
        a_off.append(off); a_len.append(a.size); off += a.size
        b_off.append(off); b_len.append(b.size); off += b.size
    u = lambda x: np.array(x, np.uint64)  # noqa: E731
    return ds.PairBatch(pool, u(a_off), u(a_len), u(b_off), u(b_len))


def test_batch_long_pairs_split(ctx, orc):
    """Long pairs split into units give the same results through host arrays
    (exact unit count), device arrays (unit room from the output capacity)
    and a replayed plan, for every search ratio."""
    import torch
    b = long_pairs_batch()
    want = expected(orc, b)
    v0, r0 = C.c_int(), C.c_uint32()
    ctx.check(_lib.lib.setops_gpu_batch_get_policy(ctx.handle, C.byref(v0), C.byref(r0)))
    t = lambda x, dt: torch.from_numpy(np.ascontiguousarray(x).view(dt)).cuda()  # noqa: E731
    pool = t(b.pool, np.int32)
    arrs = [t(x, np.int64) for x in (b.a_off, b.a_len, b.b_off, b.b_len)]
    n = len(b)
    caps = np.minimum(b.a_len, b.b_len)
    cap = int(caps.sum())
    offs = np.zeros(n, np.uint64)
    offs[1:] = np.cumsum(caps[:-1])

    def check_dev(out, lens):
        o, ln = out.cpu().numpy().view(np.uint32), lens.cpu().numpy()
        for p, w in enumerate(want):
            lo, m = int(offs[p]), int(ln[p])
            assert m == w.size and np.array_equal(o[lo:lo + m], w), p

    try:
        for v in range(_lib.lib.setops_gpu_batch_num_variants()):
            for ratio in (0, 1, 16):
                ctx.check(_lib.lib.setops_gpu_batch_set_policy(ctx.handle, v, ratio))
                check_batch(ctx, orc, b, want)
                out = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
                lens = torch.zeros(n, dtype=torch.int64, device="cuda")
                ctx.check(_lib.lib.setops_gpu_batch_intersect(
                    ctx.handle, pool.data_ptr(), pool.numel(), *[a.data_ptr() for a in arrs], n,
                    out.data_ptr(), cap, None, lens.data_ptr(), 0))
                check_dev(out, lens)
        ctx.check(_lib.lib.setops_gpu_batch_set_policy(ctx.handle, v0.value, 16))
        out = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
        lens = torch.zeros(n, dtype=torch.int64, device="cuda")
        plan = C.c_void_p()
        ctx.check(_lib.lib.setops_gpu_batch_plan_create(
            ctx.handle, pool.data_ptr(), pool.numel(), *[a.data_ptr() for a in arrs], n,
            out.data_ptr(), cap, None, lens.data_ptr(), C.byref(plan)))
        try:
            for _ in range(3):
                out.fill_(-1)
                lens.zero_()
                ctx.check(_lib.lib.setops_gpu_batch_plan_launch(plan))
                ctx.check(_lib.lib.setops_gpu_synchronize(ctx.handle))
                check_dev(out, lens)
        finally:
            ctx.check(_lib.lib.setops_gpu_batch_plan_destroy(plan))
        counts = torch.zeros(n, dtype=torch.int64, device="cuda")
        ctx.check(_lib.lib.setops_gpu_batch_plan_create(
            ctx.handle, pool.data_ptr(), pool.numel(), *[a.data_ptr() for a in arrs], n,
            None, 0, None, counts.data_ptr(), C.byref(plan)))
        try:
            for _ in range(2):
                ctx.check(_lib.lib.setops_gpu_batch_plan_launch(plan))
                ctx.check(_lib.lib.setops_gpu_synchronize(ctx.handle))
                assert [int(c) for c in counts.cpu().numpy()] == [w.size for w in want]
        finally:
            ctx.check(_lib.lib.setops_gpu_batch_plan_destroy(plan))
    finally:
        ctx.check(_lib.lib.setops_gpu_batch_set_policy(ctx.handle, v0.value, r0.value))


# ---- BSR pairs ---------------------------------------------------------------

def expected_bsr(orc, bb):
    want = []
    for p in range(len(bb)):
        ba, sa, bb_, sb = bb.pair(p)
        want.append(orc.branchless_merge_bsr(ba, sa, bb_, sb))
    return want


def check_bsr_batch(ctx, orc, bb):
    """Every pair of a BSR batch equals branchless_merge_bsr of that pair
    (setops/src/intersect/merge.rs:62-87), materialised and counted."""
    want = expected_bsr(orc, bb)
    ob, os_, off, lens = so.batch_intersect_bsr(bb.bases, bb.states, bb.a_off, bb.a_len,
                                                bb.b_off, bb.b_len, ctx=ctx)
    for p, (wb, ws) in enumerate(want):
        lo, n = int(off[p]), int(lens[p])
        assert n == wb.size, (p, n, wb.size)
        assert np.array_equal(ob[lo:lo + n], wb) and np.array_equal(os_[lo:lo + n], ws), p
    counts = so.batch_count_bsr(bb.bases, bb.states, bb.a_off, bb.a_len, bb.b_off, bb.b_len,
                                ctx=ctx)
    assert [int(c) for c in counts] == [int(np.unpackbits(ws.view(np.uint8)).sum())
                                        for _, ws in want]


def test_batch_bsr_dense_subset(ctx, orc):
    # the reference's BSR subset shape (density 0.5), scaled down; sets up to
    # 2^16 elements, so some longer sets exceed the shared-memory stage
    b = ds.gen_batch(20240614, 400, 16, 1 << 16, density=(0.5, 0.5))
    check_bsr_batch(ctx, orc, ds.bsr_encode_batch(b))


def test_batch_bsr_mixed_density_and_edges(ctx, orc):
    # edge cases (empty sides, identical, disjoint, values near 2^32, long
    # and skewed pairs), then mixed densities
    check_bsr_batch(ctx, orc, ds.bsr_encode_batch(handmade_batch()))
    b = ds.gen_batch(20240615, 300, 1, 1 << 12, density=(0.01, 0.9))
    check_bsr_batch(ctx, orc, ds.bsr_encode_batch(b))


def test_batch_bsr_device_arrays_and_capacity(ctx, orc):
    import torch
    bb = ds.bsr_encode_batch(ds.gen_batch(20240616, 500, 16, 1 << 13, density=(0.5, 0.5)))
    want = expected_bsr(orc, bb)
    t = lambda x, dt: torch.from_numpy(np.ascontiguousarray(x).view(dt)).cuda()  # noqa: E731
    bases, states = t(bb.bases, np.int32), t(bb.states, np.int32)
    arrs = [t(x, np.int64) for x in (bb.a_off, bb.a_len, bb.b_off, bb.b_len)]
    n = len(bb)
    caps = np.minimum(bb.a_len, bb.b_len)
    cap = int(caps.sum())
    offs = np.zeros(n, np.uint64)
    offs[1:] = np.cumsum(caps[:-1])
    ob = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
    os_ = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
    lens = torch.zeros(n, dtype=torch.int64, device="cuda")
    ctx.check(_lib.lib.setops_gpu_batch_intersect_bsr(
        ctx.handle, bases.data_ptr(), states.data_ptr(), bases.numel(),
        *[a.data_ptr() for a in arrs], n, ob.data_ptr(), os_.data_ptr(), cap, None,
        lens.data_ptr(), 0))
    hb, hs, hl = (ob.cpu().numpy().view(np.uint32), os_.cpu().numpy().view(np.uint32),
                  lens.cpu().numpy())
    for p, (wb, ws) in enumerate(want):
        lo, m = int(offs[p]), int(hl[p])
        assert m == wb.size and np.array_equal(hb[lo:lo + m], wb) and np.array_equal(hs[lo:lo + m], ws), p
    rc = _lib.lib.setops_gpu_batch_intersect_bsr(
        ctx.handle, bases.data_ptr(), states.data_ptr(), bases.numel(),
        *[a.data_ptr() for a in arrs], n, ob.data_ptr(), os_.data_ptr(), cap - 1, None,
        lens.data_ptr(), 0)
    assert rc == _lib.ERR_CAPACITY


# ---- steady-state replay (CUDA graph) ---------------------------------------

def test_batch_plan_replays(ctx, orc, generated):
    """A plan captured once replays the batch exactly, again after its inputs
    were rewritten in place, in count form too; an overflowing output is
    reported by the next synchronising call."""
    import torch
    want = expected(orc, generated)
    t = lambda x, dt: torch.from_numpy(np.ascontiguousarray(x).view(dt)).cuda()  # noqa: E731
    pool = t(generated.pool, np.int32)
    arrs = [t(x, np.int64) for x in (generated.a_off, generated.a_len, generated.b_off,
                                     generated.b_len)]
    n = len(generated)
    caps = np.minimum(generated.a_len, generated.b_len)
    cap = int(caps.sum())
    offs = np.zeros(n, np.uint64)
    offs[1:] = np.cumsum(caps[:-1])
    out = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
    lens = torch.zeros(n, dtype=torch.int64, device="cuda")
    plan = C.c_void_p()
    ctx.check(_lib.lib.setops_gpu_batch_plan_create(
        ctx.handle, pool.data_ptr(), pool.numel(), *[a.data_ptr() for a in arrs], n,
        out.data_ptr(), cap, None, lens.data_ptr(), C.byref(plan)))
    try:
        def check(shift):
            ctx.check(_lib.lib.setops_gpu_synchronize(ctx.handle))
            o, ln = out.cpu().numpy().view(np.uint32), lens.cpu().numpy()
            for p, w in enumerate(want):
                lo, m = int(offs[p]), int(ln[p])
                assert m == w.size and np.array_equal(o[lo:lo + m], w + np.uint32(shift)), p
        for _ in range(3):
            out.fill_(-1)
            lens.zero_()
            ctx.check(_lib.lib.setops_gpu_batch_plan_launch(plan))
            check(0)
        # new contents, same shape: every value + 1000 (order and matches keep)
        pool.add_(1000)
        ctx.check(_lib.lib.setops_gpu_batch_plan_launch(plan))
        check(1000)
        pool.sub_(1000)
    finally:
        ctx.check(_lib.lib.setops_gpu_batch_plan_destroy(plan))
    # count form
    counts = torch.zeros(n, dtype=torch.int64, device="cuda")
    ctx.check(_lib.lib.setops_gpu_batch_plan_create(
        ctx.handle, pool.data_ptr(), pool.numel(), *[a.data_ptr() for a in arrs], n,
        None, 0, None, counts.data_ptr(), C.byref(plan)))
    ctx.check(_lib.lib.setops_gpu_batch_plan_launch(plan))
    ctx.check(_lib.lib.setops_gpu_synchronize(ctx.handle))
    ctx.check(_lib.lib.setops_gpu_batch_plan_destroy(plan))
    assert [int(c) for c in counts.cpu().numpy()] == [w.size for w in want]
    # capacity checked on the device
    ctx.check(_lib.lib.setops_gpu_batch_plan_create(
        ctx.handle, pool.data_ptr(), pool.numel(), *[a.data_ptr() for a in arrs], n,
        out.data_ptr(), cap - 1, None, lens.data_ptr(), C.byref(plan)))
    ctx.check(_lib.lib.setops_gpu_batch_plan_launch(plan))
    assert _lib.lib.setops_gpu_synchronize(ctx.handle) == _lib.ERR_CAPACITY
    ctx.check(_lib.lib.setops_gpu_batch_plan_destroy(plan))


def test_batch_full_size_range_autotuned(ctx, orc):
    """The batched configuration's full size range: 20,000 pairs with set
    sizes log-uniform in [2^4, 2^16], density U[0.01, 0.5], selectivity
    U[0, 0.5]; the policy autotuned on the batch, then every pair of one
    launch equal to naive_merge of that pair, and the counts too."""
    batch = ds.gen_batch(20240621, 20000, 16, 1 << 16)
    assert int(max(batch.a_len.max(), batch.b_len.max())) > 1 << 15
    want = expected(orc, batch)
    v0, r0 = C.c_int(), C.c_uint32()
    ctx.check(_lib.lib.setops_gpu_batch_get_policy(ctx.handle, C.byref(v0), C.byref(r0)))
    try:
        so.batch_autotune(batch.pool, batch.a_off, batch.a_len, batch.b_off, batch.b_len,
                          reps=1, ctx=ctx)
        check_batch(ctx, orc, batch, want)
    finally:
        ctx.check(_lib.lib.setops_gpu_batch_set_policy(ctx.handle, v0.value, r0.value))
