"""k-set small_adaptive on the GPU (setops_gpu_adaptive / _count): the same
elements in the same order as svs_generic (setops/src/intersect/svs.rs:50-73)
and as the oracle's small_adaptive (setops/src/intersect/adaptive.rs:107-148),
for random groups, the k-set configuration's shape, served-query shapes
(a short list against long ones), edge cases, host and device arrays."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rand_set

pytestmark = pytest.mark.gpu

import simd_set_operations_gb300 as so  # noqa: E402
from simd_set_operations_gb300 import datasets as ds  # noqa: E402


def group(rng, k, n0, grow, core, hi):
    c = rand_set(rng, core, hi)
    sets = []
    for i in range(k):
        extra = rand_set(rng, min(int(n0 * grow ** i), hi // 2), hi)
        sets.append(np.union1d(c, extra).astype(np.uint32))
    return sets


def check(ctx, orc, sets):
    want = orc.svs_generic(sorted(sets, key=len))
    assert np.array_equal(orc.small_adaptive(sorted(sets, key=len)), want)
    w = so.VecWriter()
    so.gpu_small_adaptive(sets, w, ctx=ctx)
    assert np.array_equal(w.into(), want), [s.size for s in sets]
    c = so.Counter()
    so.gpu_small_adaptive(sets, c, ctx=ctx)
    assert c.count() == want.size
    return want


@pytest.mark.parametrize("k", [2, 3, 5, 8, 16])
def test_adaptive_random(ctx, orc, k):
    rng = np.random.default_rng(100 + k)
    for n0, grow, core, hi in ((50, 1.5, 10, 1 << 12), (3000, 2.0, 300, 1 << 22),
                               (200_000, 1.3, 5_000, 1 << 26)):
        if k == 16 and n0 > 3000:
            continue
        check(ctx, orc, group(rng, k, n0, grow, core, hi))


@pytest.mark.parametrize("k", [3, 5, 8])
def test_adaptive_kset_config_shape(ctx, orc, k):
    """The k-set configuration's shape, scaled down: |S_i| = 2^18 / i,
    density 0.2, a core of 5 % of the smallest set."""
    sets = ds.gen_kset(20240618 + k, 0.2, 0.05, 1 << 18, 1.0, k)
    want = check(ctx, orc, sets)
    assert want.size >= int(0.05 * min(s.size for s in sets))


def test_adaptive_served_query_shapes(ctx, orc):
    """A short list against long ones: the lookups touch a few sectors of the
    long lists; the order of the given sets does not matter."""
    rng = np.random.default_rng(9)
    big = [rand_set(rng, 1 << 20, 1 << 26), rand_set(rng, 1 << 19, 1 << 26)]
    short = np.union1d(rand_set(rng, 40, 1 << 26),
                       np.intersect1d(big[0], big[1])[:25]).astype(np.uint32)
    check(ctx, orc, [big[0], short, big[1]])
    check(ctx, orc, [big[1], big[0], short[:1]])


def test_adaptive_edges(ctx, orc):
    e = np.empty(0, np.uint32)
    x = np.array([0, 1, 5, 77, 0xFFFFFFFE, 0xFFFFFFFF], np.uint32)
    for sets in ([e, x], [x, e, x], [x, x.copy()], [x, x.copy(), x.copy()],
                 [np.array([5], np.uint32), x], [x, np.array([2, 6, 78], np.uint32)],
                 [np.arange(0, 5000, 2, dtype=np.uint32), np.arange(1, 5000, 2, dtype=np.uint32)]):
        check(ctx, orc, sets)


def test_adaptive_device_arrays(ctx, orc):
    import torch
    rng = np.random.default_rng(12)
    sets = group(rng, 4, 30_000, 2.0, 2_000, 1 << 24)
    want = orc.svs_generic(sorted(sets, key=len))
    dev = [torch.from_numpy(s.view(np.int32)).cuda() for s in sets]
    w = so.VecWriter()
    so.gpu_small_adaptive(dev, w, ctx=ctx)
    assert np.array_equal(w.into(), want)
