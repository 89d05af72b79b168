"""Bounded device waits: a wait that nothing satisfies ends at the limit set
by setops_gpu_set_wait_limit_ns, the call returns SETOPS_ERR_TIMEOUT (never
a hang, trap or fault), and the same context then gives exact results."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import pair_with_overlap

pytestmark = pytest.mark.gpu

import simd_set_operations_gb300 as so  # noqa: E402
from simd_set_operations_gb300 import _lib  # noqa: E402


def test_wait_ends_at_its_limit_and_context_stays_usable(ctx, orc):
    rng = np.random.default_rng(20261205)
    a, b = pair_with_overlap(rng, 300_000, 500_000, 12_345)
    want = orc.naive_merge(a, b)
    out, n = so.intersect(a, b, ctx=ctx)
    assert np.array_equal(out[:n], want)
    limit = 2_000_000  # 2 ms
    ctx.set_wait_limit_ns(limit)
    try:
        for _ in range(2):
            rc, waited = ctx.check_wait_limit()
            assert rc == _lib.ERR_TIMEOUT, _lib.status_string(rc)
            assert limit <= waited < 500_000_000, waited
            assert "look-back" in _lib.lib.setops_gpu_last_error(ctx.handle).decode()
    finally:
        ctx.set_wait_limit_ns(0)  # back to the default
    # the context is still usable and exact, on every algorithm
    for algo in (so.ALGO_AUTO, so.ALGO_MERGE, so.ALGO_GALLOP, so.ALGO_BITMAP):
        out, n = so.intersect(a, b, algo=algo, ctx=ctx)
        assert np.array_equal(out[:n], want), hex(algo)
        assert so.intersect_count(a, b, algo=algo, ctx=ctx) == want.size


def test_wait_limit_arguments():
    from simd_set_operations_gb300 import _lib as L
    assert L.lib.setops_gpu_set_wait_limit_ns(None, 5) == L.ERR_INVALID
    assert L.lib.setops_gpu_check_wait_limit(None, None) == L.ERR_INVALID
