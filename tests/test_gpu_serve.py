"""Serving k-set queries (setops_srv_*): every answer must equal svs_generic
over the query's lists (the reference's k-set path, setops/src/intersect/
svs.rs:50-73, with naive_merge), and be the same whether the query runs alone
or batched with others, under an open-loop Poisson load included."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import simd_set_operations_gb300 as so  # noqa: E402
from simd_set_operations_gb300 import datasets as ds  # noqa: E402


@pytest.fixture(scope="module")
def index():
    return ds.gen_index(20240612, 20000, 1 << 14, 1.1, 1 << 22)


@pytest.fixture(scope="module")
def queries(index):
    return ds.gen_queries(20240613, 400, len(index), 2, 6, 1.1)


def oracle_answers(orc, index, ids, ks):
    groups = [[index.list(int(i)) for i in ids[q][:ks[q]]] for q in range(ks.size)]
    outs = [np.empty(max(min(g.size for g in grp), 1), np.uint32) for grp in groups]
    counts = orc.run_svs_groups(groups, 8, outs=outs)
    return [o[:int(c)] for o, c in zip(outs, counts)]


def test_serve_alone_mix_and_oracle(ctx, orc, index, queries):
    ids, ks = queries
    want = oracle_answers(orc, index, ids, ks)
    with so.Server(index.pool, index.offs, index.lens, ctx=ctx) as srv:
        # alone: one query on the GPU at a time
        alone = []
        for q in range(ks.size):
            srv.submit(ids[q][:ks[q]], q)
            tag, res, lat = srv.wait(q)
            assert tag == q and lat > 0
            alone.append(res)
        # in the mix: all submitted at once, batched together
        for q in range(ks.size):
            srv.submit(ids[q][:ks[q]], 10_000 + q)
        mix = {}
        while len(mix) < ks.size:
            r = srv.poll()
            if r is not None:
                mix[r[0] - 10_000] = r[1]
        st = srv.stats()
        assert st["max_batch"] > 1, st  # the mix really was batched
        for q in range(ks.size):
            assert np.array_equal(alone[q], want[q]), q
            assert np.array_equal(mix[q], want[q]), q


def test_serve_poisson_load(ctx, orc, index, queries):
    ids, ks = queries
    want = oracle_answers(orc, index, ids, ks)
    reps = 5
    ids_r, ks_r = np.tile(ids, (reps, 1)), np.tile(ks, reps)
    stride = max(max(w.size for w in want), 1)
    with so.Server(index.pool, index.offs, index.lens, budget=16 << 20, ctx=ctx) as srv:
        lat, cnt, el, answers = srv.run_load(ids_r, ks_r, rate_qps=200000, seed=3,
                                             answer_stride=stride)
        st = srv.stats()
    assert el > 0 and np.all(lat > 0)
    assert st["max_batch"] > 1, st  # queries arriving under load were batched together
    assert [int(c) for c in cnt] == [w.size for w in want] * reps
    for q, got in enumerate(answers):  # every answer under load, element by element
        assert np.array_equal(got, want[q % ks.size]), q


def test_serve_rejects_bad_queries(ctx, index):
    with so.Server(index.pool, index.offs, index.lens, ctx=ctx) as srv:
        with pytest.raises(so.SetopsError):
            srv.submit([1], 0)  # k < 2
        with pytest.raises(so.SetopsError):
            srv.submit([0, len(index)], 0)  # no such list


def test_serve_long_lists_split(ctx, orc):
    """Queries over lists longer than one unit (16384 elements), whose steps
    are split over CTAs: answers equal svs_generic alone and batched."""
    index = ds.gen_index(20240617, 3000, 1 << 17, 1.0, 1 << 21)
    ids, ks = ds.gen_queries(20240618, 120, len(index), 2, 5, 1.3)
    want = oracle_answers(orc, index, ids, ks)
    assert max(int(min(index.lens[int(i)] for i in ids[q][:ks[q]])) for q in range(ks.size)) > 16384
    with so.Server(index.pool, index.offs, index.lens, ctx=ctx) as srv:
        for q in range(0, ks.size, 7):
            srv.submit(ids[q][:ks[q]], q)
            tag, res, _ = srv.wait(q)
            assert tag == q and np.array_equal(res, want[q]), q
        for q in range(ks.size):
            srv.submit(ids[q][:ks[q]], 10_000 + q)
        mix = {}
        while len(mix) < ks.size:
            r = srv.poll()
            if r is not None:
                mix[r[0] - 10_000] = r[1]
        for q in range(ks.size):
            assert np.array_equal(mix[q], want[q]), q
