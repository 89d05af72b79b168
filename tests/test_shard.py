"""Spreading the work over ranks (simd_set_operations_gb300/shard.py) on CPU:
the byte-balanced split of independent units, the value-aligned split of one
pair (whose pieces' results, in rank order, are the whole result), and two
gloo ranks running both through torch.distributed with the oracle as each
rank's intersection -- no GPU."""
from __future__ import annotations

import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import pair_with_overlap, rand_set

ROOT = Path(__file__).resolve().parents[1]


def test_split_by_bytes_covers_and_balances():
    from simd_set_operations_gb300 import shard
    rng = np.random.default_rng(1)
    for n, world in ((1, 1), (5, 8), (100, 3), (10_000, 8), (7, 7)):
        b = rng.integers(0, 1 << 20, n)
        runs = shard.split_by_bytes(b, world)
        assert len(runs) == world and runs[0][0] == 0 and runs[-1][1] == n
        assert all(runs[r][1] == runs[r + 1][0] for r in range(world - 1))  # contiguous
        assert all(s <= e for s, e in runs)
        loads = [int(b[s:e].sum()) for s, e in runs]
        # each run is within one unit of the even share
        assert max(loads) <= b.sum() / world + b.max() + 1
    assert shard.split_by_bytes([], 3) == [(0, 0)] * 3
    assert shard.split_by_bytes([0, 0, 0, 0], 2) == [(0, 2), (2, 4)]


def test_split_pair_pieces_make_the_whole(orc):
    from simd_set_operations_gb300 import shard
    rng = np.random.default_rng(2)
    cases = [pair_with_overlap(rng, 5000, 7000, 900), pair_with_overlap(rng, 30, 90_000, 20),
             (np.arange(0, 1000, dtype=np.uint32), np.arange(0, 1000, dtype=np.uint32)),
             (np.arange(0, 1000, 2, dtype=np.uint32), np.arange(1, 1000, 2, dtype=np.uint32)),
             (np.empty(0, np.uint32), rand_set(rng, 50, 1000)),
             (rand_set(rng, 3, 1 << 32), rand_set(rng, 3, 1 << 32))]
    for a, b in cases:
        want = orc.naive_merge(a, b)
        for world in (1, 2, 3, 5, 8):
            pieces = shard.split_pair(a, b, world)
            assert pieces[0][0] == 0 and pieces[0][2] == 0
            assert pieces[-1][1] == a.size and pieces[-1][3] == b.size
            got = np.concatenate([orc.naive_merge(a[i0:i1], b[j0:j1])
                                  for i0, i1, j0, j1 in pieces])
            assert np.array_equal(got, want), (a.size, b.size, world)
            if a.size + b.size >= 1000:  # pieces of about equal size: a cut moves in
                # steps of one A element and the B elements before the next one
                sizes = [(i1 - i0) + (j1 - j0) for i0, i1, j0, j1 in pieces]
                step = 1 + int(np.diff(np.searchsorted(b, a)).max()) if a.size > 1 else b.size
                assert max(sizes) <= (a.size + b.size) / world + 2 * step
    assert shard.exclusive_offsets([3, 0, 5]) == [0, 3, 3]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests"))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle
        from conftest import pair_with_overlap as pwo
        from simd_set_operations_gb300 import shard
        rng = np.random.default_rng(3)  # the same inputs on every rank
        a, b = pwo(rng, 40_000, 60_000, 3_000)
        piece, off, total = shard.sharded_pair(a, b, local=oracle.naive_merge)
        whole = shard.gather_pieces(piece, off, total)
        pairs = [pwo(rng, int(rng.integers(1, 5000)), int(rng.integers(1, 5000)), 10)
                 for _ in range(50)]
        s, e, res = shard.sharded_pairs(pairs, local=oracle.naive_merge)
        ok_pairs = all(np.array_equal(r, oracle.naive_merge(*pairs[s + i]))
                       for i, r in enumerate(res))
        q.put((rank, off, total, None if whole is None else whole.tolist() ==
               oracle.naive_merge(a, b).tolist(), s, e, ok_pairs))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_a_pair_and_a_batch():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=180) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, off0, tot0, whole0, s0, e0, ok0), (r1, off1, tot1, whole1, s1, e1, ok1) = res
    assert off0 == 0 and 0 < off1 < tot0 == tot1 == 3_000
    assert whole0 is True and whole1 is None          # assembled on rank 0 only
    assert s0 == 0 and e0 == s1 and e1 == 50 and ok0 and ok1  # every pair once
