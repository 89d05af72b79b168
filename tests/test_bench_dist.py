"""The bench's multi-process host logic on CPU: two gloo ranks (one process
each, as torchrun would start them) agree on the slowest rank's time, compute
the same whole-job value, and intersect distinct pairs of the same shapes.
No GPU: only the host-side pieces of bench.py run."""
from __future__ import annotations

import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        r, w, local = bench.dist_env()
        t = bench.max_over_ranks(0.5 + rank)  # rank 1 is the slow one
        v = bench.job_value(w, 4, 10, t)
        q.put((r, w, local, t, v, bench.sweep_seeds(r)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 and r[2] == r[0] for r in res)
    assert all(r[3] == 1.5 for r in res)                  # max over ranks
    assert all(abs(r[4] - 2 * 4 * 10 / 1.5) < 1e-9 for r in res)  # whole-job pairs/s
    s0, s1 = res[0][5], res[1][5]
    assert len(s0) == len(s1) == 4 and not set(s0) & set(s1)      # distinct pairs per rank


def test_single_process_defaults(monkeypatch):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.dist_env() == (0, 1, 0)
    assert bench.max_over_ranks(2.0) == 2.0
    assert bench.job_value(1, 4, 10, 2.0) == 20.0


def test_touched_bytes_and_summary():
    """The bench's estimate of the bytes a search-band pair touches (the
    sectors its probes reach, capped at the whole larger set) and the
    summary object built from the legs (absent legs give no keys)."""
    sys.path.insert(0, str(ROOT))
    import bench
    ns, nl = 1 << 10, 1 << 24
    per = 14 - 2  # ceil(log2(2^14)) - 2 sectors per small element
    assert bench.touched_bytes(ns, nl, 10) == 4 * ns + 40 + 32 * per * ns
    assert bench.touched_bytes(1 << 22, nl, 0) == 4 * (1 << 22) + 4 * nl  # capped
    sizes = [bench.touched_bytes(1 << e, nl, 0) for e in range(4, 20)]
    assert sizes == sorted(sizes)
    assert bench.algorithmic_bytes(1 << 24, 1 << 24, 167_772) == 134_888_816
    s = bench.summarize({"frac": 0.4123}, None, None, None, None, None, None)
    assert s == {"headline_frac": 0.412, "sweep_e2e_pairs_per_s": None,
                 "sweep_e2e_per_call_pairs_per_s": None, "sweep_cpu_pairs_per_s": None}
