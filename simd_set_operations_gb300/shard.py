"""Spreading intersection work over several GPUs, one process per GPU.

The path shards without exchanging data: independent pairs, k-set groups and
served queries are units of their own, so each rank takes a contiguous run of
units holding about 1/world of the bytes and no collective touches the data
path.  A single pair too large for one GPU is cut by value into contiguous
pieces of about equal size: rank r intersects A[i_r, i_{r+1}) with the part
of B whose values fall in [A[i_r], A[i_{r+1}]), so an element present in
both inputs lies in one piece, and the pieces' results, in rank order, are
the whole result.  Placing them needs only each rank's count: one all-gather
of 8-byte counts, then an exclusive scan.

The partition functions are plain host logic.  The distributed drivers take
the per-rank intersection as a function (the GPU library by default) and a
torch.distributed process group, so the same code runs over NCCL on GPUs and
over gloo on CPU processes in the tests.
"""
from __future__ import annotations

from typing import Callable, Sequence

import numpy as np


def split_by_bytes(unit_bytes: Sequence[int], world: int) -> list[tuple[int, int]]:
    """Contiguous runs [start, end) of units, one per rank, each holding about
    1/world of the total bytes: rank r's run ends at the first unit whose
    cumulative bytes reach (r+1)/world of the total.  Every unit lands in
    exactly one run; runs may be empty when there are fewer units than
    ranks."""
    if world < 1:
        raise ValueError("world must be >= 1")
    b = np.asarray(unit_bytes, dtype=np.float64)
    n = b.size
    if n == 0:
        return [(0, 0)] * world
    cum = np.cumsum(b)
    total = cum[-1]
    bounds = [0]
    for r in range(1, world):
        # the first unit index whose prefix (inclusive) reaches r/world
        bounds.append(int(np.searchsorted(cum, total * r / world, side="left")) + 1
                      if total > 0 else (n * r) // world)
    bounds.append(n)
    bounds = np.maximum.accumulate(np.minimum(np.array(bounds), n)).tolist()
    return [(int(bounds[r]), int(bounds[r + 1])) for r in range(world)]


def pair_unit_bytes(a_len, b_len) -> np.ndarray:
    """Bytes a pair moves: both u32 inputs read (4 (|A| + |B|))."""
    return 4 * (np.asarray(a_len, np.int64) + np.asarray(b_len, np.int64))


def group_unit_bytes(lens_per_group: Sequence[Sequence[int]]) -> np.ndarray:
    """Bytes a k-set group or served query reads: every list once."""
    return np.array([4 * int(sum(g)) for g in lens_per_group], np.int64)


def split_pair(a: np.ndarray, b: np.ndarray, world: int) -> list[tuple[int, int, int, int]]:
    """Cuts one pair of sorted, duplicate-free arrays into `world` pieces by
    value: piece r = (A[ia_r, ia_{r+1}), B[ib_r, ib_{r+1})) with
    ib_r = lower_bound(B, A[ia_r]), and ia_r the least index whose diagonal
    ia_r + ib_r reaches r (|A| + |B|) / world (the merge path's co-rank, kept
    on a value boundary).  Returns (ia0, ia1, ib0, ib1) per rank."""
    na, nb = int(a.size), int(b.size)
    total = na + nb
    ia = [0]
    for r in range(1, world):
        d = total * r // world
        lo, hi = ia[-1], na  # least i in [lo, na] with i + lower_bound(B, A[i]) >= d
        while lo < hi:
            mid = (lo + hi) // 2
            if mid + int(np.searchsorted(b, a[mid], side="left")) >= d:
                hi = mid
            else:
                lo = mid + 1
        ia.append(lo)
    ia.append(na)
    ib = [0] + [int(np.searchsorted(b, a[i], side="left")) if i < na else nb
                for i in ia[1:-1]] + [nb]
    return [(ia[r], ia[r + 1], ib[r], ib[r + 1]) for r in range(world)]


def exclusive_offsets(counts: Sequence[int]) -> list[int]:
    """Where each rank's result starts in the whole result."""
    out, run = [], 0
    for c in counts:
        out.append(run)
        run += int(c)
    return out


# ---------------------------------------------------------------------------
# distributed drivers (torch.distributed; NCCL on GPUs, gloo on CPUs)

def _gpu_pair(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    from . import intersect
    out, n = intersect(a, b)
    return np.asarray(out[:n])


def _all_counts(n: int, group=None) -> list[int]:
    """One all-gather of each rank's 8-byte count."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    mine = torch.tensor([n], dtype=torch.int64, device=dev)
    every = [torch.zeros(1, dtype=torch.int64, device=dev) for _ in range(world)]
    dist.all_gather(every, mine, group=group)
    return [int(t.item()) for t in every]


def sharded_pair(a: np.ndarray, b: np.ndarray,
                 local: Callable[[np.ndarray, np.ndarray], np.ndarray] | None = None,
                 group=None) -> tuple[np.ndarray, int, int]:
    """This rank's piece of A ∩ B for a pair cut by split_pair: returns
    (piece result, its offset in the whole result, the whole result's
    length).  Every rank holds (or can read) both inputs; the only exchange
    is the count all-gather."""
    import torch.distributed as dist
    local = local or _gpu_pair
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    ia0, ia1, ib0, ib1 = split_pair(a, b, world)[rank]
    piece = local(a[ia0:ia1], b[ib0:ib1])
    counts = _all_counts(int(piece.size), group)
    return piece, exclusive_offsets(counts)[rank], sum(counts)


def sharded_pairs(pairs: Sequence[tuple[np.ndarray, np.ndarray]],
                  local: Callable[[np.ndarray, np.ndarray], np.ndarray] | None = None,
                  group=None) -> tuple[int, int, list[np.ndarray]]:
    """This rank's run of independent pairs (split_by_bytes over their input
    bytes), each intersected by `local`: returns (first pair index, end,
    results).  No collective."""
    import torch.distributed as dist
    local = local or _gpu_pair
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    sizes = pair_unit_bytes([p[0].size for p in pairs], [p[1].size for p in pairs])
    s, e = split_by_bytes(sizes, world)[rank]
    return s, e, [local(pairs[i][0], pairs[i][1]) for i in range(s, e)]


def gather_pieces(piece: np.ndarray, offset: int, total: int, group=None,
                  dst: int = 0) -> np.ndarray | None:
    """Assembles the whole result on rank `dst` from every rank's piece and
    offset (a gather of the pieces padded to the longest); other ranks get
    None."""
    import torch
    import torch.distributed as dist
    world, rank = dist.get_world_size(group), dist.get_rank(group)
    counts = _all_counts(int(piece.size), group)
    longest = max(max(counts), 1)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    buf = torch.zeros(longest, dtype=torch.int64, device=dev)
    buf[:piece.size] = torch.from_numpy(piece.astype(np.int64)).to(dev)
    bufs = [torch.zeros(longest, dtype=torch.int64, device=dev) for _ in range(world)] \
        if rank == dst else None
    dist.gather(buf, bufs, dst=dst, group=group)
    if rank != dst:
        return None
    out = np.empty(total, np.uint32)
    for r, (c, o) in enumerate(zip(counts, exclusive_offsets(counts))):
        out[o:o + c] = bufs[r][:c].cpu().numpy().astype(np.uint32)
    return out
