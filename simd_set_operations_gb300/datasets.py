"""Benchmark-side inputs: seeded synthetic generators and the datafile format.

Python face of include/setops_bench.h.  The generators restate
benchmark/src/generators.rs of the reference with a seeded PRNG; the
datafile functions restate benchmark/src/datafile.rs.  Host only.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

# (name, restype, argtypes) of the generator and datafile functions of
# include/setops_bench.h
_vp, _sz, _u64, _d = C.c_void_p, C.c_size_t, C.c_uint64, C.c_double
GEN_SIGNATURES = [
    ("setops_gen_twoset", C.c_int, [_u64, _d, _d, _sz, _sz, _vp, _vp]),
    ("setops_gen_kset_lens", C.c_int, [_sz, _d, _sz, C.POINTER(_sz)]),
    ("setops_gen_kset", C.c_int, [_u64, _d, _d, _sz, _d, _sz, C.POINTER(_vp)]),
    ("setops_gen_batch_sizes", C.c_int, [_u64, _sz, _sz, _sz, _vp, _vp]),
    ("setops_gen_batch_fill", C.c_int, [_u64, _sz, _vp, _vp, _vp, _vp, _d, _d, _d, _d, _vp,
                                        C.c_int]),
    ("setops_gen_index_lens", C.c_int, [_sz, _sz, _d, _vp]),
    ("setops_gen_index_fill", C.c_int, [_u64, _sz, _vp, _vp, _u64, _vp, C.c_int]),
    ("setops_gen_queries", C.c_int, [_u64, _sz, _sz, C.c_uint32, C.c_uint32, _d, _vp, _vp]),
    ("setops_gen_bsr_encode", C.c_int, [_vp, _sz, _vp, _vp, _vp, _vp, _vp, _vp]),
    ("setops_gen_sorted_sample", C.c_int, [_u64, _sz, _u64, _vp]),
    ("setops_datafile_write", C.c_int, [C.c_char_p, C.POINTER(_vp), _vp, _sz]),
    ("setops_datafile_read_header", C.c_int, [C.c_char_p, C.POINTER(_u64), _vp, _sz]),
    ("setops_datafile_read_sets", C.c_int, [C.c_char_p, C.POINTER(_vp)]),
]

_gen = None


def use_library(cdll: C.CDLL) -> None:
    """Run the generators in `cdll`, any library built from csrc/gen.cpp.

    The default is libsetops_gpu.so.  A CPU-only process that must not map
    the GPU library (the timed CPU reference path) loads this module on its
    own and passes the CPU oracle's library, which is built from the same
    generator source and so gives the same inputs."""
    global _gen
    for name, res, args in GEN_SIGNATURES:
        fn = getattr(cdll, name)
        fn.restype = res
        fn.argtypes = args
    _gen = cdll


def _L() -> C.CDLL:
    if _gen is None:
        from ._lib import lib
        use_library(lib)
    return _gen


def _cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def gen_twoset(seed: int, density: float, selectivity: float, small_len: int,
               large_len: int) -> tuple[np.ndarray, np.ndarray]:
    """gen_twoset (generators.rs:30-68) for explicit lengths."""
    s = np.empty(max(small_len, 1), np.uint32)
    l = np.empty(max(large_len, 1), np.uint32)
    rc = _L().setops_gen_twoset(seed, density, selectivity, small_len, large_len,
                               s.ctypes.data, l.ctypes.data)
    if rc != 0:
        raise ValueError("setops_gen_twoset: bad arguments")
    return s[:small_len], l[:large_len]


def kset_lens(max_len: int, skewness: float, set_count: int) -> list[int]:
    lens = (C.c_size_t * set_count)()
    if _L().setops_gen_kset_lens(max_len, skewness, set_count, lens) != 0:
        raise ValueError("setops_gen_kset_lens: bad arguments")
    return list(lens)


def gen_kset(seed: int, density: float, selectivity: float, max_len: int,
             skewness: float, set_count: int) -> list[np.ndarray]:
    """gen_kset (generators.rs:112-135): smallest set first."""
    lens = kset_lens(max_len, skewness, set_count)
    outs = [np.empty(max(n, 1), np.uint32) for n in lens]
    ptrs = (C.c_void_p * set_count)(*[o.ctypes.data for o in outs])
    if _L().setops_gen_kset(seed, density, selectivity, max_len, skewness, set_count, ptrs) != 0:
        raise ValueError("setops_gen_kset: bad arguments")
    return [o[:n] for o, n in zip(outs, lens)]


def sorted_sample(seed: int, n: int, max_value: int) -> np.ndarray:
    out = np.empty(max(n, 1), np.uint32)
    if _L().setops_gen_sorted_sample(seed, n, max_value, out.ctypes.data) != 0:
        raise ValueError("setops_gen_sorted_sample: bad arguments")
    return out[:n]


@dataclass
class PairBatch:
    """Uneven pairs stored in one pool: pair p is
    pool[a_off[p]:a_off[p]+a_len[p]] and pool[b_off[p]:b_off[p]+b_len[p]]."""
    pool: np.ndarray
    a_off: np.ndarray
    a_len: np.ndarray
    b_off: np.ndarray
    b_len: np.ndarray

    def __len__(self) -> int:
        return int(self.a_len.size)

    def pair(self, p: int) -> tuple[np.ndarray, np.ndarray]:
        return (self.pool[self.a_off[p]:self.a_off[p] + self.a_len[p]],
                self.pool[self.b_off[p]:self.b_off[p] + self.b_len[p]])


def gen_batch(seed: int, npairs: int, min_len: int = 16, max_len: int = 1 << 16,
              density: tuple[float, float] = (0.01, 0.5),
              selectivity: tuple[float, float] = (0.0, 0.5),
              nthreads: int | None = None) -> PairBatch:
    """Batched uneven pairs: lengths log-uniform in [min_len, max_len]."""
    a_len = np.empty(npairs, np.uint64)
    b_len = np.empty(npairs, np.uint64)
    if _L().setops_gen_batch_sizes(seed, npairs, min_len, max_len, a_len.ctypes.data,
                                  b_len.ctypes.data) != 0:
        raise ValueError("setops_gen_batch_sizes: bad arguments")
    lens = np.empty(2 * npairs, np.uint64)
    lens[0::2], lens[1::2] = a_len, b_len
    offs = np.zeros(2 * npairs, np.uint64)
    if npairs:
        offs[1:] = np.cumsum(lens[:-1])
    a_off, b_off = offs[0::2].copy(), offs[1::2].copy()
    pool = np.empty(max(int(lens.sum()), 1), np.uint32)
    if _L().setops_gen_batch_fill(seed ^ 0x5EED, npairs, a_len.ctypes.data, b_len.ctypes.data,
                                 a_off.ctypes.data, b_off.ctypes.data, density[0], density[1],
                                 selectivity[0], selectivity[1], pool.ctypes.data,
                                 nthreads or _cores()) != 0:
        raise ValueError("setops_gen_batch_fill: bad arguments")
    return PairBatch(pool, a_off, a_len, b_off, b_len)


@dataclass
class BsrBatch:
    """Pairs of BSR sets in one pool: set words are (bases[i], states[i]);
    pair p is words [a_off[p], +a_len[p]) and [b_off[p], +b_len[p])."""
    bases: np.ndarray
    states: np.ndarray
    a_off: np.ndarray
    a_len: np.ndarray
    b_off: np.ndarray
    b_len: np.ndarray

    def __len__(self) -> int:
        return int(self.a_len.size)

    def pair(self, p: int):
        a0, na, b0, nb = (int(self.a_off[p]), int(self.a_len[p]), int(self.b_off[p]),
                          int(self.b_len[p]))
        return (self.bases[a0:a0 + na], self.states[a0:a0 + na],
                self.bases[b0:b0 + nb], self.states[b0:b0 + nb])


def bsr_encode_batch(batch: PairBatch) -> BsrBatch:
    """BSR form (BsrVec::from_sorted, setops/src/bsr.rs:140-163) of every set
    of a PairBatch, packed in one pool."""
    n = len(batch)
    offs = np.empty(2 * n, np.uint64)
    lens = np.empty(2 * n, np.uint64)
    offs[0::2], offs[1::2] = batch.a_off, batch.b_off
    lens[0::2], lens[1::2] = batch.a_len, batch.b_len
    cap = max(int(lens.sum()), 1)
    bases = np.empty(cap, np.uint32)
    states = np.empty(cap, np.uint32)
    woffs = np.empty(2 * n, np.uint64)
    wlens = np.empty(2 * n, np.uint64)
    if _L().setops_gen_bsr_encode(batch.pool.ctypes.data, 2 * n, offs.ctypes.data,
                                 lens.ctypes.data, bases.ctypes.data, states.ctypes.data,
                                 woffs.ctypes.data, wlens.ctypes.data) != 0:
        raise ValueError("setops_gen_bsr_encode: bad arguments")
    total = int(wlens.sum())
    return BsrBatch(bases[:max(total, 1)], states[:max(total, 1)], woffs[0::2].copy(),
                    wlens[0::2].copy(), woffs[1::2].copy(), wlens[1::2].copy())


@dataclass
class PostingIndex:
    """Posting lists stored in one pool: list i is pool[offs[i]:offs[i]+lens[i]]."""
    pool: np.ndarray
    offs: np.ndarray
    lens: np.ndarray
    doc_space: int

    def __len__(self) -> int:
        return int(self.lens.size)

    def list(self, i: int) -> np.ndarray:
        return self.pool[self.offs[i]:self.offs[i] + self.lens[i]]


def gen_index(seed: int, nlists: int, max_len: int = 1 << 20, s: float = 1.1,
              doc_space: int = 1 << 26, nthreads: int | None = None) -> PostingIndex:
    """Rank-size Zipf posting lists: |list r| = clip(max_len / r^s, 1, max_len)."""
    lens = np.empty(nlists, np.uint64)
    if _L().setops_gen_index_lens(nlists, max_len, s, lens.ctypes.data) != 0:
        raise ValueError("setops_gen_index_lens: bad arguments")
    offs = np.zeros(nlists, np.uint64)
    if nlists:
        offs[1:] = np.cumsum(lens[:-1])
    pool = np.empty(max(int(lens.sum()), 1), np.uint32)
    if _L().setops_gen_index_fill(seed, nlists, lens.ctypes.data, offs.ctypes.data, doc_space,
                                 pool.ctypes.data, nthreads or _cores()) != 0:
        raise ValueError("setops_gen_index_fill: bad arguments")
    return PostingIndex(pool, offs, lens, doc_space)


def gen_queries(seed: int, nq: int, nlists: int, kmin: int = 2, kmax: int = 6,
                s: float = 1.1) -> tuple[np.ndarray, np.ndarray]:
    """k-set queries: k uniform in [kmin, kmax], then k distinct list ids
    drawn Zipf(s) over popularity rank.  Returns (ids[nq, kmax], ks[nq])."""
    ids = np.zeros((nq, kmax), np.uint32)
    ks = np.zeros(nq, np.uint32)
    if _L().setops_gen_queries(seed, nq, nlists, kmin, kmax, s, ids.ctypes.data,
                              ks.ctypes.data) != 0:
        raise ValueError("setops_gen_queries: bad arguments")
    return ids, ks


# ---- datafile (benchmark/src/datafile.rs) ---------------------------------

class DatafileError(ValueError):
    CODES = {-1: "bad argument", -2: "I/O error", -3: "bad set count",
             -4: "bad magic", -5: "bad endianness", -6: "too many sets"}

    def __init__(self, code: int):
        super().__init__(self.CODES.get(code, f"error {code}"))
        self.code = code


def datafile_write(path: str, sets) -> None:
    arrs = [np.ascontiguousarray(s, dtype=np.uint32) for s in sets]
    n = len(arrs)
    ptrs = (C.c_void_p * max(n, 1))(*[a.ctypes.data if a.size else None for a in arrs])
    lens = np.array([a.size for a in arrs], np.uint64)
    rc = _L().setops_datafile_write(str(path).encode(), ptrs, lens.ctypes.data if n else None, n)
    if rc != 0:
        raise DatafileError(rc)


def datafile_read(path: str) -> list[np.ndarray]:
    cnt = C.c_uint64()
    rc = _L().setops_datafile_read_header(str(path).encode(), C.byref(cnt), None, 0)
    if rc != 0:
        raise DatafileError(rc)
    lens = np.empty(cnt.value, np.uint64)
    rc = _L().setops_datafile_read_header(str(path).encode(), C.byref(cnt), lens.ctypes.data,
                                         lens.size)
    if rc != 0:
        raise DatafileError(rc)
    outs = [np.empty(max(int(n), 1), np.uint32) for n in lens]
    ptrs = (C.c_void_p * len(outs))(*[o.ctypes.data for o in outs])
    rc = _L().setops_datafile_read_sets(str(path).encode(), ptrs)
    if rc != 0:
        raise DatafileError(rc)
    return [o[:int(n)] for o, n in zip(outs, lens)]
