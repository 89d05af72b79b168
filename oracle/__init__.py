"""CPU oracle for the GPU intersection path -- TEST INFRASTRUCTURE ONLY.

ctypes wrapper of ``liboracle.so`` (oracle.c, a plain-C restatement of the
reference's CPU path; each function cites the reference file:line it
follows) and, where it was built, of ``_ref/libref_qfilter.so`` (the
reference's own C++ kernels, setops/ffi/qfilter/qfilter.cpp, compiled
unchanged; x86 hosts only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline and
reference legs may use this package, as the checker or as the timed CPU
baseline.  The product (simd_set_operations_gb300) never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libref_qfilter.so"

NAIVE_MERGE = 0
BRANCHLESS_MERGE = 1
GALLOPING = 2
SHUFFLING_W8 = 3
SIMD_GALLOPING_W16 = 4
BMISS_W4 = 5
ALGO_NAMES = {
    NAIVE_MERGE: "naive_merge",
    BRANCHLESS_MERGE: "branchless_merge",
    GALLOPING: "galloping",
    SHUFFLING_W8: "shuffling_avx2 (portable 8-lane restatement)",
    SIMD_GALLOPING_W16: "galloping_avx512 (portable 16-lane restatement)",
    BMISS_W4: "bmiss (portable restatement)",
}


GEN_SRC = HERE.parent / "simd_set_operations_gb300" / "csrc" / "gen.cpp"


def build(ref_root: str | None = None) -> None:
    """make liboracle.so and, when `ref_root` (the reference tree) is given,
    the reference's own kernels into _ref/."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    if ref_root:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF_ROOT={ref_root}"],
                       check=True)


_lib = None
_ref = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists() or any(LIB.stat().st_mtime < p.stat().st_mtime
                                   for p in (HERE / "oracle.c", GEN_SRC)):
            build()
        L = C.CDLL(str(LIB))
        vp, sz = C.c_void_p, C.c_size_t
        for name in ("orc_naive_merge", "orc_branchless_merge", "orc_galloping",
                     "orc_binary_search_intersect", "orc_shuffling_w8",
                     "orc_simd_galloping_w16", "orc_bmiss_w4"):
            f = getattr(L, name)
            f.restype = sz
            f.argtypes = [vp, sz, vp, sz, vp]
        L.orc_binary_search.restype = sz
        L.orc_binary_search.argtypes = [vp, C.c_uint32, C.c_ssize_t, C.c_ssize_t]
        L.orc_bsr_from_sorted.restype = sz
        L.orc_bsr_from_sorted.argtypes = [vp, sz, vp, vp]
        L.orc_bsr_to_sorted.restype = sz
        L.orc_bsr_to_sorted.argtypes = [vp, vp, sz, vp]
        for name in ("orc_branchless_merge_bsr", "orc_galloping_bsr"):
            f = getattr(L, name)
            f.restype = sz
            f.argtypes = [vp, vp, sz, vp, vp, sz, vp, vp, vp]
        L.orc_broadcast_bsr.restype = sz
        L.orc_broadcast_bsr.argtypes = [C.c_int, vp, vp, sz, vp, vp, sz, vp, vp, vp]
        L.orc_svs_generic.restype = sz
        L.orc_svs_generic.argtypes = [C.POINTER(vp), C.POINTER(sz), sz, vp, vp,
                                      C.POINTER(vp)]
        L.orc_run_pairs.restype = C.c_int
        L.orc_run_pairs.argtypes = [C.c_int, sz, C.POINTER(vp), C.POINTER(sz),
                                    C.POINTER(vp), C.POINTER(sz), C.POINTER(vp),
                                    C.POINTER(C.c_uint64), C.c_int]
        L.orc_run_svs_groups.restype = C.c_int
        L.orc_run_svs_groups.argtypes = [sz, C.POINTER(vp), C.POINTER(sz),
                                         C.POINTER(sz), C.POINTER(vp),
                                         C.POINTER(C.c_uint64), C.c_int]
        L.orc_small_adaptive.restype = sz
        L.orc_small_adaptive.argtypes = [C.POINTER(vp), C.POINTER(sz), sz, vp]
        L.orc_run_bsr_pairs.restype = C.c_int
        L.orc_run_bsr_pairs.argtypes = [C.c_int, sz] + [C.POINTER(vp)] * 2 + [C.POINTER(sz)] + \
            [C.POINTER(vp)] * 2 + [C.POINTER(sz)] + [C.POINTER(vp)] * 2 + \
            [C.POINTER(C.c_uint64), C.c_int]
        L.orc_run_svs_groups_algo.restype = C.c_int
        L.orc_run_svs_groups_algo.argtypes = [C.c_int, sz, C.POINTER(vp), C.POINTER(sz),
                                              C.POINTER(sz), C.POINTER(vp),
                                              C.POINTER(C.c_uint64), C.c_int]
        _lib = L
    return _lib


def _u32(x) -> np.ndarray:
    return np.ascontiguousarray(x, dtype=np.uint32)


def _ptr(a: np.ndarray):
    return a.ctypes.data if a.size else None


def _two(fn_name: str, a, b) -> np.ndarray:
    a, b = _u32(a), _u32(b)
    out = np.empty(max(min(a.size, b.size), 1), np.uint32)
    n = getattr(lib(), fn_name)(_ptr(a), a.size, _ptr(b), b.size, out.ctypes.data)
    return out[:n].copy()


def _two_count(fn_name: str, a, b) -> int:
    a, b = _u32(a), _u32(b)
    return int(getattr(lib(), fn_name)(_ptr(a), a.size, _ptr(b), b.size, None))


def naive_merge(a, b) -> np.ndarray:
    return _two("orc_naive_merge", a, b)


def naive_merge_count(a, b) -> int:
    return _two_count("orc_naive_merge", a, b)


def branchless_merge(a, b) -> np.ndarray:
    return _two("orc_branchless_merge", a, b)


def galloping(small, large) -> np.ndarray:
    return _two("orc_galloping", small, large)


def binary_search_intersect(small, large) -> np.ndarray:
    return _two("orc_binary_search_intersect", small, large)


def shuffling_w8(a, b) -> np.ndarray:
    return _two("orc_shuffling_w8", a, b)


def simd_galloping_w16(a, b) -> np.ndarray:
    return _two("orc_simd_galloping_w16", a, b)


def bmiss_w4(a, b) -> np.ndarray:
    return _two("orc_bmiss_w4", a, b)


def binary_search(arr, target: int, lo: int, hi: int) -> int:
    a = _u32(arr)
    return int(lib().orc_binary_search(_ptr(a), target, lo, hi))


def bsr_from_sorted(arr):
    a = _u32(arr)
    bases = np.empty(max(a.size, 1), np.uint32)
    states = np.empty(max(a.size, 1), np.uint32)
    w = lib().orc_bsr_from_sorted(_ptr(a), a.size, bases.ctypes.data, states.ctypes.data)
    return bases[:w].copy(), states[:w].copy()


def bsr_to_sorted(bases, states) -> np.ndarray:
    b, s = _u32(bases), _u32(states)
    n = lib().orc_bsr_to_sorted(_ptr(b), _ptr(s), b.size, None)
    out = np.empty(max(n, 1), np.uint32)
    lib().orc_bsr_to_sorted(_ptr(b), _ptr(s), b.size, out.ctypes.data)
    return out[:n].copy()


def _bsr2(fn_name, ba, sa, bb, sb, count_only=False):
    ba, sa, bb, sb = map(_u32, (ba, sa, bb, sb))
    cnt = C.c_uint64()
    if count_only:
        getattr(lib(), fn_name)(_ptr(ba), _ptr(sa), ba.size, _ptr(bb), _ptr(sb), bb.size,
                                None, None, C.byref(cnt))
        return int(cnt.value)
    m = max(min(ba.size, bb.size), 1)
    ob, os_ = np.empty(m, np.uint32), np.empty(m, np.uint32)
    w = getattr(lib(), fn_name)(_ptr(ba), _ptr(sa), ba.size, _ptr(bb), _ptr(sb), bb.size,
                                ob.ctypes.data, os_.ctypes.data, C.byref(cnt))
    return ob[:w].copy(), os_[:w].copy()


def branchless_merge_bsr(ba, sa, bb, sb):
    return _bsr2("orc_branchless_merge_bsr", ba, sa, bb, sb)


def branchless_merge_bsr_count(ba, sa, bb, sb) -> int:
    return _bsr2("orc_branchless_merge_bsr", ba, sa, bb, sb, count_only=True)


def galloping_bsr(ba, sa, bb, sb):
    return _bsr2("orc_galloping_bsr", ba, sa, bb, sb)


def broadcast_bsr(ba, sa, bb, sb, w: int = 8):
    """broadcast_*_bsr (setops/src/intersect/broadcast.rs:163-357) with
    blocks of w bases."""
    ba, sa, bb, sb = map(_u32, (ba, sa, bb, sb))
    cnt = C.c_uint64()
    m = max(min(ba.size, bb.size), 1)
    ob, os_ = np.empty(m, np.uint32), np.empty(m, np.uint32)
    n = lib().orc_broadcast_bsr(int(w), _ptr(ba), _ptr(sa), ba.size, _ptr(bb), _ptr(sb), bb.size,
                                ob.ctypes.data, os_.ctypes.data, C.byref(cnt))
    return ob[:n].copy(), os_[:n].copy()


def svs_generic(sets) -> np.ndarray:
    """svs_generic with naive_merge, sets in the given order."""
    arrs = [_u32(s) for s in sets]
    k = len(arrs)
    cap = max(max((a.size for a in arrs), default=0), 1)
    left, right = np.empty(cap, np.uint32), np.empty(cap, np.uint32)
    ptrs = (C.c_void_p * k)(*[_ptr(a) for a in arrs])
    lens = (C.c_size_t * k)(*[a.size for a in arrs])
    res = C.c_void_p()
    n = lib().orc_svs_generic(ptrs, lens, k, left.ctypes.data, right.ctypes.data, C.byref(res))
    buf = left if res.value == left.ctypes.data else right
    return buf[:n].copy()


def small_adaptive(sets) -> np.ndarray:
    """small_adaptive (setops/src/intersect/adaptive.rs:107-148) over
    [s0, s1, ...]; s0 is the set whose elements are looked up."""
    arrs = [_u32(s) for s in sets]
    k = len(arrs)
    out = np.empty(max(arrs[0].size if arrs else 0, 1), np.uint32)
    P = (C.c_void_p * k)(*[_ptr(a) for a in arrs])
    N = (C.c_size_t * k)(*[a.size for a in arrs])
    n = lib().orc_small_adaptive(P, N, k, out.ctypes.data)
    return out[:n].copy()


def run_pairs(algo: int, pairs, nthreads: int = 1, outs=None) -> np.ndarray:
    """Runs `algo` over [(a, b), ...] on `nthreads` threads; returns counts.
    `outs` (list of uint32 arrays, capacity >= min len) materialises."""
    n = len(pairs)
    keep = [(_u32(a), _u32(b)) for a, b in pairs]
    A = (C.c_void_p * n)(*[_ptr(a) for a, _ in keep])
    NA = (C.c_size_t * n)(*[a.size for a, _ in keep])
    B = (C.c_void_p * n)(*[_ptr(b) for _, b in keep])
    NB = (C.c_size_t * n)(*[b.size for _, b in keep])
    O = (C.c_void_p * n)(*[o.ctypes.data for o in outs]) if outs is not None else None
    counts = np.zeros(n, np.uint64)
    rc = lib().orc_run_pairs(algo, n, A, NA, B, NB, O,
                             counts.ctypes.data_as(C.POINTER(C.c_uint64)), nthreads)
    if rc != 0:
        raise ValueError("orc_run_pairs: bad argument")
    return counts


def run_svs_groups(groups, nthreads: int = 1, outs=None, algo: int = NAIVE_MERGE) -> np.ndarray:
    """k-set groups [[s0, s1, ...], ...] through svs_generic with the 2-set
    function `algo` in every step (naive_merge by default)."""
    flat = [_u32(s) for g in groups for s in g]
    offs = np.zeros(len(groups) + 1, np.uintp)
    offs[1:] = np.cumsum([len(g) for g in groups])
    m = len(flat)
    S = (C.c_void_p * m)(*[_ptr(s) for s in flat])
    L = (C.c_size_t * m)(*[s.size for s in flat])
    OF = (C.c_size_t * (len(groups) + 1))(*[int(x) for x in offs])
    O = (C.c_void_p * len(groups))(*[o.ctypes.data for o in outs]) if outs is not None else None
    counts = np.zeros(len(groups), np.uint64)
    rc = lib().orc_run_svs_groups_algo(algo, len(groups), S, L, OF, O,
                                       counts.ctypes.data_as(C.POINTER(C.c_uint64)), nthreads)
    if rc != 0:
        raise ValueError("orc_run_svs_groups_algo: bad argument")
    return counts


def run_bsr_pairs(pairs, nthreads: int = 1, outs=None, algo: int = 0) -> np.ndarray:
    """BSR pairs [(ba, sa, bb, sb), ...] through branchless_merge_bsr (algo
    0) or galloping_bsr (1) on `nthreads` threads; returns word counts.
    `outs` ([(out_bases, out_states), ...]) materialises."""
    n = len(pairs)
    keep = [tuple(_u32(x) for x in p) for p in pairs]
    P = lambda j: (C.c_void_p * n)(*[_ptr(p[j]) for p in keep])  # noqa: E731
    NA = (C.c_size_t * n)(*[p[0].size for p in keep])
    NB = (C.c_size_t * n)(*[p[2].size for p in keep])
    OB = (C.c_void_p * n)(*[o[0].ctypes.data for o in outs]) if outs is not None else None
    OS = (C.c_void_p * n)(*[o[1].ctypes.data for o in outs]) if outs is not None else None
    words = np.zeros(n, np.uint64)
    rc = lib().orc_run_bsr_pairs(algo, n, P(0), P(1), NA, P(2), P(3), NB, OB, OS,
                                 words.ctypes.data_as(C.POINTER(C.c_uint64)), nthreads)
    if rc != 0:
        raise ValueError("orc_run_bsr_pairs: bad argument")
    return words


# ---- the reference's own C++ kernels (x86 only) ---------------------------

def ref_lib():
    """libref_qfilter.so when built (x86 host with the reference tree), else
    None.  Functions take int* and compare as signed 32-bit."""
    global _ref
    if _ref is None and REF_LIB.exists():
        L = C.CDLL(str(REF_LIB))
        ip = C.c_void_p
        for name in ("intersect_bmiss_uint_b4", "intersect_qfilter_uint_b4_v2",
                     "intersect_qfilter_uint_b4", "intersect_bmiss_uint_sttni_b8"):
            f = getattr(L, name)
            f.restype = C.c_int
            f.argtypes = [ip, C.c_int, ip, C.c_int, ip]
        for name in ("intersect_qfilter_bsr_b4", "intersect_qfilter_bsr_b4_v2"):
            f = getattr(L, name)
            f.restype = C.c_int
            f.argtypes = [ip, ip, C.c_int, ip, ip, C.c_int, ip, ip]
        _ref = L
    return _ref


def ref_two(fn_name: str, a, b) -> np.ndarray:
    L = ref_lib()
    if L is None:
        raise RuntimeError("reference kernels not built (needs x86 and the reference tree)")
    a = np.ascontiguousarray(a, np.int32)
    b = np.ascontiguousarray(b, np.int32)
    # QFilter reads up to one 16-byte block past each input: pad the copies.
    ap = np.zeros(a.size + 16, np.int32)
    bp = np.zeros(b.size + 16, np.int32)
    ap[:a.size], bp[:b.size] = a, b
    out = np.zeros(max(min(a.size, b.size), 1) + 16, np.int32)
    n = getattr(L, fn_name)(ap.ctypes.data, a.size, bp.ctypes.data, b.size, out.ctypes.data)
    return out[:n].view(np.uint32).copy()


def ref_bsr(fn_name: str, ba, sa, bb, sb):
    L = ref_lib()
    if L is None:
        raise RuntimeError("reference kernels not built (needs x86 and the reference tree)")
    arrs = []
    for x in (ba, sa, bb, sb):
        x = np.ascontiguousarray(x, np.int32)
        p = np.zeros(x.size + 16, np.int32)
        p[:x.size] = x
        arrs.append((p, x.size))
    m = max(min(arrs[0][1], arrs[2][1]), 1) + 16
    ob, os_ = np.zeros(m, np.int32), np.zeros(m, np.int32)
    n = getattr(L, fn_name)(arrs[0][0].ctypes.data, arrs[1][0].ctypes.data, arrs[0][1],
                            arrs[2][0].ctypes.data, arrs[3][0].ctypes.data, arrs[2][1],
                            ob.ctypes.data, os_.ctypes.data)
    return ob[:n].view(np.uint32).copy(), os_[:n].view(np.uint32).copy()


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1
