"""GB300-native sorted-u32 set intersection: a drop-in for the hot path of
the Rust crate ``setops`` (UNSW-database/simd_set_operations).

Python mirror of the reference's public interface for that path, over the C
ABI of ``libsetops_gpu.so`` (include/setops_gpu.h):

* ``Intersect2`` functions ``f(set_a, set_b, visitor)``
  (setops/src/intersect.rs:40): ``gpu_auto``, ``gpu_merge``,
  ``gpu_galloping``;
* ``Intersect2C`` functions ``f(set_a, set_b, result) -> int``
  (intersect.rs:41): ``gpu_auto_c``;
* visitors (setops/src/visitor.rs): ``Counter`` (:24), ``VecWriter`` (:51),
  ``SliceWriter`` (:100), ``UnsafeWriter`` (:759);
* runners ``run_2set`` / ``run_2set_c`` / ``run_kset`` / ``run_2set_bsr``
  (intersect.rs:44-90), ``svs_generic`` / ``run_svs``
  (setops/src/intersect/svs.rs:50-116);
* BSR: ``BsrVec`` / ``BsrRef`` (setops/src/bsr.rs:17-163) and ``gpu_bsr``
  (an ``Intersect2Bsr``, bsr.rs:16).

Sets are numpy arrays (host memory; the call copies in and out) or CUDA
tensors (device memory).  Every intersection runs on the GPU; there is no CPU
path, and errors raise ``SetopsError`` instead of the reference's abort.
"""
from __future__ import annotations

import ctypes as C
import threading
import time
from typing import Callable, Sequence

import numpy as np

from . import _lib
from ._lib import (ALGO_AUTO, ALGO_BITMAP, ALGO_GALLOP, ALGO_MERGE, HOST, VARIANT,
                   SetopsError, lib)

__all__ = [
    "Context", "default_context", "SetopsError",
    "Counter", "VecWriter", "SliceWriter", "UnsafeWriter",
    "BsrVec", "BsrRef",
    "gpu_auto", "gpu_merge", "gpu_galloping", "gpu_auto_c", "gpu_bsr",
    "gpu_svs", "gpu_small_adaptive", "intersect", "intersect_count", "intersect_pairs",
    "run_2set", "run_2set_c", "run_kset", "run_2set_bsr",
    "svs_generic", "run_svs", "validate_sorted",
    "ALGO_AUTO", "ALGO_MERGE", "ALGO_GALLOP", "ALGO_BITMAP", "VARIANT", "num_variants",
    "batch_intersect", "batch_count", "batch_intersect_bsr", "batch_count_bsr", "batch_autotune",
    "autotune", "describe_flags", "SIZE_CLASSES",
    "Server",
]


# ---------------------------------------------------------------------------
# context

class Context:
    """Owns one ``setops_ctx`` (stream, scratch pool, policy table)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        rc = lib.setops_gpu_create(C.byref(h), device)
        if rc != 0:
            raise SetopsError(rc, f"setops_gpu_create(device={device}) failed: "
                              f"{_lib.status_string(rc)}")
        self._h = h
        self.device = device

    @property
    def handle(self) -> C.c_void_p:
        if self._h is None:
            raise SetopsError(_lib.ERR_INVALID, "context is closed")
        return self._h

    def check(self, rc: int) -> None:
        if rc != 0:
            msg = lib.setops_gpu_last_error(self.handle).decode()
            raise SetopsError(rc, f"{_lib.status_string(rc)}: {msg}")

    def close(self) -> None:
        if self._h is not None:
            lib.setops_gpu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream) -> None:
        """Use an external CUDA stream (int handle or torch.cuda.Stream)."""
        ptr = getattr(stream, "cuda_stream", stream)
        self.check(lib.setops_gpu_set_stream(self.handle, C.c_void_p(ptr or 0)))

    def synchronize(self) -> None:
        self.check(lib.setops_gpu_synchronize(self.handle))

    @property
    def launch_count(self) -> int:
        return int(lib.setops_gpu_launch_count(self.handle))

    def set_wait_limit_ns(self, ns: int) -> None:
        """Time limit of the kernels' bounded device waits on this context's
        device (0 = the default, 2 s)."""
        self.check(lib.setops_gpu_set_wait_limit_ns(self.handle, int(ns)))

    def check_wait_limit(self) -> tuple[int, int]:
        """Runs one device wait that nothing satisfies; returns (status,
        waited_ns): SETOPS_ERR_TIMEOUT once the limit ended the wait."""
        w = C.c_uint64()
        rc = lib.setops_gpu_check_wait_limit(self.handle, C.byref(w))
        return int(rc), int(w.value)

    def set_policy(self, bsr: bool, ratio_band: int, algo_flags: int) -> None:
        self.check(lib.setops_gpu_set_policy(self.handle, int(bsr), ratio_band, algo_flags))

    def get_policy(self, bsr: bool, ratio_band: int) -> int:
        v = C.c_uint()
        self.check(lib.setops_gpu_get_policy(self.handle, int(bsr), ratio_band, C.byref(v)))
        return v.value

    def get_policy_class(self, bsr: bool, ratio_band: int, size_class: int) -> int:
        v = C.c_uint()
        self.check(lib.setops_gpu_get_policy_class(self.handle, int(bsr), ratio_band, size_class,
                                                   C.byref(v)))
        return v.value

    def set_policy_class(self, bsr: bool, ratio_band: int, size_class: int,
                         algo_flags: int) -> None:
        self.check(lib.setops_gpu_set_policy_class(self.handle, int(bsr), ratio_band, size_class,
                                                   algo_flags))

    def device_key(self) -> str:
        buf = C.create_string_buffer(256)
        self.check(lib.setops_gpu_device_key(self.handle, buf, 256))
        return buf.value.decode()


_default: Context | None = None
_default_lock = threading.Lock()


def default_context() -> Context:
    global _default
    with _default_lock:
        if _default is None:
            _default = Context(0)
        return _default


def num_variants(algo: int, bsr: bool = False) -> int:
    return int(lib.setops_gpu_num_variants(algo, int(bsr)))


# ---------------------------------------------------------------------------
# buffers: numpy (host) or CUDA tensors (device)

def _is_device(x) -> bool:
    return hasattr(x, "__cuda_array_interface__") or (
        hasattr(x, "is_cuda") and bool(getattr(x, "is_cuda")))


def _dev_ptr(x) -> int:
    if hasattr(x, "data_ptr"):
        if x.element_size() != 4 or not x.is_contiguous():
            raise SetopsError(_lib.ERR_INVALID, "device sets must be contiguous 32-bit tensors")
        return int(x.data_ptr())
    iface = x.__cuda_array_interface__
    return int(iface["data"][0])


class _Buf:
    """A set argument: pointer, length, memory space, keep-alive reference."""

    __slots__ = ("ptr", "n", "device", "obj")

    def __init__(self, x):
        if _is_device(x):
            self.obj = x
            self.ptr = _dev_ptr(x)
            self.n = int(x.numel() if hasattr(x, "numel") else len(x))
            self.device = True
        else:
            arr = np.ascontiguousarray(x)
            if arr.dtype != np.uint32:
                if arr.size and (arr.min() < 0 or arr.max() > 0xFFFFFFFF):
                    raise SetopsError(_lib.ERR_INVALID, "set values must fit in u32")
                arr = arr.astype(np.uint32)
            self.obj = arr
            self.ptr = arr.ctypes.data if arr.size else 0
            self.n = int(arr.size)
            self.device = False


def _space(bufs: Sequence[_Buf]) -> int:
    kinds = {b.device for b in bufs if b.n > 0}
    if len(kinds) > 1:
        raise SetopsError(_lib.ERR_INVALID, "mixing host and device sets in one call")
    return 0 if (kinds and kinds.pop()) else HOST


def _empty_like_space(n: int, device: bool, ref=None):
    if device:
        import torch
        dev = ref.device if ref is not None and hasattr(ref, "device") else "cuda"
        return torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    return np.empty(max(n, 1), dtype=np.uint32)


def _to_host(x, n: int) -> np.ndarray:
    if hasattr(x, "cpu"):
        return x[:n].cpu().numpy().view(np.uint32).copy()
    return np.asarray(x[:n], dtype=np.uint32).copy()


# ---------------------------------------------------------------------------
# visitors (setops/src/visitor.rs)

class Counter:
    """Counts intersection size without storing it (visitor.rs:24-49).  For
    BSR results it counts elements: sum of popcount(state) (visitor.rs:399)."""

    def __init__(self):
        self._count = 0

    def visit(self, value) -> None:
        self._count += 1

    def count(self) -> int:
        return self._count

    def clear(self) -> None:
        self._count = 0


class VecWriter:
    """Stores the result in a growable vector (visitor.rs:51-98)."""

    def __init__(self, capacity: int = 0):
        self._items = np.empty(0, dtype=np.uint32)

    def visit(self, value) -> None:
        self._items = np.append(self._items, np.uint32(value))

    def _extend(self, arr: np.ndarray) -> None:
        self._items = arr if self._items.size == 0 else np.concatenate([self._items, arr])

    def clear(self) -> None:
        self._items = np.empty(0, dtype=np.uint32)

    def as_array(self) -> np.ndarray:
        return self._items

    def into(self) -> np.ndarray:
        return self._items

    def __len__(self) -> int:
        return int(self._items.size)


class SliceWriter:
    """Writes the result into a caller-provided buffer (visitor.rs:100-130)."""

    def __init__(self, data):
        self.data = data
        self._pos = 0

    def visit(self, value) -> None:
        self.data[self._pos] = value
        self._pos += 1

    def _extend(self, arr: np.ndarray) -> None:
        n = int(arr.size)
        if self._pos + n > len(self.data):
            raise SetopsError(_lib.ERR_CAPACITY, "SliceWriter capacity exceeded")
        self.data[self._pos:self._pos + n] = arr
        self._pos += n

    def position(self) -> int:
        return self._pos

    def clear(self) -> None:
        self._pos = 0

    def as_array(self) -> np.ndarray:
        return np.asarray(self.data[:self._pos], dtype=np.uint32)


class UnsafeWriter(SliceWriter):
    """Preallocated writer used by the reference's benchmark
    (visitor.rs:759-778): capacity fixed up front."""

    def __init__(self, capacity: int):
        super().__init__(np.empty(max(capacity, 0), dtype=np.uint32))

    @classmethod
    def with_capacity(cls, capacity: int) -> "UnsafeWriter":
        return cls(capacity)

    def into(self) -> np.ndarray:
        return self.as_array().copy()


# ---------------------------------------------------------------------------
# batched pairs (many pairs, one launch)

def _u64(x) -> np.ndarray:
    return np.ascontiguousarray(x, dtype=np.uint64)


def batch_intersect(pool, a_off, a_len, b_off, b_len, *, ctx: Context | None = None):
    """Intersects every pair of a batch in one launch (host arrays).  Pair p
    is pool[a_off[p]:+a_len[p]] and pool[b_off[p]:+b_len[p]].  Returns
    (out, out_off, out_lens): pair p's ascending intersection is
    out[out_off[p]:out_off[p] + out_lens[p]]."""
    ctx = ctx or default_context()
    pool = np.ascontiguousarray(pool, dtype=np.uint32)
    a_off, a_len, b_off, b_len = _u64(a_off), _u64(a_len), _u64(b_off), _u64(b_len)
    n = a_len.size
    caps = np.minimum(a_len, b_len)
    out_off = np.zeros(n, np.uint64)
    if n:
        out_off[1:] = np.cumsum(caps[:-1])
    out = np.empty(max(int(caps.sum()), 1), np.uint32)
    lens = np.zeros(n, np.uint64)
    ctx.check(lib.setops_gpu_batch_intersect(
        ctx.handle, pool.ctypes.data, pool.size, a_off.ctypes.data, a_len.ctypes.data,
        b_off.ctypes.data, b_len.ctypes.data, n, out.ctypes.data, out.size,
        out_off.ctypes.data, lens.ctypes.data, HOST))
    return out, out_off, lens


def batch_count(pool, a_off, a_len, b_off, b_len, *, ctx: Context | None = None) -> np.ndarray:
    """Per-pair |A ∩ B| of a batch in one launch (host arrays)."""
    ctx = ctx or default_context()
    pool = np.ascontiguousarray(pool, dtype=np.uint32)
    a_off, a_len, b_off, b_len = _u64(a_off), _u64(a_len), _u64(b_off), _u64(b_len)
    counts = np.zeros(a_len.size, np.uint64)
    ctx.check(lib.setops_gpu_batch_count(
        ctx.handle, pool.ctypes.data, pool.size, a_off.ctypes.data, a_len.ctypes.data,
        b_off.ctypes.data, b_len.ctypes.data, a_len.size, counts.ctypes.data, HOST))
    return counts


def batch_intersect_bsr(bases, states, a_off, a_len, b_off, b_len, *,
                        ctx: Context | None = None):
    """Intersects every BSR pair of a batch in one launch (host arrays): pair
    p is words [a_off[p], +a_len[p]) and [b_off[p], +b_len[p]) of (bases,
    states).  Returns (out_bases, out_states, out_off, out_lens)."""
    ctx = ctx or default_context()
    bases = np.ascontiguousarray(bases, dtype=np.uint32)
    states = np.ascontiguousarray(states, dtype=np.uint32)
    a_off, a_len, b_off, b_len = _u64(a_off), _u64(a_len), _u64(b_off), _u64(b_len)
    n = a_len.size
    caps = np.minimum(a_len, b_len)
    out_off = np.zeros(n, np.uint64)
    if n:
        out_off[1:] = np.cumsum(caps[:-1])
    cap = max(int(caps.sum()), 1)
    ob, os_ = np.empty(cap, np.uint32), np.empty(cap, np.uint32)
    lens = np.zeros(n, np.uint64)
    ctx.check(lib.setops_gpu_batch_intersect_bsr(
        ctx.handle, bases.ctypes.data, states.ctypes.data, bases.size, a_off.ctypes.data,
        a_len.ctypes.data, b_off.ctypes.data, b_len.ctypes.data, n, ob.ctypes.data,
        os_.ctypes.data, cap, out_off.ctypes.data, lens.ctypes.data, HOST))
    return ob, os_, out_off, lens


def batch_count_bsr(bases, states, a_off, a_len, b_off, b_len, *,
                    ctx: Context | None = None) -> np.ndarray:
    """Per-pair element counts (popcount sums) of a BSR batch in one launch."""
    ctx = ctx or default_context()
    bases = np.ascontiguousarray(bases, dtype=np.uint32)
    states = np.ascontiguousarray(states, dtype=np.uint32)
    a_off, a_len, b_off, b_len = _u64(a_off), _u64(a_len), _u64(b_off), _u64(b_len)
    counts = np.zeros(a_len.size, np.uint64)
    ctx.check(lib.setops_gpu_batch_count_bsr(
        ctx.handle, bases.ctypes.data, states.ctypes.data, bases.size, a_off.ctypes.data,
        a_len.ctypes.data, b_off.ctypes.data, b_len.ctypes.data, a_len.size,
        counts.ctypes.data, HOST))
    return counts


def batch_autotune(pool, a_off, a_len, b_off, b_len, *, reps: int = 3,
                   ctx: Context | None = None) -> tuple[int, int]:
    """Times the batch kernel shapes and search ratios on a sample batch and
    keeps the fastest as the context's batch policy; returns it."""
    ctx = ctx or default_context()
    pool = np.ascontiguousarray(pool, dtype=np.uint32)
    a_off, a_len, b_off, b_len = _u64(a_off), _u64(a_len), _u64(b_off), _u64(b_len)
    ctx.check(lib.setops_gpu_batch_autotune(
        ctx.handle, pool.ctypes.data, pool.size, a_off.ctypes.data, a_len.ctypes.data,
        b_off.ctypes.data, b_len.ctypes.data, a_len.size, reps, HOST))
    v, r = C.c_int(), C.c_uint32()
    ctx.check(lib.setops_gpu_batch_get_policy(ctx.handle, C.byref(v), C.byref(r)))
    return int(v.value), int(r.value)


SIZE_CLASSES = 4  # SETOPS_SIZE_CLASSES: smaller input < 2^12, < 2^16, < 2^22, larger


def autotune(*, band_lo: int = 0, band_hi: int = 16, max_elems: int = 1 << 25,
             density: float = 0.05, reps: int = 3, bsr: bool = True, cache: str | None = None,
             ctx: Context | None = None) -> dict:
    """Fills the context's policy tables (algorithm and kernel variant per
    size-ratio band and size class) by timing every candidate on generated
    pairs -- the array table (setops_gpu_autotune) and, with `bsr`, the BSR
    table (setops_gpu_autotune_bsr) -- and returns them.  With `cache` (a
    JSON file), tables saved there for the same GPU, driver and tuning
    arguments are applied instead of tuning, and new ones are saved."""
    import json
    import os
    ctx = ctx or default_context()
    key = {"device": ctx.device_key(), "band_lo": band_lo, "band_hi": band_hi,
           "max_elems": int(max_elems), "density": float(density), "bsr": bool(bsr)}
    if cache and os.path.exists(cache):
        try:
            saved = json.load(open(cache))
        except (OSError, ValueError):
            saved = None
        if saved and saved.get("key") == key:
            for name, is_bsr in (("cells", False), ("bsr_cells", True)):
                for cell, flags in saved.get(name, {}).items():
                    band, cls = (int(x) for x in cell.split(","))
                    ctx.set_policy_class(is_bsr, band, cls, int(flags))
            return dict(saved, from_cache=True)
    n = C.c_int()
    ctx.check(lib.setops_gpu_autotune(ctx.handle, band_lo, band_hi, int(max_elems),
                                      float(density), reps, C.byref(n)))
    cells = {f"{b},{c}": ctx.get_policy_class(False, b, c)
             for b in range(band_lo, band_hi + 1) for c in range(SIZE_CLASSES)}
    table = {"key": key, "tuned_cells": int(n.value), "cells": cells, "from_cache": False}
    if bsr:
        nb = C.c_int()
        ctx.check(lib.setops_gpu_autotune_bsr(ctx.handle, band_lo, band_hi, int(max_elems),
                                              float(density), reps, C.byref(nb)))
        table["bsr_tuned_cells"] = int(nb.value)
        table["bsr_cells"] = {f"{b},{c}": ctx.get_policy_class(True, b, c)
                              for b in range(band_lo, band_hi + 1) for c in range(SIZE_CLASSES)}
    if cache:
        with open(cache, "w") as f:
            json.dump(table, f, indent=1)
    return table


def describe_flags(flags: int) -> str:
    """'bitmap/8', 'gallop/3', ... for a policy entry."""
    names = {ALGO_MERGE: "merge", ALGO_GALLOP: "gallop", ALGO_BITMAP: "bitmap"}
    return f"{names.get(flags & 0xFF00, '?')}/{(flags >> 16) & 0xFF}"


# ---------------------------------------------------------------------------
# serving k-set queries against a resident index

class Server:
    """A query server over a posting-list index (setops_srv_*): queries of
    k list ids, answered by their ascending intersection, batched on the GPU
    as they arrive."""

    def __init__(self, pool, offs, lens, *, budget: int = 0, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self._pool = np.ascontiguousarray(pool, dtype=np.uint32)
        self._offs = np.ascontiguousarray(offs, dtype=np.uint64)
        self._lens = np.ascontiguousarray(lens, dtype=np.uint64)
        h = C.c_void_p()
        self.ctx.check(lib.setops_srv_start(
            self.ctx.handle, self._pool.ctypes.data, self._pool.size, self._offs.ctypes.data,
            self._lens.ctypes.data, self._lens.size, budget, HOST, C.byref(h)))
        self._h = h
        self._buf = np.empty(1 << 16, np.uint32)
        self._early = {}  # results polled while waiting for another tag

    def submit(self, list_ids, tag: int) -> None:
        ids = np.ascontiguousarray(list_ids, dtype=np.uint32)
        rc = lib.setops_srv_submit(self._h, ids.ctypes.data, ids.size, tag)
        if rc != 0:
            raise SetopsError(rc, _lib.status_string(rc))

    def poll(self):
        """(tag, answer, latency_ns) of one finished query, or None."""
        tag, n, lat = C.c_uint64(), C.c_size_t(), C.c_uint64()
        while True:
            rc = lib.setops_srv_poll(self._h, C.byref(tag), self._buf.ctypes.data,
                                     self._buf.size, C.byref(n), C.byref(lat))
            if rc == _lib.ERR_CAPACITY:
                self._buf = np.empty(max(int(n.value), 2 * self._buf.size), np.uint32)
                continue
            if rc == _lib.ERR_NOT_READY:
                return None
            if rc != 0:
                raise SetopsError(rc, _lib.status_string(rc))
            return int(tag.value), self._buf[:int(n.value)].copy(), int(lat.value)

    def wait(self, tag: int):
        """Polls until the query `tag` is done (other results are kept)."""
        while True:
            if tag in self._early:
                return self._early.pop(tag)
            r = self.poll()
            if r is None:
                time.sleep(0)
                continue
            if r[0] == tag:
                return r
            self._early[r[0]] = r

    def stats(self) -> dict:
        v = [C.c_uint64() for _ in range(4)]
        self.ctx.check(lib.setops_srv_stats(self._h, *[C.byref(x) for x in v]))
        return dict(zip(("batches", "queries", "max_batch", "launches"), (x.value for x in v)))

    def run_load(self, ids, ks, rate_qps: float, seed: int = 1, answer_stride: int = 0):
        """Open-loop Poisson load; returns (latency_ns[nq], counts[nq],
        elapsed_s), and with answer_stride > 0 also the answers themselves
        (a list of arrays; each answer at most answer_stride long)."""
        ids = np.ascontiguousarray(ids, dtype=np.uint32)
        ks = np.ascontiguousarray(ks, dtype=np.uint32)
        nq = ks.size
        lat = np.zeros(nq, np.uint64)
        cnt = np.zeros(nq, np.uint64)
        ans = np.zeros((nq, answer_stride), np.uint32) if answer_stride > 0 else None
        el = C.c_double()
        rc = lib.setops_srv_run_load(self._h, ids.ctypes.data, ks.ctypes.data, ids.shape[1], nq,
                                     rate_qps, seed, lat.ctypes.data, cnt.ctypes.data,
                                     ans.ctypes.data if ans is not None else None,
                                     answer_stride, C.byref(el))
        if rc != 0:
            raise SetopsError(rc, _lib.status_string(rc))
        if ans is None:
            return lat, cnt, float(el.value)
        return lat, cnt, float(el.value), [ans[q, :int(cnt[q])] for q in range(nq)]

    def stop(self) -> None:
        if self._h is not None:
            rc = lib.setops_srv_stop(self._h)
            self._h = None
            if rc != 0:
                raise SetopsError(rc, _lib.status_string(rc))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.stop()


# ---------------------------------------------------------------------------
# 2-set u32

def intersect_count(set_a, set_b, *, algo: int = ALGO_AUTO,
                    ctx: Context | None = None) -> int:
    """|A ∩ B| on the GPU (the Counter visitor)."""
    ctx = ctx or default_context()
    a, b = _Buf(set_a), _Buf(set_b)
    flags = _space([a, b]) | algo
    c = C.c_uint64()
    ctx.check(lib.setops_gpu_intersect_count(ctx.handle, a.ptr, a.n, b.ptr, b.n,
                                             C.byref(c), flags))
    return int(c.value)


def intersect(set_a, set_b, out=None, *, algo: int = ALGO_AUTO,
              ctx: Context | None = None):
    """A ∩ B, ascending, on the GPU.  Returns (out, length); `out` is
    allocated in the inputs' memory space when not given (capacity must be
    >= min(|A|, |B|))."""
    ctx = ctx or default_context()
    a, b = _Buf(set_a), _Buf(set_b)
    flags = _space([a, b]) | algo
    mn = min(a.n, b.n)
    device = not (flags & HOST)
    if out is None:
        out = _empty_like_space(mn, device, set_a if device else None)
    o = _Buf(out) if device else None
    if not device:
        if not (isinstance(out, np.ndarray) and out.dtype == np.uint32 and out.flags.c_contiguous):
            raise SetopsError(_lib.ERR_INVALID, "host output must be a contiguous uint32 array")
        optr, ocap = out.ctypes.data, out.size
    else:
        optr, ocap = o.ptr, o.n
    n = C.c_size_t()
    ctx.check(lib.setops_gpu_intersect(ctx.handle, a.ptr, a.n, b.ptr, b.n, optr, ocap,
                                       C.byref(n), flags))
    return out, int(n.value)


def intersect_pairs(pairs, outs=None, *, algo: int = ALGO_AUTO,
                    ctx: Context | None = None):
    """A ∩ B for many independent pairs of host arrays in one call
    (setops_gpu_intersect_pairs): returns [(out, length)], each what
    intersect() gives for that pair.  `outs` are host uint32 arrays of
    capacity >= min(|A|, |B|) (allocated when not given); pinned inputs and
    outputs let search-band pairs be read in place while the other pairs'
    inputs are copied."""
    ctx = ctx or default_context()
    bufs = [(_Buf(x), _Buf(y)) for x, y in pairs]
    for a, b in bufs:
        if a.device or b.device:
            raise SetopsError(_lib.ERR_INVALID, "intersect_pairs takes host arrays")
    n = len(bufs)
    if outs is None:
        outs = [np.empty(max(min(a.n, b.n), 1), np.uint32) for a, b in bufs]
    for o in outs:
        if not (isinstance(o, np.ndarray) and o.dtype == np.uint32 and o.flags.c_contiguous):
            raise SetopsError(_lib.ERR_INVALID, "host output must be a contiguous uint32 array")
    P = C.c_void_p * max(n, 1)
    S = C.c_size_t * max(n, 1)
    pa, pb = P(*[a.ptr for a, _ in bufs]), P(*[b.ptr for _, b in bufs])
    la, lb = S(*[a.n for a, _ in bufs]), S(*[b.n for _, b in bufs])
    po, co = P(*[o.ctypes.data for o in outs]), S(*[o.size for o in outs])
    lens = S()
    ctx.check(lib.setops_gpu_intersect_pairs(ctx.handle, n, pa, la, pb, lb, po, co, lens,
                                             HOST | algo))
    return [(outs[i], int(lens[i])) for i in range(n)]


def _run_visitor(set_a, set_b, visitor, algo: int, ctx: Context | None) -> None:
    if isinstance(visitor, Counter):
        visitor._count += intersect_count(set_a, set_b, algo=algo, ctx=ctx)
        return
    out, n = intersect(set_a, set_b, algo=algo, ctx=ctx)
    visitor._extend(_to_host(out, n))


def gpu_auto(set_a, set_b, visitor, *, ctx: Context | None = None) -> None:
    """``Intersect2``: the tuned kernel for the pair's size ratio."""
    _run_visitor(set_a, set_b, visitor, ALGO_AUTO, ctx)


def gpu_merge(set_a, set_b, visitor, *, variant: int = 0,
              ctx: Context | None = None) -> None:
    """``Intersect2``: the merge-path kernel (naive_merge semantics)."""
    _run_visitor(set_a, set_b, visitor, ALGO_MERGE | VARIANT(variant), ctx)


def gpu_galloping(set_a, set_b, visitor, *, variant: int = 0,
                  ctx: Context | None = None) -> None:
    """``Intersect2``: the search kernel (galloping semantics)."""
    _run_visitor(set_a, set_b, visitor, ALGO_GALLOP | VARIANT(variant), ctx)


def gpu_auto_c(set_a, set_b, result, *, ctx: Context | None = None) -> int:
    """``Intersect2C``: writes into `result` (capacity >= min(|A|, |B|)) and
    returns the length."""
    _, n = intersect(set_a, set_b, out=result, ctx=ctx)
    return n


def run_2set(set_a, set_b, intersect_fn: Callable = gpu_auto) -> np.ndarray:
    """intersect.rs:44-52."""
    w = VecWriter()
    intersect_fn(set_a, set_b, w)
    return w.into()


def run_2set_c(set_a, set_b, intersect_fn: Callable = gpu_auto_c) -> np.ndarray:
    """intersect.rs:54-68: result buffer of capacity min(|A|, |B|)."""
    n = min(len(set_a), len(set_b))
    result = np.zeros(n, dtype=np.uint32)
    m = intersect_fn(set_a, set_b, result)
    return result[:m]


# ---------------------------------------------------------------------------
# k-set

_ALGO_OF = {}


def _algo_of(fn) -> int:
    return _ALGO_OF.get(fn, ALGO_AUTO)


def _svs(sets, out=None, count_only=False, algo=ALGO_AUTO, ctx=None, adaptive=False):
    ctx = ctx or default_context()
    bufs = [_Buf(s) for s in sets]
    flags = _space(bufs) | algo
    k = len(bufs)
    ptrs = (C.c_void_p * k)(*[b.ptr for b in bufs])
    lens = (C.c_size_t * k)(*[b.n for b in bufs])
    if count_only:
        c = C.c_uint64()
        fn = lib.setops_gpu_adaptive_count if adaptive else lib.setops_gpu_svs_count
        ctx.check(fn(ctx.handle, ptrs, lens, k, C.byref(c), flags))
        return int(c.value)
    mn = min((b.n for b in bufs), default=0)
    device = not (flags & HOST)
    if out is None:
        out = _empty_like_space(mn, device, sets[0] if device else None)
    optr = _Buf(out).ptr if device else out.ctypes.data
    ocap = (out.numel() if device and hasattr(out, "numel") else len(out))
    n = C.c_size_t()
    fn = lib.setops_gpu_adaptive if adaptive else lib.setops_gpu_svs
    ctx.check(fn(ctx.handle, ptrs, lens, k, optr, ocap, C.byref(n), flags))
    return out, int(n.value)


def gpu_small_adaptive(sets, visitor, *, ctx: Context | None = None) -> None:
    """``IntersectK`` by the small_adaptive scheme
    (setops/src/intersect/adaptive.rs:107-148): each element of the smallest
    set looked up in the others, smallest first, dropped at the first set
    that lacks it.  Same result as gpu_svs."""
    if len(sets) < 2:
        raise SetopsError(_lib.ERR_INVALID, "k-set intersection needs >= 2 sets")
    if isinstance(visitor, Counter):
        visitor._count += _svs(sets, count_only=True, ctx=ctx, adaptive=True)
        return
    out, n = _svs(sets, ctx=ctx, adaptive=True)
    visitor._extend(_to_host(out, n))


def gpu_svs(sets, visitor, *, ctx: Context | None = None) -> None:
    """``IntersectK`` (intersect.rs:42): device SvS with intermediates kept in
    HBM."""
    if len(sets) < 2:
        raise SetopsError(_lib.ERR_INVALID, "k-set intersection needs >= 2 sets")
    if isinstance(visitor, Counter):
        visitor._count += _svs(sets, count_only=True, ctx=ctx)
        return
    out, n = _svs(sets, ctx=ctx)
    visitor._extend(_to_host(out, n))


def svs_generic(sets, left, right, intersect_fn: Callable = gpu_auto, *,
                ctx: Context | None = None):
    """svs.rs:50-73.  The reference ping-pongs the two visitors on the CPU;
    here the intermediates live in device buffers and the final result is
    written to `left`, which is returned (`right` is left untouched)."""
    if len(sets) < 2:
        raise SetopsError(_lib.ERR_INVALID, "svs_generic needs >= 2 sets")
    if hasattr(left, "clear"):
        left.clear()
    algo = _algo_of(intersect_fn)
    if isinstance(left, Counter):
        left._count += _svs(sets, count_only=True, algo=algo, ctx=ctx)
        return left
    out, n = _svs(sets, algo=algo, ctx=ctx)
    left._extend(_to_host(out, n))
    return left


def run_svs(sets, intersect_fn: Callable = gpu_auto) -> np.ndarray:
    """svs.rs:103-116."""
    left, right = VecWriter(), VecWriter()
    return svs_generic(sets, left, right, intersect_fn).into()


def run_kset(sets, intersect_k: Callable = gpu_svs) -> np.ndarray:
    """intersect.rs:70-80."""
    if len(sets) < 2:
        raise SetopsError(_lib.ERR_INVALID, "run_kset needs >= 2 sets")
    w = VecWriter()
    intersect_k(sets, w)
    return w.into()


_ALGO_OF.update({gpu_auto: ALGO_AUTO, gpu_merge: ALGO_MERGE,
                 gpu_galloping: ALGO_GALLOP})


# ---------------------------------------------------------------------------
# BSR

class BsrRef:
    """Borrowed (bases, states) pair (bsr.rs:17-46)."""

    def __init__(self, bases, states):
        if len(bases) != len(states):
            raise SetopsError(_lib.ERR_INVALID, "bases and states differ in length")
        self.bases = bases
        self.states = states

    def __len__(self) -> int:
        return len(self.bases)


class BsrVec:
    """Owned BSR set (bsr.rs:49-110): bases strictly increasing, states
    non-zero 32-bit bitmaps; element = base << 5 | bit."""

    def __init__(self, bases=None, states=None):
        self.bases = np.asarray(bases if bases is not None else [], dtype=np.uint32)
        self.states = np.asarray(states if states is not None else [], dtype=np.uint32)

    @classmethod
    def from_sorted(cls, sorted_set, *, ctx: Context | None = None) -> "BsrVec":
        """bsr.rs:140-163, encoded on the GPU."""
        ctx = ctx or default_context()
        s = _Buf(sorted_set)
        if s.device:
            raise SetopsError(_lib.ERR_INVALID, "BsrVec holds host arrays")
        bases = np.empty(max(s.n, 1), np.uint32)
        states = np.empty(max(s.n, 1), np.uint32)
        w = C.c_size_t()
        ctx.check(lib.setops_gpu_bsr_from_sorted(ctx.handle, s.ptr, s.n, bases.ctypes.data,
                                                 states.ctypes.data, C.byref(w), HOST))
        return cls(bases[:w.value].copy(), states[:w.value].copy())

    def to_sorted_set(self, *, ctx: Context | None = None) -> np.ndarray:
        """bsr.rs:77-88, decoded on the GPU."""
        ctx = ctx or default_context()
        n = len(self.bases)
        states = np.ascontiguousarray(self.states, dtype=np.uint32)
        cap = int(np.unpackbits(states.view(np.uint8)).sum()) if n else 0
        out = np.empty(max(cap, 1), np.uint32)
        m = C.c_size_t()
        b = np.ascontiguousarray(self.bases)
        s = np.ascontiguousarray(self.states)
        ctx.check(lib.setops_gpu_bsr_to_sorted(ctx.handle, b.ctypes.data, s.ctypes.data, n,
                                               out.ctypes.data, cap, C.byref(m), HOST))
        return out[:m.value].copy()

    def bsr_ref(self) -> BsrRef:
        return BsrRef(self.bases, self.states)

    def append(self, base: int, state: int) -> None:
        self.bases = np.append(self.bases, np.uint32(base))
        self.states = np.append(self.states, np.uint32(state))

    def _extend(self, bases: np.ndarray, states: np.ndarray) -> None:
        self.bases = np.concatenate([self.bases, bases])
        self.states = np.concatenate([self.states, states])

    def clear(self) -> None:
        self.bases = np.empty(0, np.uint32)
        self.states = np.empty(0, np.uint32)

    def __len__(self) -> int:
        return int(self.bases.size)

    def __eq__(self, other) -> bool:
        return (isinstance(other, BsrVec) and np.array_equal(self.bases, other.bases)
                and np.array_equal(self.states, other.states))


def gpu_bsr(set_a: BsrRef, set_b: BsrRef, visitor, *, algo: int = ALGO_AUTO,
            ctx: Context | None = None) -> None:
    """``Intersect2Bsr`` (bsr.rs:16) with branchless_merge_bsr semantics
    (merge.rs:62-87).  visitor: BsrVec (materialise) or Counter (elements)."""
    ctx = ctx or default_context()
    ba, sa, bb, sb = (_Buf(x) for x in (set_a.bases, set_a.states, set_b.bases, set_b.states))
    flags = _space([ba, sa, bb, sb]) | algo
    if isinstance(visitor, Counter):
        c = C.c_uint64()
        ctx.check(lib.setops_gpu_intersect_bsr_count(ctx.handle, ba.ptr, sa.ptr, ba.n,
                                                     bb.ptr, sb.ptr, bb.n, C.byref(c), flags))
        visitor._count += int(c.value)
        return
    mn = min(ba.n, bb.n)
    device = not (flags & HOST)
    ob = _empty_like_space(mn, device, set_a.bases if device else None)
    os_ = _empty_like_space(mn, device, set_a.bases if device else None)
    optr_b = _Buf(ob).ptr if device else ob.ctypes.data
    optr_s = _Buf(os_).ptr if device else os_.ctypes.data
    n = C.c_size_t()
    ctx.check(lib.setops_gpu_intersect_bsr(ctx.handle, ba.ptr, sa.ptr, ba.n, bb.ptr, sb.ptr,
                                           bb.n, optr_b, optr_s, mn, C.byref(n), flags))
    visitor._extend(_to_host(ob, n.value), _to_host(os_, n.value))


def run_2set_bsr(set_a: BsrRef, set_b: BsrRef, intersect_fn: Callable = gpu_bsr) -> BsrVec:
    """intersect.rs:82-90."""
    w = BsrVec()
    intersect_fn(set_a, set_b, w)
    return w


def validate_sorted(arr, *, ctx: Context | None = None) -> bool:
    """True when `arr` is strictly increasing (checked on the GPU)."""
    ctx = ctx or default_context()
    b = _Buf(arr)
    ok = C.c_int()
    ctx.check(lib.setops_gpu_validate_sorted(ctx.handle, b.ptr, b.n, C.byref(ok),
                                             _space([b])))
    return bool(ok.value)
