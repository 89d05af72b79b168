"""ctypes binding of libsetops_gpu.so (include/setops_gpu.h, setops_bench.h).

There is no CPU fallback: if the library is missing, importing this module
raises ImportError telling how to build it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from .datasets import GEN_SIGNATURES

LIB_PATH = Path(__file__).resolve().parent / "libsetops_gpu.so"

OK = 0
ERR_INVALID = -1
ERR_CAPACITY = -2
ERR_CUDA = -3
ERR_NOMEM = -4
ERR_TIMEOUT = -5
ERR_UNSORTED = -6
ERR_BUSY = -7
ERR_TOO_LARGE = -8
ERR_NOT_READY = -9

HOST = 0x1
ALGO_SHIFT = 8
ALGO_AUTO = 0 << ALGO_SHIFT
ALGO_MERGE = 1 << ALGO_SHIFT
ALGO_GALLOP = 2 << ALGO_SHIFT
ALGO_BITMAP = 3 << ALGO_SHIFT
VARIANT_SHIFT = 16


def VARIANT(v: int) -> int:
    return (v & 0xFF) << VARIANT_SHIFT


u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
szp = C.POINTER(C.c_size_t)
vp = C.c_void_p
sz = C.c_size_t
u64 = C.c_uint64
uint = C.c_uint


def _load() -> C.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build it with "
            "`python simd_set_operations_gb300/build.py` (needs nvcc); "
            "this package has no CPU fallback")
    return C.CDLL(str(LIB_PATH))


lib = _load()

# (name, restype, argtypes) -- every symbol declared in include/*.h
SIGNATURES = [
    ("setops_status_string", C.c_char_p, [C.c_int]),
    ("setops_gpu_create", C.c_int, [C.POINTER(vp), C.c_int]),
    ("setops_gpu_destroy", C.c_int, [vp]),
    ("setops_gpu_set_stream", C.c_int, [vp, vp]),
    ("setops_gpu_get_stream", vp, [vp]),
    ("setops_gpu_synchronize", C.c_int, [vp]),
    ("setops_gpu_last_error", C.c_char_p, [vp]),
    ("setops_gpu_num_variants", C.c_int, [uint, C.c_int]),
    ("setops_gpu_launch_count", u64, [vp]),
    ("setops_gpu_set_wait_limit_ns", C.c_int, [vp, u64]),
    ("setops_gpu_check_wait_limit", C.c_int, [vp, u64p]),
    ("setops_gpu_set_policy", C.c_int, [vp, C.c_int, C.c_int, uint]),
    ("setops_gpu_get_policy", C.c_int, [vp, C.c_int, C.c_int, C.POINTER(uint)]),
    ("setops_gpu_set_policy_class", C.c_int, [vp, C.c_int, C.c_int, C.c_int, uint]),
    ("setops_gpu_get_policy_class", C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.POINTER(uint)]),
    ("setops_gpu_autotune", C.c_int, [vp, C.c_int, C.c_int, sz, C.c_double, C.c_int,
                                      C.POINTER(C.c_int)]),
    ("setops_gpu_autotune_bsr", C.c_int, [vp, C.c_int, C.c_int, sz, C.c_double, C.c_int,
                                      C.POINTER(C.c_int)]),
    ("setops_gpu_device_key", C.c_int, [vp, C.c_char_p, sz]),
    ("setops_gpu_intersect_count", C.c_int, [vp, vp, sz, vp, sz, u64p, uint]),
    ("setops_gpu_intersect", C.c_int, [vp, vp, sz, vp, sz, vp, sz, szp, uint]),
    ("setops_gpu_intersect_async", C.c_int, [vp, vp, sz, vp, sz, vp, sz, vp, uint]),
    ("setops_gpu_intersect_pairs", C.c_int, [vp, sz, vp, vp, vp, vp, vp, vp, vp, uint]),
    ("setops_gpu_intersect_bsr_count", C.c_int, [vp, vp, vp, sz, vp, vp, sz, u64p, uint]),
    ("setops_gpu_intersect_bsr", C.c_int, [vp, vp, vp, sz, vp, vp, sz, vp, vp, sz, szp, uint]),
    ("setops_gpu_bsr_from_sorted", C.c_int, [vp, vp, sz, vp, vp, szp, uint]),
    ("setops_gpu_bsr_to_sorted", C.c_int, [vp, vp, vp, sz, vp, sz, szp, uint]),
    ("setops_gpu_svs", C.c_int, [vp, C.POINTER(vp), szp, sz, vp, sz, szp, uint]),
    ("setops_gpu_svs_count", C.c_int, [vp, C.POINTER(vp), szp, sz, u64p, uint]),
    ("setops_gpu_svs_async", C.c_int, [vp, C.POINTER(vp), szp, sz, vp, sz, vp, uint]),
    ("setops_gpu_adaptive", C.c_int, [vp, C.POINTER(vp), szp, sz, vp, sz, szp, uint]),
    ("setops_gpu_adaptive_count", C.c_int, [vp, C.POINTER(vp), szp, sz, u64p, uint]),
    ("setops_gpu_validate_sorted", C.c_int, [vp, vp, sz, C.POINTER(C.c_int), uint]),
    ("setops_gpu_intersect_noalloc", C.c_int, [vp, sz, vp, sz, vp, sz, szp, vp]),
    ("setops_gpu_batch_intersect", C.c_int, [vp, vp, sz, vp, vp, vp, vp, sz, vp, sz, vp, vp, uint]),
    ("setops_gpu_batch_count", C.c_int, [vp, vp, sz, vp, vp, vp, vp, sz, vp, uint]),
    ("setops_gpu_batch_intersect_bsr", C.c_int,
     [vp, vp, vp, sz, vp, vp, vp, vp, sz, vp, vp, sz, vp, vp, uint]),
    ("setops_gpu_batch_count_bsr", C.c_int, [vp, vp, vp, sz, vp, vp, vp, vp, sz, vp, uint]),
    ("setops_gpu_batch_plan_create", C.c_int, [vp, vp, sz, vp, vp, vp, vp, sz, vp, sz, vp, vp, vp]),
    ("setops_gpu_batch_plan_launch", C.c_int, [vp]),
    ("setops_gpu_batch_plan_destroy", C.c_int, [vp]),
    ("setops_gpu_batch_set_policy", C.c_int, [vp, C.c_int, C.c_uint32]),
    ("setops_gpu_batch_get_policy", C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_uint32)]),
    ("setops_gpu_batch_num_variants", C.c_int, []),
    ("setops_gpu_batch_autotune", C.c_int, [vp, vp, sz, vp, vp, vp, vp, sz, C.c_int, uint]),
    ("setops_srv_start", C.c_int, [vp, vp, sz, vp, vp, sz, sz, uint, C.POINTER(vp)]),
    ("setops_srv_submit", C.c_int, [vp, vp, sz, u64]),
    ("setops_srv_poll", C.c_int, [vp, u64p, vp, sz, szp, u64p]),
    ("setops_srv_stats", C.c_int, [vp, u64p, u64p, u64p, u64p]),
    ("setops_srv_stop", C.c_int, [vp]),
    # setops_bench.h (the generators and datafile functions are listed in datasets.py)
    ("setops_srv_run_load", C.c_int, [vp, vp, vp, sz, sz, C.c_double, u64, vp, vp, vp, sz,
                                      C.POINTER(C.c_double)]),
    ("setops_bench_pairs_one_by_one", C.c_int, [vp, vp, vp, vp, vp, vp, sz, vp, vp, vp,
                                                C.POINTER(C.c_double)]),
    ("setops_bench_bsr_pairs_one_by_one", C.c_int, [vp, vp, vp, vp, vp, vp, vp, sz, vp, vp, vp,
                                                    vp, C.POINTER(C.c_double)]),
    ("setops_bench_record_event", C.c_int, [vp, vp]),
    ("setops_bench_queries_one_by_one", C.c_int, [vp, vp, vp, vp, vp, vp, sz, sz, vp, sz, vp,
                                                  vp, C.POINTER(C.c_double)]),
]
SIGNATURES += GEN_SIGNATURES


def _bind() -> None:
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)  # AttributeError if the library lacks it
        fn.restype = res
        fn.argtypes = args


_bind()


class SetopsError(RuntimeError):
    """A non-zero status from the C ABI."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


def status_string(status: int) -> str:
    return lib.setops_status_string(status).decode()
