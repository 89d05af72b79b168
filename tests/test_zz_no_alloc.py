"""setops_gpu_intersect_noalloc: the intersection entry point that allocates
no device memory.

It serves callers of this library that cannot allocate: a host program that
owns all device memory through its own pool, a latency-bound path that cannot
afford cudaMalloc/cudaFree (device-wide synchronisation, unbounded latency),
or a process whose GPU memory is already full.  Its scratch is one fixed
array inside the library, shared by every call on the device, so these tests
check that two calls in a row each give exactly what the context entry point
(setops_gpu_intersect) gives on the same device buffers and what the CPU
oracle's naive_merge gives -- a result left over from the first call must not
leak into the second -- that a call after set-up leaves the device's free
memory unchanged, and that inputs beyond the array's limit are refused.

This file is named to be collected last, so that a run stopping at its first
failure has already run every other test.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import pair_with_overlap

pytestmark = pytest.mark.gpu

MAX_SMALL = 1 << 20  # SETOPS_NOALLOC_MAX_SMALL in include/setops_gpu.h


def _dev(x: np.ndarray):
    import torch
    return torch.from_numpy(x.view(np.int32)).cuda()


def _noalloc(ta, na, tb, nb, tout, cap):
    from simd_set_operations_gb300 import _lib
    n = C.c_size_t(12345)
    rc = _lib.lib.setops_gpu_intersect_noalloc(
        ta.data_ptr() if ta is not None else None, na,
        tb.data_ptr() if tb is not None else None, nb,
        tout.data_ptr() if tout is not None else None, cap, C.byref(n), None)
    return rc, n.value


def _context_path(ctx, ta, na, tb, nb, tout, cap):
    from simd_set_operations_gb300 import _lib
    n = C.c_size_t(0)
    rc = _lib.lib.setops_gpu_intersect(ctx.handle, ta.data_ptr(), na, tb.data_ptr(), nb,
                                       tout.data_ptr(), cap, C.byref(n), 0)
    assert rc == 0, _lib.status_string(rc)
    return n.value


def test_noalloc_matches_context_entry_point(ctx, orc):
    import torch
    from simd_set_operations_gb300 import _lib
    rng = np.random.default_rng(20261203)
    # first call: the largest smaller set allowed, many matches; then fewer
    # matches and none at all, so stale staging from an earlier call would show
    cases = [(MAX_SMALL, 3 * MAX_SMALL, MAX_SMALL // 3), (70_001, 1_000_003, 1_234),
             (50_000, 400_000, 0)]
    for na, nb, shared in cases:
        a, b = pair_with_overlap(rng, na, nb, shared)
        ta, tb = _dev(a), _dev(b)
        cap = min(na, nb)
        out_new = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
        out_ref = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
        rc, n_new = _noalloc(ta, na, tb, nb, out_new, cap)
        assert rc == 0, _lib.status_string(rc)
        n_ref = _context_path(ctx, ta, na, tb, nb, out_ref, cap)
        assert n_new == n_ref == shared
        torch.cuda.synchronize()
        got = out_new[:n_new].cpu().numpy().view(np.uint32)
        want = out_ref[:n_ref].cpu().numpy().view(np.uint32)
        np.testing.assert_array_equal(got, want)  # bit-exact
        np.testing.assert_array_equal(got, orc.naive_merge(a, b))
        # operands the other way round give the same result
        out_new.fill_(-1)
        rc, n_sw = _noalloc(tb, nb, ta, na, out_new, cap)
        assert rc == 0 and n_sw == n_ref
        np.testing.assert_array_equal(out_new[:n_sw].cpu().numpy().view(np.uint32), want)


def test_noalloc_limits_and_arguments(ctx):
    import torch
    from simd_set_operations_gb300 import _lib
    big = torch.zeros(MAX_SMALL + 1, dtype=torch.int32, device="cuda")
    out = torch.zeros(MAX_SMALL + 1, dtype=torch.int32, device="cuda")
    # the smaller set above the limit is refused before any GPU work
    rc, n = _noalloc(big, MAX_SMALL + 1, big, MAX_SMALL + 1, out, MAX_SMALL + 1)
    assert rc == _lib.ERR_TOO_LARGE and n == 0
    # the larger set alone may exceed it; output capacity is still checked
    rc, n = _noalloc(big, 10, big, MAX_SMALL + 1, out, 9)
    assert rc == _lib.ERR_CAPACITY
    # missing output-length pointer, missing input
    assert _lib.lib.setops_gpu_intersect_noalloc(big.data_ptr(), 4, big.data_ptr(), 4,
                                                 out.data_ptr(), 4, None, None) == _lib.ERR_INVALID
    rc, n = _noalloc(None, 5, big, 5, out, 5)
    assert rc == _lib.ERR_INVALID
    # an empty input intersects to nothing
    rc, n = _noalloc(big, 0, big, 100, out, 0)
    assert rc == 0 and n == 0


def test_noalloc_allocates_nothing_after_setup():
    """After a first call on the device (set-up and loading of the device
    code), a call on the largest allowed smaller set -- whose 4 MiB staging
    area a context would allocate -- leaves the device's free memory as it
    was."""
    import torch
    from simd_set_operations_gb300 import _lib
    rng = np.random.default_rng(20261204)
    a, b = pair_with_overlap(rng, MAX_SMALL, 2 * MAX_SMALL, 4_321)
    ta, tb = _dev(a), _dev(b)
    out = torch.empty(MAX_SMALL, dtype=torch.int32, device="cuda")
    rc, _ = _noalloc(ta[:16], 16, tb[:16], 16, out, 16)  # set-up call, tiny inputs
    assert rc == 0, _lib.status_string(rc)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        rc, n = _noalloc(ta, MAX_SMALL, tb, 2 * MAX_SMALL, out, MAX_SMALL)
        assert rc == 0 and n == 4_321, _lib.status_string(rc)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"free device memory changed by {free0 - free1} bytes"
