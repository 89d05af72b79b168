"""The autotuners of the array and BSR policies (setops_gpu_autotune,
setops_gpu_autotune_bsr): they write an (algorithm, kernel variant) into
every cell they can measure, and the tuned tables still give naive_merge's /
branchless_merge_bsr's result in every size-ratio band and size class; saved
tables are applied again for the same GPU and arguments."""
from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import pair_with_overlap

pytestmark = pytest.mark.gpu

import simd_set_operations_gb300 as so  # noqa: E402
from simd_set_operations_gb300 import _lib  # noqa: E402


@pytest.fixture(scope="module")
def tuned(tmp_path_factory):
    c = so.Context(0)  # its own context: the session context keeps the default table
    path = tmp_path_factory.mktemp("tune") / "policy.json"
    table = so.autotune(band_lo=0, band_hi=12, max_elems=1 << 20, density=0.05, reps=2,
                        cache=str(path), ctx=c)
    yield c, table, path
    c.close()


def test_autotune_fills_cells(tuned):
    c, table, path = tuned
    assert not table["from_cache"]
    # cells whose test pair fits 2^20 elements: class 0 (2^10) bands 0-9,
    # class 1 (2^14) bands 0-5, class 2 (2^19) band 0
    assert table["tuned_cells"] == 10 + 6 + 1
    for cell, flags in table["cells"].items():
        band, cls = (int(x) for x in cell.split(","))
        assert flags & 0xFF00 in (so.ALGO_MERGE, so.ALGO_GALLOP, so.ALGO_BITMAP), cell
        if band == 0:
            assert flags & 0xFF00 != so.ALGO_GALLOP, cell
    saved = json.loads(path.read_text())
    assert saved["cells"] == table["cells"] and saved["key"]["device"] == c.device_key()


def test_tuned_table_is_exact_in_every_band(tuned, orc):
    c, table, _ = tuned
    rng = np.random.default_rng(77)
    for cls, mn in enumerate((600, 9_000, 70_000)):
        for band in range(0, 10):
            mx = int(mn * (1 << band) * 1.5)
            if mx > 3_000_000:
                continue
            a, b = pair_with_overlap(rng, mn, mx, mn // 7)
            want = orc.naive_merge(a, b)
            out, n = so.intersect(a, b, ctx=c)
            assert np.array_equal(out[:n], want), (cls, band, so.describe_flags(
                c.get_policy_class(False, band, cls)))
            assert so.intersect_count(b, a, ctx=c) == want.size


def test_autotune_fills_bsr_cells(tuned):
    c, table, path = tuned
    assert table["bsr_tuned_cells"] > 0
    for cell, flags in table["bsr_cells"].items():
        band, cls = (int(x) for x in cell.split(","))
        assert flags & 0xFF00 in (so.ALGO_MERGE, so.ALGO_GALLOP), cell
        if band == 0:
            assert flags & 0xFF00 != so.ALGO_GALLOP, cell
    assert json.loads(path.read_text())["bsr_cells"] == table["bsr_cells"]


def test_tuned_bsr_table_is_exact_in_every_band(tuned, orc):
    c, table, _ = tuned
    rng = np.random.default_rng(78)
    for mn in (300, 6_000, 60_000):
        for band in range(0, 11):
            mx = int(mn * (1 << band) * 1.5)
            if mx > 3_000_000:
                continue
            a, b = pair_with_overlap(rng, mn, mx, mn // 5, hi=max(40 * mx, 1 << 20))
            ba, sa = orc.bsr_from_sorted(a)
            bb, sb = orc.bsr_from_sorted(b)
            wb, ws = orc.branchless_merge_bsr(ba, sa, bb, sb)
            v = so.BsrVec()
            so.gpu_bsr(so.BsrRef(ba, sa), so.BsrRef(bb, sb), v, ctx=c)
            assert np.array_equal(v.bases, wb) and np.array_equal(v.states, ws), (mn, band)
            cnt = so.Counter()
            so.gpu_bsr(so.BsrRef(bb, sb), so.BsrRef(ba, sa), cnt, ctx=c)
            assert cnt.count() == orc.branchless_merge_bsr_count(ba, sa, bb, sb)


def test_saved_table_is_applied_again(tuned):
    c, table, path = tuned
    c2 = so.Context(0)
    try:
        again = so.autotune(band_lo=0, band_hi=12, max_elems=1 << 20, density=0.05, reps=2,
                            cache=str(path), ctx=c2)
        assert again["from_cache"]
        for cell, flags in table["cells"].items():
            band, cls = (int(x) for x in cell.split(","))
            assert c2.get_policy_class(False, band, cls) == flags
        for cell, flags in table["bsr_cells"].items():
            band, cls = (int(x) for x in cell.split(","))
            assert c2.get_policy_class(True, band, cls) == flags
    finally:
        c2.close()


def test_autotune_arguments(tuned):
    c, _, _ = tuned
    L = _lib.lib
    n = _lib.C.c_int()
    assert L.setops_gpu_autotune(None, 0, 1, 1 << 20, 0.05, 1, _lib.C.byref(n)) == _lib.ERR_INVALID
    assert L.setops_gpu_autotune(c.handle, 3, 1, 1 << 20, 0.05, 1, None) == _lib.ERR_INVALID
    assert L.setops_gpu_autotune(c.handle, 0, 1, 1 << 20, 0.0, 1, None) == _lib.ERR_INVALID
    assert L.setops_gpu_autotune_bsr(None, 0, 1, 1 << 20, 0.05, 1, None) == _lib.ERR_INVALID
    assert L.setops_gpu_autotune_bsr(c.handle, 2, 1, 1 << 20, 0.05, 1, None) == _lib.ERR_INVALID
    assert L.setops_gpu_autotune_bsr(c.handle, 0, 1, 1, 0.05, 1, None) == _lib.ERR_INVALID
