"""The C-ABI library: loads, exports every declared symbol, and behaves on a
host without a GPU (no compute calls here)."""
from __future__ import annotations

import ctypes as C
import re

import pytest

from conftest import ROOT, gpu_available


def declared_symbols() -> set[str]:
    names = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        names |= set(re.findall(r"\b(setops_[a-z0-9_]+)\s*\(", text))
    return names


def test_headers_declare_the_abi():
    names = declared_symbols()
    for must in ("setops_gpu_create", "setops_gpu_intersect", "setops_gpu_intersect_count",
                 "setops_gpu_intersect_bsr", "setops_gpu_intersect_bsr_count",
                 "setops_gpu_svs", "setops_gpu_svs_count", "setops_datafile_write",
                 "setops_gen_twoset"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from simd_set_operations_gb300 import _lib
    missing = [n for n in sorted(declared_symbols()) if not hasattr(_lib.lib, n)]
    assert not missing, missing
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert declared_symbols() <= bound, declared_symbols() - bound


def test_status_strings_and_variants():
    from simd_set_operations_gb300 import _lib, num_variants, ALGO_MERGE, ALGO_GALLOP
    assert _lib.status_string(0) == "ok"
    assert "capacity" in _lib.status_string(_lib.ERR_CAPACITY)
    assert _lib.status_string(-100) == "unknown status"
    assert num_variants(ALGO_MERGE) >= 1 and num_variants(ALGO_GALLOP) >= 1
    assert num_variants(ALGO_MERGE, bsr=True) >= 1
    assert num_variants(0) == 0


def test_null_arguments_rejected_without_gpu():
    from simd_set_operations_gb300 import _lib
    assert _lib.lib.setops_gpu_create(None, 0) == _lib.ERR_INVALID
    assert _lib.lib.setops_gpu_destroy(None) == _lib.ERR_INVALID
    c = C.c_uint64()
    assert _lib.lib.setops_gpu_intersect_count(None, None, 0, None, 0, C.byref(c), 0) \
        == _lib.ERR_INVALID
    assert _lib.lib.setops_gpu_synchronize(None) == _lib.ERR_INVALID


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU error path")
def test_context_without_gpu_fails_cleanly():
    import simd_set_operations_gb300 as so
    with pytest.raises(so.SetopsError):
        so.Context(0)
