"""Shared pytest setup.

Markers: ``gpu`` -- needs a CUDA GPU (run with ``-m gpu``); everything else
runs on a CPU-only host.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def ctx():
    """One library context for the GPU tests (device 0)."""
    if not gpu_available():
        pytest.skip("no CUDA GPU")
    import simd_set_operations_gb300 as so
    c = so.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.lib()
    return oracle


def rand_set(rng, n, hi=1 << 32):
    """Sorted, duplicate-free u32 set of exactly n values below hi."""
    if n == 0:
        return np.empty(0, np.uint32)
    if n > hi:
        raise ValueError(f"cannot draw {n} distinct values below {hi}")
    out = np.unique(rng.integers(0, hi, int(n * 1.3) + 16, dtype=np.uint64))
    while out.size < n:
        out = np.unique(np.concatenate([out, rng.integers(0, hi, n, dtype=np.uint64)]))
    sel = np.sort(rng.choice(out.size, n, replace=False))
    return out[sel].astype(np.uint32)


def pair_with_overlap(rng, na, nb, shared, hi=1 << 32):
    """Two sets of sizes na, nb sharing `shared` elements."""
    allv = rand_set(rng, na + nb - shared, hi)
    perm = rng.permutation(allv.size)
    s = allv[perm[:shared]]
    a = np.sort(np.concatenate([s, allv[perm[shared:shared + na - shared]]]))
    b = np.sort(np.concatenate([s, allv[perm[na:na + nb - shared]]]))
    return a.astype(np.uint32), b.astype(np.uint32)
