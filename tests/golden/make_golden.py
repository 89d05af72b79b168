"""Generates the golden fixtures in tests/golden/.

    python tests/golden/make_golden.py

1. ``unit_tests.json`` -- the reference's known-answer tests,
   setops/tests/unit_tests.rs:7-33 (five 2-set cases; case 5's expectation
   is what const_intersect, setops/src/intersect/merge.rs:89-117, computes at
   compile time) and :49-59 (galloping: small = [1 << 12 + 1], which Rust
   parses as 1 << 13, against 0..12345).
2. ``datafile_roundtrip.json`` -- the datafile round-trip vectors of
   benchmark/src/datafile.rs:184-222.
3. ``ref_kernels.npz`` -- outputs of the reference's own C++ kernels
   (setops/ffi/qfilter/qfilter.cpp: intersect_bmiss_uint_b4,
   intersect_qfilter_uint_b4_v2, intersect_qfilter_bsr_b4), compiled
   unchanged from the reference tree into oracle/_ref/ (``make -C oracle
   ref``; x86 only), on seeded inputs shaped like the reference's
   property-test generators (setops/tests/testlib/mod.rs:102-153).  Values
   stay below 2^31 because those kernels compare as signed int.

Items 1-2 are fixed data; item 3 needs an x86 host with the reference tree,
named by the environment variable SETOPS_REF_ROOT.
"""
from __future__ import annotations

import json
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

UNIT_TESTS = {
    "source": "setops/tests/unit_tests.rs:7-33,49-59",
    "twoset": [
        {"name": "test_2set_intersect1", "a": [1, 2, 3, 4], "b": [1, 2, 3, 4, 5],
         "expected": [1, 2, 3, 4]},
        {"name": "test_2set_intersect2", "a": [0, 4, 5, 8], "b": [1, 2, 3, 6],
         "expected": []},
        {"name": "test_2set_intersect3", "a": [1, 4, 5], "b": [1, 4, 5],
         "expected": [1, 4, 5]},
        {"name": "test_2set_intersect4", "a": [10, 42],
         "b": [1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 22, 25, 28, 39, 42, 43, 47, 49],
         "expected": [10, 42]},
        {"name": "test_2set_intersect5", "a": [1, 3, 5, 8, 9, 10, 14, 15, 18, 20],
         "b": [1, 2, 3, 4, 9, 10, 11, 15, 20, 21], "expected": [1, 3, 9, 10, 15, 20]},
    ],
    "galloping": {"name": "test_simd_galloping", "small": [1 << 13],
                  "large_range": [0, 12345], "expected": [1 << 13]},
}

DATAFILE = {
    "source": "benchmark/src/datafile.rs:184-222",
    "magic": [0xE9, 0xAA, 0x05],
    "cases": {
        "test_pair": [[0, 4, 10, 20, 21, 26, 99], [0, 5, 6]],
        "test_kset": [
            [122, 120, 161, 155, 97, 86, 36, 32, 80, 9, 149, 140, 200, 82, 143, 30, 71, 33],
            [19, 6, 141, 90, 194, 167, 119, 125, 156, 197, 79, 98, 160, 28, 42, 111, 124, 18],
            [74, 196, 139, 159, 78, 48, 168, 199, 169, 26, 15, 55, 182, 59, 10, 49, 165, 75],
            [99, 190, 11, 107, 193, 69, 38, 137, 65, 44, 127, 62, 146, 135, 94, 50, 105, 123],
            [41, 72, 68, 198, 195, 31, 134, 46, 103, 7, 61, 185, 188, 47, 152, 70, 189, 130],
            [126, 117, 148, 8, 178, 93, 166, 138, 171, 158, 131, 183, 157, 176, 16, 40, 34],
            [52, 54, 67, 122, 106, 12, 187, 150, 22, 172, 64, 163, 101, 37, 110, 170, 144],
            [113, 181, 87, 24, 60, 88, 164, 51, 63, 179, 43, 92, 186, 84, 25, 95, 115, 133],
            [85, 96, 132, 1, 56, 53, 89, 136, 21, 45, 27, 29, 58, 116, 2, 118, 39, 23, 20, 3],
            [100, 154, 4, 17, 129, 174, 57, 73, 145, 112, 14, 177, 184, 76, 91, 104, 83, 151],
            [173, 162, 81, 13, 114, 77, 66, 5, 191, 108, 180, 147, 175, 109, 35, 153, 128],
            [142, 192, 102],
        ],
        "test_many_empty_sets": [[], [], [], [], []],
    },
    # test_large_sets: ranges (0..(1<<16)-2), (0..(1<<17)+5), (0..(1<<14)/3)
    "range_cases": {"test_large_sets": [[0, (1 << 16) - 2], [0, (1 << 17) + 5],
                                        [0, (1 << 14) // 3]]},
}


def similar_pair(rng, max_len):
    """SimilarSetPair (testlib/mod.rs:102-121): a shared vector added to two
    random vectors, each sorted and deduplicated."""
    shared = rng.integers(0, 1 << 31, rng.integers(0, max_len + 1))
    a = np.concatenate([rng.integers(0, 1 << 31, rng.integers(0, max_len + 1)), shared])
    b = np.concatenate([rng.integers(0, 1 << 31, rng.integers(0, max_len + 1)), shared])
    return np.unique(a).astype(np.uint32), np.unique(b).astype(np.uint32)


def dense_pair(rng, n, span):
    """Two sets drawn from a small span, so that BSR words hold many bits."""
    a = np.unique(rng.integers(0, span, n)).astype(np.uint32)
    b = np.unique(rng.integers(0, span, n)).astype(np.uint32)
    return a, b


def skewed_pair(rng):
    """SkewedSetPair (testlib/mod.rs:124-153)."""
    small_size = int(rng.integers(0, 1 << 20)) % 128 + 1
    large_size = int(rng.integers(0, 1 << 20)) % 8192 + 128
    shared_n = int(rng.integers(0, 1 << 20)) % small_size
    shared = rng.integers(0, 1 << 31, shared_n)
    s = np.concatenate([rng.integers(0, 1 << 31, small_size - shared_n), shared])
    l = np.concatenate([rng.integers(0, 1 << 31, large_size - shared_n), shared])
    return np.unique(s).astype(np.uint32), np.unique(l).astype(np.uint32)


def make_ref_kernels(path: Path) -> None:
    import oracle

    oracle.build(ref_root=os.environ.get("SETOPS_REF_ROOT"))
    if oracle.ref_lib() is None:
        print("skip ref_kernels.npz: reference kernels unavailable on this host")
        return
    rng = np.random.default_rng(20260101)
    arrays = {}
    meta = []
    cases = []
    for i in range(12):
        cases.append(("similar", *similar_pair(rng, [8, 100, 1000, 3000][i % 4])))
    for i in range(8):
        cases.append(("skewed", *skewed_pair(rng)))
    for i in range(6):
        cases.append(("dense", *dense_pair(rng, [50, 400, 2000][i % 3], [300, 2000, 5000][i % 3])))
    for idx, (kind, a, b) in enumerate(cases):
        arrays[f"a{idx}"] = a
        arrays[f"b{idx}"] = b
        arrays[f"bmiss{idx}"] = oracle.ref_two("intersect_bmiss_uint_b4", a, b)
        arrays[f"qfilter{idx}"] = oracle.ref_two("intersect_qfilter_uint_b4_v2", a, b)
        ba, sa = oracle.bsr_from_sorted(a)
        bb, sb = oracle.bsr_from_sorted(b)
        ob, os_ = oracle.ref_bsr("intersect_qfilter_bsr_b4", ba, sa, bb, sb)
        arrays[f"qbsr_bases{idx}"] = ob
        arrays[f"qbsr_states{idx}"] = os_
        meta.append(kind)
    arrays["kinds"] = np.array(meta)
    np.savez_compressed(path, **arrays)
    print(f"wrote {path} ({len(cases)} cases)")


def main() -> None:
    (HERE / "unit_tests.json").write_text(json.dumps(UNIT_TESTS, indent=1) + "\n")
    (HERE / "datafile_roundtrip.json").write_text(json.dumps(DATAFILE, indent=1) + "\n")
    make_ref_kernels(HERE / "ref_kernels.npz")


if __name__ == "__main__":
    main()
