"""The index arithmetic of the tiled bitmap kernels (csrc/window.cuh,
csrc/tile.cuh), restated in Python over 32-bit words: the shift that fits a
tile's span into its bitmap, and the clamp that sends elements outside the
tile onto a bit that is never set.  CPU only."""
from __future__ import annotations

import numpy as np

M32 = (1 << 32) - 1


def clz32(x: int) -> int:
    return 32 - x.bit_length()


def shift_for(span: int, spanbits: int) -> int:
    """sh: 0 when span < spanbits, else 32 - clz(span / spanbits)."""
    return 0 if span < spanbits else 32 - clz32(span // spanbits)


def probe_index(x: int, w: int, sh: int, ssp: int) -> int:
    """min(((x - w) mod 2^32) >> sh, ssp + 1) -- the bit a B element tests."""
    return min(((x - w) & M32) >> sh, ssp + 1)


def test_shift_fits_and_is_least():
    rng = np.random.default_rng(5)
    for spanbits in (65536, 131072, 32768):
        spans = [0, 1, spanbits - 1, spanbits, spanbits + 1, 2 * spanbits - 1, 2 * spanbits,
                 M32, M32 - 1, 1 << 31, (1 << 31) - 1]
        spans += [int(v) for v in rng.integers(0, 1 << 32, 2000, dtype=np.uint64)]
        for span in spans:
            sh = shift_for(span, spanbits)
            assert (span >> sh) < spanbits, (span, sh)          # the span fits T
            if sh > 0:
                assert (span >> (sh - 1)) >= spanbits, (span, sh)  # and sh is the least


def test_elements_inside_map_inside_and_outside_clamp():
    rng = np.random.default_rng(6)
    spanbits = 65536
    for _ in range(3000):
        w = int(rng.integers(0, 1 << 32))
        span = int(rng.integers(0, 1 << 32)) if rng.random() < 0.5 else int(rng.integers(0, spanbits))
        span = min(span, M32 - w)  # alast = w + span stays a u32
        sh = shift_for(span, spanbits)
        ssp = span >> sh
        # inside [w, w + span]: a bit of T, at most ssp
        for x in (w, w + span, w + span // 2):
            assert probe_index(x, w, sh, ssp) <= ssp
        # outside: a dense tile (sh = 0) always lands past T's last bit, which
        # is never set; a coarse tile may land inside, and its candidates are
        # then checked against the sorted tile
        for x in ([w - 1, 0] if w > 0 else []) + ([w + span + 1, M32] if w + span < M32 else []):
            o = probe_index(x, w, sh, ssp)
            if sh == 0:
                assert o == ssp + 1, (x, w, span, o)
            assert o <= ssp + 1
        # T's words: the probe's word index never passes the region
        assert (ssp + 1) >> 5 <= spanbits // 32
