// tile.cuh -- tiled bitmap intersection of two sorted, duplicate-free u32
// arrays: the same result as the merge-path kernel (the reference's
// naive_merge, setops/src/intersect/merge.rs:7-33; Counter semantics,
// setops/src/visitor.rs:24-49), organised for streaming.
//
// Work layout
// -----------
// Let A be the smaller input.  CTA c of the G resident CTAs owns the
// contiguous run A[c*na/G, (c+1)*na/G) and walks it in tiles of up to TA
// elements.  For a tile A[i0, i1) with values [w, alast]:
//
//   1. Warp 0 finds where the tile's B range ends, b1 = the first B index
//      with a value above alast, by a warp-wide search of B in global memory
//      (the range starts where the previous tile's ended; the CTA's first
//      tile searches its start too, on warp 1), while the other warps stream
//      A[i0, i1) with 128-bit loads: into a bitmap T of the value range when
//      it is dense enough (span < 32*VW), else as the sorted A tile itself.
//   2. All warps stream B[b0, b1) with 128-bit loads; each element tests its
//      bit in T (dense) or binary-searches the A tile (sparse).
//   3. Count mode counts.  Materialise mode marks each match in bitmap M
//      (by value offset when dense, by A position when sparse; either way M
//      is in ascending order) and appends the tile's matches, in order, to
//      the CTA's staging run, which starts at the CTA's first A index -- an
//      exclusive region, since a CTA cannot match more elements than it owns.
//
// Materialise mode then publishes each CTA's match count, passes one
// grid-wide barrier (the kernel is launched cooperatively, so every CTA is
// resident) and copies the CTA's staged run to its offset, the sum of the
// counts of CTAs 0..c-1.  Count mode adds per-CTA totals atomically.
//
// There are no mbarriers and no asynchronous copies: every input element is
// read once with a coalesced 128-bit load (ragged ends with plain loads);
// the only wait is the bounded grid barrier.
#pragma once

#include "common.cuh"
#include "merge.cuh"  // MergeArgs

namespace setops {

template <int NT, int TA, int VW, bool MAT>
struct TileCfg {
  static_assert(NT % 32 == 0 && NT >= 128, "at least four warps");
  static_assert(TA % 4 == 0 && TA <= VW, "a sparse tile is kept in T's words");
  static_assert((VW & (VW - 1)) == 0 && VW % 4 == 0, "power-of-two table");
  static constexpr uint32_t kSpan = uint32_t(VW) * 32u;  // values per dense tile
  static constexpr int kTabWords = VW + 4;                // + zero pad word group
  // match bitmap M (materialise), whose upper half doubles as the coarse
  // bitmap C of a sparse tile (M then holds one bit per A position, at most
  // TA bits); count mode: C alone
  // (+ 4: a zero word past C's last, where probes beyond the tile land)
  static constexpr int kMWords = MAT ? VW + 4 : VW / 2 + 4;
  static constexpr int kCOff = MAT ? VW / 2 : 0;          // C's first word in M
  static constexpr uint32_t kCSpan = uint32_t(VW / 2) * 32u;  // values per coarse bitmap
  static_assert(!MAT || (TA + 6 + 31) / 32 <= VW / 2, "M's position bits stay below C");
  static constexpr size_t kSmemBytes = size_t(kTabWords + kMWords) * 4;
  static constexpr int kTile = TA;
};

// First index i in [0, n) with B[i] >= v (n when none).  All 32 lanes of the
// calling warp take part and get the result.  `est` is a guess of the answer:
// one round probes 32 points around it; (32+1)-ary rounds narrow the rest.
__device__ __forceinline__ uint64_t warp_lower_bound(const uint32_t *__restrict__ B,
                                                     uint64_t n, uint32_t v,
                                                     uint64_t est) {
  const int lane = threadIdx.x & 31;
  uint64_t lo = 0, hi = n;  // answer in [lo, hi]
  if (n > 64) {
    // probes at est + d, d in {-2^15, ..., -2^0, 0, 2^0, ..., 2^14} (scaled
    // by 16): narrows to one gap in a few thousand elements when the guess
    // is close, and to a power-of-two bracket when it is not
    if (est >= n) est = n - 1;
    const int k = lane - 16;
    const uint64_t d = (k == 0) ? 0 : (uint64_t(16) << ((k < 0 ? -k : k) - 1));
    bool ok;
    uint64_t x;
    if (k < 0) {
      ok = est >= d;
      x = ok ? est - d : 0;
    } else {
      x = est + d;
      ok = x < n;
    }
    const bool below = ok && (__ldg(B + x) < v);  // answer > x
    const bool above = ok && !below;              // answer <= x
    // largest probe below the answer and smallest probe at or above it
    uint64_t l = below ? x + 1 : 0, h = above ? x : n;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const uint64_t lo2 = __shfl_xor_sync(0xffffffffu, l, o);
      const uint64_t hi2 = __shfl_xor_sync(0xffffffffu, h, o);
      l = lo2 > l ? lo2 : l;
      h = hi2 < h ? hi2 : h;
    }
    lo = l;
    hi = h;
  }
  while (hi - lo > 32) {
    const uint64_t span = hi - lo;
    const uint64_t x = lo + (uint64_t(lane) + 1) * span / 33;  // < hi
    const unsigned m = __ballot_sync(0xffffffffu, __ldg(B + x) < v);
    const int c = __popc(m);  // probes below v form a prefix
    const uint64_t nlo = c ? lo + uint64_t(c) * span / 33 + 1 : lo;
    const uint64_t nhi = (c < 32) ? lo + (uint64_t(c) + 1) * span / 33 : hi;
    lo = nlo;
    hi = nhi;
  }
  const uint64_t x = lo + uint64_t(lane);
  const unsigned m = __ballot_sync(0xffffffffu, x < hi && __ldg(B + x) < v);
  return lo + uint64_t(__popc(m));
}

// [v0, v1): the part of [lo, hi) of u32 array `base` whose elements can be
// read with 16-byte loads (v0 the first index with a 16-byte aligned
// address, v1 the last such boundary); v0 == v1 when there is none.
__device__ __forceinline__ void aligned_body(const uint32_t *base, uint64_t lo, uint64_t hi,
                                             uint64_t &v0, uint64_t &v1) {
  const uint64_t mis = (reinterpret_cast<uintptr_t>(base) >> 2) & 3;  // words past 16 B
  v0 = lo + ((4 - ((mis + lo) & 3)) & 3);
  const uint64_t r = (mis + hi) & 3;
  v1 = hi >= r ? hi - r : 0;  // (unsigned: never below zero)
  if (v0 > hi) v0 = hi;
  if (v1 < v0) v1 = v0;
}

// Streams [0, n) of array `src` (16-byte aligned from element h to element
// e; plain loads outside) through `f(j, value)` for every element j, one
// 16-byte load per thread per step: latency is hidden by running up to 64
// warps per SM (the kernel stays within 32 registers), not by unrolling.
// Threads `tt` of `ns`.
template <class F>
__device__ __forceinline__ void stream_elems(const uint32_t *src, uint32_t n, uint32_t h,
                                             uint32_t e, uint32_t tt, uint32_t ns, F f) {
  for (uint32_t j = tt; j < h; j += ns) f(j, __ldg(src + j));
  for (uint32_t j = e + tt; j < n; j += ns) f(j, __ldg(src + j));
  const uint4 *s4 = reinterpret_cast<const uint4 *>(src + h);  // 16-byte aligned
  const uint32_t n4 = (e - h) / 4;
  for (uint32_t u0 = tt; u0 < n4; u0 += ns) {
    const uint4 x = __ldcs(s4 + u0);
    const uint32_t j = h + 4 * u0;
    f(j, x.x);
    f(j + 1, x.y);
    f(j + 2, x.z);
    f(j + 3, x.w);
  }
}

// Grid-wide barrier for a cooperatively launched grid: every CTA adds one to
// *arrived, and waits (polling with back-off, bounded) until it reaches
// `target`.  Returns false after recording a timeout.  Call from all threads.
__device__ __forceinline__ bool grid_barrier(uint32_t *arrived, uint32_t target, int *err) {
  __shared__ uint32_t s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(arrived, 1u);
    uint32_t ok = 1;
    const uint64_t t0 = global_ns();
    while (ld_acquire_u32(arrived) < target) {
      __nanosleep(200);  // one load per CTA every few hundred ns
      if (global_ns() - t0 > wait_limit_ns()) {
        record_error(err, DEV_ERR_TIMEOUT_LOOKBACK);
        ok = 0;
        break;
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Shared-memory words of one CTA used by tile_run.
template <int NT>
struct TileShared {
  unsigned long long b0, b1;
  uint32_t warp_sums[NT / 32];
};

// Intersects the run A[i_begin, i_end) of a sorted set with the sorted set
// B[0, nb), tile by tile (see the file comment).  `search`: find each tile's
// B range by warp searches (B is long and the run covers part of it); else
// every tile probes all of B (a short B, e.g. a pair that fits one tile).
// T and M (tab, mbits) must be zero on entry; they are zero again on return.
// Materialise: appends the matches in ascending order at dst[0, ...) and
// returns their number (the same in every thread).  Count mode: returns this
// thread's share of the count (the caller sums over the CTA).  All NT
// threads call it.
template <int NT, int TA, int VW, bool MAT>
__device__ __forceinline__ uint64_t tile_run(const uint32_t *A, uint64_t i_begin,
                                             uint64_t i_end, const uint32_t *B, uint64_t nb,
                                             bool search, uint32_t *dst, uint32_t *tab,
                                             uint32_t *mbits, TileShared<NT> &sh) {
  using Cfg = TileCfg<NT, TA, VW, MAT>;
  constexpr uint32_t SPAN = Cfg::kSpan;
  constexpr int NW = NT / 32;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  uint32_t *cbits = mbits + Cfg::kCOff;  // C (sparse tiles)
  // B's first and last values guide the searches (uniformly spread values
  // land close to the guess)
  const uint32_t bfirst = (search && nb) ? __ldg(B) : 0u;
  const uint32_t blast = (search && nb) ? __ldg(B + nb - 1) : 0u;
  auto guess = [&](uint32_t key) -> uint64_t {
    if (blast <= bfirst || key <= bfirst) return 0;
    return guess_scale(key - bfirst, blast - bfirst, nb - 1);
  };
  uint32_t cnt = 0;       // count mode
  uint64_t staged = 0;    // materialise: matches written so far
  uint64_t b_next = 0;    // B range start of the next tile
  for (uint64_t i0 = i_begin; i0 < i_end; i0 += TA) {
    const uint64_t i1 = (i0 + TA < i_end) ? i0 + TA : i_end;
    const uint32_t ntile = uint32_t(i1 - i0);
    const bool first = i0 == i_begin;
    // warps searching B this tile (none when B is probed whole)
    const int searchers = !search ? 0 : (first ? 2 : 1);
    const uint32_t w = __ldg(A + i0), alast = __ldg(A + i1 - 1);
    const bool dense = alast - w < SPAN;
    const uint32_t span = alast - w;
    // sparse: C holds one bit per 2^csh values (the least shift that fits)
    const uint32_t csh = dense ? 0u : 32u - __clz(span / Cfg::kCSpan);
    const uint32_t cssp = span >> csh;  // C's last bit

    // ---- 1. B range (search warps) and A tile (the other warps) ----
    if (warp < searchers) {
      uint64_t r;
      if (warp == 0) {  // b1: first B value above alast
        r = (alast == 0xffffffffu) ? nb : warp_lower_bound(B, nb, alast + 1u, guess(alast + 1u));
        if (lane == 0) sh.b1 = r;
      } else {          // b0 of the CTA's first tile
        r = warp_lower_bound(B, nb, w, guess(w));
        if (lane == 0) sh.b0 = r;
      }
    } else {
      const uint32_t tt = uint32_t(t - 32 * searchers);
      const uint32_t ns = uint32_t(NT - 32 * searchers);
      uint64_t v0, v1;
      aligned_body(A, i0, i1, v0, v1);
      const uint32_t h = uint32_t(v0 - i0), e = uint32_t(v1 - i0);  // tile-relative
      if (dense) {
        stream_elems(A + i0, ntile, h, e, tt, ns, [&](uint32_t, uint32_t x) {
          const uint32_t o = x - w;
          atomicOr(&tab[o >> 5], 1u << (o & 31));
        });
      } else {
        // the sorted tile in T; C: one bit per 2^csh values of it
        stream_elems(A + i0, ntile, h, e, tt, ns, [&](uint32_t j, uint32_t x) {
          tab[j] = x;
          const uint32_t o = (x - w) >> csh;
          atomicOr(&cbits[o >> 5], 1u << (o & 31));
        });
      }
    }
    __syncthreads();
    const uint64_t b0 = !search ? 0 : (first ? uint64_t(sh.b0) : b_next);
    const uint64_t b1 = !search ? nb : (sh.b1 > b0 ? uint64_t(sh.b1) : b0);
    b_next = b1;

    // ---- 2. probe B[b0, b1) ----
    {
      uint64_t v0, v1;
      aligned_body(B, b0, b1, v0, v1);
      const uint32_t nbt = uint32_t(b1 - b0);
      const uint32_t h = uint32_t(v0 - b0), e = uint32_t(v1 - b0);  // relative to b0
      if (dense) {
        // every B element here lies in [w, alast]: its bit is in T (the
        // clamp only guards T's bounds)
        stream_elems(B + b0, nbt, h, e, uint32_t(t), uint32_t(NT), [&](uint32_t, uint32_t x) {
          uint32_t pos = x - w;
          pos = pos <= span ? pos : span + 1;
          if ((tab[pos >> 5] >> (pos & 31)) & 1u) {
            if (MAT) atomicOr(&mbits[pos >> 5], 1u << (pos & 31));
            else ++cnt;
          }
        });
      } else {
        // C's bit first (a few per cent of the elements land on a set bit);
        // candidates binary-search the sorted tile.  Each thread takes two
        // 16-byte words per step and searches only its candidates, one at a
        // time, so a warp runs a search per candidate, not per element.
        auto cbit = [&](uint32_t x) -> uint32_t {
          const uint32_t o = min((x - w) >> csh, cssp + 1);
          return (cbits[o >> 5] >> (o & 31)) & 1u;
        };
        auto check = [&](uint32_t x) {
          uint32_t lo = 0, len = ntile;
          while (len > 0) {
            const uint32_t hh = len >> 1;
            if (tab[lo + hh] < x) {
              lo += hh + 1;
              len -= hh + 1;
            } else {
              len = hh;
            }
          }
          if (lo < ntile && tab[lo] == x) {  // M bit by A position
            if (MAT) atomicOr(&mbits[lo >> 5], 1u << (lo & 31));
            else ++cnt;
          }
        };
        const uint32_t *src = B + b0;
        for (uint32_t j = uint32_t(t); j < h; j += NT) {
          const uint32_t x = __ldg(src + j);
          if (cbit(x)) check(x);
        }
        for (uint32_t j = e + uint32_t(t); j < nbt; j += NT) {
          const uint32_t x = __ldg(src + j);
          if (cbit(x)) check(x);
        }
        const uint4 *s4 = reinterpret_cast<const uint4 *>(src + h);  // 16-byte aligned
        const uint32_t n4 = (e - h) / 4;
        for (uint32_t u0 = uint32_t(t); u0 < n4; u0 += 2 * NT) {
          const bool two = u0 + NT < n4;
          const uint4 xa = __ldcs(s4 + u0);
          const uint4 xb = two ? __ldcs(s4 + u0 + NT) : xa;
          uint32_t cm = cbit(xa.x) | (cbit(xa.y) << 1) | (cbit(xa.z) << 2) | (cbit(xa.w) << 3);
          if (two) cm |= (cbit(xb.x) | (cbit(xb.y) << 1) | (cbit(xb.z) << 2) | (cbit(xb.w) << 3)) << 4;
          while (cm) {
            const uint32_t c = uint32_t(__ffs(cm)) - 1u;
            cm &= cm - 1u;
            const uint4 v = c < 4u ? xa : xb;
            const uint32_t k = c & 3u;
            check(k == 0u ? v.x : k == 1u ? v.y : k == 2u ? v.z : v.w);
          }
        }
      }
    }
    __syncthreads();

    // ---- 3. output (materialise): M in order, appended to the staging run ----
    if (MAT) {
      const uint32_t mw = dense ? (span >> 5) + 1 : (ntile + 31) / 32;  // M words in use
      // thread t owns M words [t*per, t*per + per)
      const uint32_t per = (mw + NT - 1) / NT;
      const uint32_t m0 = uint32_t(t) * per;
      const uint32_t m1 = (m0 + per < mw) ? m0 + per : mw;
      uint32_t pc = 0;
      for (uint32_t i = m0; i < m1; ++i) pc += __popc(mbits[i]);
      uint32_t incl = pc;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      if (lane == 31) sh.warp_sums[warp] = incl;
      __syncthreads();
      uint32_t before = 0, tot = 0;
#pragma unroll
      for (int k = 0; k < NW; ++k) {
        const uint32_t sm = sh.warp_sums[k];
        before += (k < warp) ? sm : 0u;
        tot += sm;
      }
      uint64_t q = staged + before + incl - pc;
      for (uint32_t i = m0; i < m1; ++i) {
        uint32_t m = mbits[i];
        if (!m) continue;
        mbits[i] = 0;
        while (m) {
          const uint32_t pos = i * 32u + uint32_t(__ffs(m) - 1);
          m &= m - 1;
          dst[q++] = dense ? w + pos : tab[pos];
        }
      }
      staged += tot;
      __syncthreads();  // sparse: the A tile was read above; warp sums reused
    }
    // clear T for the next tile (dense: the words used; sparse: the tile,
    // and C's words used)
    {
      const uint32_t tw = dense ? (span >> 5) + 1 : ntile;
      for (uint32_t i = 4u * uint32_t(t); i < tw; i += 4u * NT)
        *reinterpret_cast<uint4 *>(tab + i) = make_uint4(0, 0, 0, 0);
      if (!dense)
        for (uint32_t i = uint32_t(t); i <= (cssp >> 5); i += NT) cbits[i] = 0;
    }
    __syncthreads();  // T clear before the next tile's insertion
  }

  return MAT ? staged : uint64_t(cnt);
}

template <int NT, int TA, int VW, int MINB, bool MAT>
__global__ void __launch_bounds__(NT, MINB) tile_kernel(const MergeArgs p) {
  using Cfg = TileCfg<NT, TA, VW, MAT>;
  constexpr int NW = NT / 32;

  extern __shared__ __align__(128) uint32_t smem[];
  uint32_t *tab = smem;                  // T (dense) or the sorted A tile (sparse)
  uint32_t *mbits = smem + Cfg::kTabWords;

  __shared__ TileShared<NT> sh;
  __shared__ unsigned long long red[NW];

  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;

  // ---- problem (A = smaller set) ----
  uint64_t na = p.na_dev ? *p.na_dev : p.na;
  uint64_t nb = p.nb_dev ? *p.nb_dev : p.nb;
  const uint32_t *A = p.a, *B = p.b;
  if (na > nb) {
    const uint32_t *tp = A; A = B; B = tp;
    uint64_t tn = na; na = nb; nb = tn;
  }
  if (skip_by_rule(p.skip_rule, p.ratio_thr, na, nb)) return;
  const uint32_t G = gridDim.x;
  // this CTA's run of A (empty when B is)
  const uint64_t ca0 = nb ? uint64_t(blockIdx.x) * na / G : 0;
  const uint64_t ca1 = nb ? (uint64_t(blockIdx.x) + 1) * na / G : 0;

  for (int i = t; i < (Cfg::kTabWords + Cfg::kMWords) / 4; i += NT)
    reinterpret_cast<uint4 *>(smem)[i] = make_uint4(0, 0, 0, 0);
  __syncthreads();

  const uint64_t r = tile_run<NT, TA, VW, MAT>(A, ca0, ca1, B, nb, true, p.stage + ca0, tab,
                                                mbits, sh);
  const uint32_t cnt = MAT ? 0u : uint32_t(r);
  const uint64_t staged = MAT ? r : 0;

  // ---- combine ----
  if (!MAT) {
    uint64_t v = cnt;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (t == 0) {
      unsigned long long sm = 0;
      for (int k = 0; k < NW; ++k) sm += red[k];
      if (sm) atomicAdd(&p.sync->acc, sm);
      __threadfence();
      const uint32_t prev = atomicAdd(&p.sync->done, 1u);
      if (prev == G - 1) {
        *p.out_len = atomicExch(&p.sync->acc, 0ull);
        p.sync->ticket = 0;
        p.sync->done = 0;
        __threadfence();
      }
    }
    return;
  }

  if constexpr (MAT) {
    // Materialise: publish this CTA's count; after the grid barrier (all CTAs
    // are resident: cooperative launch) add up the counts of CTAs 0..c-1 --
    // plain loads, nothing to wait for -- and copy the staged run.
    if (t == 0) p.coranks[blockIdx.x] = staged;
    if (!grid_barrier(&p.sync->done, G, p.err)) return;
    uint64_t before = 0;
    for (uint32_t c = uint32_t(t); c < blockIdx.x; c += NT) before += p.coranks[c];
  #pragma unroll
    for (int o = 16; o > 0; o >>= 1) before += __shfl_xor_sync(0xffffffffu, before, o);
    if (lane == 0) red[warp] = before;
    __syncthreads();
    uint64_t ex = 0;
  #pragma unroll
    for (int k = 0; k < NW; ++k) ex += red[k];
    if (ex + staged > p.out_cap) {
      if (t == 0) record_error(p.err, DEV_ERR_CAPACITY);
    } else {
      for (uint64_t q = uint64_t(t); q < staged; q += NT) p.out[ex + q] = p.stage[ca0 + q];
      // the last CTA's end is the total
      if (blockIdx.x == G - 1 && t == 0) *p.out_len = ex + staged;
    }
    // the last CTA out resets the coordination words for the next launch
    if (t == 0) {
      __threadfence();
      const unsigned long long prev = atomicAdd(&p.sync->acc, 1ull);
      if (prev == G - 1) {
        p.sync->ticket = 0;
        p.sync->done = 0;
        p.sync->acc = 0;
        __threadfence();
      }
    }
  }
}

}  // namespace setops
