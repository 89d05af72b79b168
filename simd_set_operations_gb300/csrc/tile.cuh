// tile.cuh -- tiled bitmap intersection of two sorted, duplicate-free u32
// arrays: the same result as the merge-path kernel (the reference's
// naive_merge, setops/src/intersect/merge.rs:7-33; Counter semantics,
// setops/src/visitor.rs:24-49), organised for streaming.
//
// Work layout
// -----------
// Let A be the smaller input.  A is cut into fixed tiles of TA elements;
// a persistent grid pulls tiles in order from an atomic ticket.  For tile t
// covering A[i0, i1) with values [w, alast]:
//
//   1. Two warps find the tile's B range [b0, b1) -- the B elements with
//      values in [w, alast] -- by warp-wide searches of B in global memory,
//      while the other warps stream A[i0, i1) with 128-bit loads: into a
//      bitmap T of the value range when it is dense enough (span < 32*VW),
//      else as the sorted A tile itself.
//   2. All warps stream B[b0, b1) with 128-bit loads; each element tests its
//      bit in T (dense) or binary-searches the A tile (sparse).
//   3. Count mode counts.  Materialise mode marks each match in bitmap M
//      (by value offset when dense, by A position when sparse; either way M
//      is in ascending order) and writes the tile's matches, in order, to a
//      staging area at i0 -- an exclusive region, since a tile cannot match
//      more elements than it has.
//
// Materialise mode ends with one grid-wide barrier (the kernel is launched
// cooperatively, so every CTA is resident), after which every CTA scans the
// per-tile match counts and copies its share of the tiles' staged matches to
// their final offsets.  Count mode adds per-CTA totals atomically.
//
// There are no mbarriers and no asynchronous copies: every input element is
// read once with a coalesced 128-bit load (boundary elements with plain
// loads), and the only waits are the bounded grid barrier and nothing else.
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
  static constexpr int kMWords = MAT ? VW : 0;            // match bitmap
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
  v1 = hi - ((mis + hi) & 3);
  if (v0 > hi) v0 = hi;
  if (v1 < v0) v1 = v0;
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
      if (global_ns() - t0 > kWaitLimitNs) {
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

template <int NT, int TA, int VW, bool MAT>
__global__ void __launch_bounds__(NT) tile_kernel(const MergeArgs p) {
  using Cfg = TileCfg<NT, TA, VW, MAT>;
  constexpr uint32_t SPAN = Cfg::kSpan;
  constexpr int NW = NT / 32;

  extern __shared__ __align__(128) uint32_t smem[];
  uint32_t *tab = smem;                  // T (dense) or the sorted A tile (sparse)
  uint32_t *mbits = smem + Cfg::kTabWords;

  __shared__ uint32_t s_tile, s_w, s_alast;
  __shared__ unsigned long long s_b0, s_b1;
  __shared__ uint32_t warp_sums[NW];
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
  const uint64_t ntiles = nb ? (na + TA - 1) / TA : 0;  // no B: nothing to match
  const uint32_t G = gridDim.x;
  // B's first and last values guide the searches (uniformly spread values
  // land close to the guess)
  const uint32_t bfirst = nb ? __ldg(B) : 0u, blast = nb ? __ldg(B + nb - 1) : 0u;

  for (int i = t; i < (Cfg::kTabWords + Cfg::kMWords) / 4; i += NT)
    reinterpret_cast<uint4 *>(smem)[i] = make_uint4(0, 0, 0, 0);

  uint32_t cnt = 0;  // count mode
  for (;;) {
    if (t == 0) s_tile = atomicAdd(&p.sync->ticket, 1u);
    __syncthreads();  // also: the last tile's T / M use is over
    const uint32_t tile = s_tile;
    if (uint64_t(tile) >= ntiles) break;
    const uint64_t i0 = uint64_t(tile) * TA;
    const uint64_t i1 = (i0 + TA < na) ? i0 + TA : na;
    const uint32_t ntile = uint32_t(i1 - i0);

    // ---- 1. B range (warps 0, 1) and A tile (the other warps) ----
    if (warp < 2) {
      const uint32_t w = __ldg(A + i0), alast = __ldg(A + i1 - 1);
      const uint32_t v = (warp == 0) ? w : alast;
      uint64_t r;
      if (warp == 1 && alast == 0xffffffffu) {
        r = nb;
      } else {
        const uint32_t key = (warp == 0) ? v : v + 1u;  // [b0, b1): values in [w, alast]
        uint64_t est = 0;
        if (blast > bfirst && key > bfirst)
          est = uint64_t(double(key - bfirst) / double(blast - bfirst) * double(nb - 1));
        r = warp_lower_bound(B, nb, key, est);
      }
      if (lane == 0) {
        if (warp == 0) {
          s_b0 = r;
          s_w = w;
        } else {
          s_b1 = r;
          s_alast = alast;
        }
      }
    } else {
      const uint32_t w = __ldg(A + i0), alast = __ldg(A + i1 - 1);
      const bool dense = alast - w < SPAN;
      const int tt = t - 64;  // 0 .. NT-65
      constexpr int NS = NT - 64;
      // aligned body [v0, v1) by 16-byte loads; the ragged ends by plain loads
      uint64_t v0, v1;
      aligned_body(A, i0, i1, v0, v1);
      auto put = [&](uint64_t i, uint32_t x) {
        if (dense) {
          const uint32_t o = x - w;
          atomicOr(&tab[o >> 5], 1u << (o & 31));
        } else {
          tab[i - i0] = x;
        }
      };
      if (v0 < v1) {
        for (uint64_t i = i0 + uint64_t(tt); i < v0; i += NS) put(i, __ldg(A + i));
        for (uint64_t i = v1 + uint64_t(tt); i < i1; i += NS) put(i, __ldg(A + i));
        for (uint64_t i = v0 + 4 * uint64_t(tt); i < v1; i += 4 * uint64_t(NS)) {
          const uint4 x = __ldcs(reinterpret_cast<const uint4 *>(A + i));
          put(i, x.x);
          put(i + 1, x.y);
          put(i + 2, x.z);
          put(i + 3, x.w);
        }
      } else {
        for (uint64_t i = i0 + uint64_t(tt); i < i1; i += NS) put(i, __ldg(A + i));
      }
    }
    __syncthreads();
    const uint32_t w = s_w, alast = s_alast;
    const bool dense = alast - w < SPAN;
    const uint32_t span = alast - w;
    const uint64_t b0 = s_b0, b1 = s_b1 > s_b0 ? s_b1 : s_b0;

    // ---- 2. probe B[b0, b1) ----
    auto probe = [&](uint32_t x) {
      bool hit;
      uint32_t pos;  // M bit: value offset (dense) or A position (sparse)
      if (dense) {
        pos = x - w;  // <= span: x is in [w, alast]
        hit = (tab[pos >> 5] >> (pos & 31)) & 1u;
      } else {
        uint32_t lo = 0, len = ntile;
        while (len > 0) {
          const uint32_t h = len >> 1;
          if (tab[lo + h] < x) {
            lo += h + 1;
            len -= h + 1;
          } else {
            len = h;
          }
        }
        pos = lo;
        hit = lo < ntile && tab[lo] == x;
      }
      if (hit) {
        if (MAT) atomicOr(&mbits[pos >> 5], 1u << (pos & 31));
        else ++cnt;
      }
    };
    {
      uint64_t v0, v1;
      aligned_body(B, b0, b1, v0, v1);
      if (v0 < v1) {
        for (uint64_t i = b0 + uint64_t(t); i < v0; i += NT) probe(__ldg(B + i));
        for (uint64_t i = v1 + uint64_t(t); i < b1; i += NT) probe(__ldg(B + i));
        const uint4 *B4 = reinterpret_cast<const uint4 *>(B + v0);  // 16-byte aligned
        const uint64_t n4 = (v1 - v0) / 4;
        uint64_t u = uint64_t(t);
        for (; u + NT < n4; u += 2 * NT) {  // two loads in flight
          const uint4 x = __ldcs(B4 + u), y = __ldcs(B4 + u + NT);
          probe(x.x); probe(x.y); probe(x.z); probe(x.w);
          probe(y.x); probe(y.y); probe(y.z); probe(y.w);
        }
        if (u < n4) {
          const uint4 x = __ldcs(B4 + u);
          probe(x.x); probe(x.y); probe(x.z); probe(x.w);
        }
      } else {
        for (uint64_t i = b0 + uint64_t(t); i < b1; i += NT) probe(__ldg(B + i));
      }
    }
    __syncthreads();

    // ---- 3. output (materialise): M in order -> staging at i0 ----
    const uint32_t mw = dense ? (span >> 5) + 1 : (ntile + 31) / 32;  // M words in use
    if (MAT) {
      // thread t owns M words [t*per, t*per + per)
      const uint32_t per = (mw + NT - 1) / NT;
      const uint32_t m0 = uint32_t(t) * per;
      const uint32_t m1 = (m0 + per < mw) ? m0 + per : mw;
      uint32_t pc = 0;
      for (uint32_t i = m0; i < m1; ++i) pc += __popc(mbits[i]);
      // block scan of pc
      uint32_t incl = pc;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      if (lane == 31) warp_sums[warp] = incl;
      __syncthreads();
      uint32_t before = 0, tot = 0;
#pragma unroll
      for (int k = 0; k < NW; ++k) {
        const uint32_t s = warp_sums[k];
        before += (k < warp) ? s : 0u;
        tot += s;
      }
      uint64_t q = i0 + before + incl - pc;
      for (uint32_t i = m0; i < m1; ++i) {
        uint32_t m = mbits[i];
        if (!m) continue;
        mbits[i] = 0;
        while (m) {
          const uint32_t pos = i * 32u + uint32_t(__ffs(m) - 1);
          m &= m - 1;
          p.stage[q++] = dense ? w + pos : tab[pos];
        }
      }
      if (t == 0) p.status[tile] = tot;  // read after the grid barrier
    }
    // clear T for the next tile (dense: the words used; sparse: the tile,
    // which the output step above may still be reading)
    if (MAT && !dense) __syncthreads();
    {
      const uint32_t tw = dense ? (span >> 5) + 1 : ntile;
      for (uint32_t i = 4u * uint32_t(t); i < tw; i += 4u * NT)
        *reinterpret_cast<uint4 *>(tab + i) = make_uint4(0, 0, 0, 0);
    }
  }

  // ---- combine ----
  if (!MAT) {
    uint64_t v = cnt;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (t == 0) {
      unsigned long long s = 0;
      for (int k = 0; k < NW; ++k) s += red[k];
      if (s) atomicAdd(&p.sync->acc, s);
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

  // Materialise: place the tiles.  The launch is cooperative, so all CTAs
  // are resident and grid-wide barriers are safe.  After every tile is
  // staged (barrier 1), CTA c sums the counts of the contiguous block of
  // tiles [c*K, c*K + K) and publishes the block total; after barrier 2 it
  // adds up the totals of blocks 0..c-1 -- plain loads, nothing to wait
  // for -- and copies its tiles' staged matches to their offsets.
  if (!grid_barrier(&p.sync->done, G, p.err)) return;
  const uint32_t nt32 = uint32_t(ntiles);
  const uint32_t K = (nt32 + G - 1) / G;
  const uint32_t r0 = (blockIdx.x * K < nt32) ? blockIdx.x * K : nt32;
  const uint32_t r1 = (r0 + K < nt32) ? r0 + K : nt32;
  auto block_sum = [&](uint64_t v) -> uint64_t {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    uint64_t s = 0;
#pragma unroll
    for (int q = 0; q < NW; ++q) s += red[q];
    __syncthreads();  // red is reused
    return s;
  };
  uint64_t mine = 0;
  for (uint32_t j = r0 + uint32_t(t); j < r1; j += NT) mine += p.status[j];
  const uint64_t block_total = block_sum(mine);
  if (t == 0) p.coranks[blockIdx.x] = block_total;
  if (!grid_barrier(&p.sync->done, 2 * G, p.err)) return;
  uint64_t before = 0;
  for (uint32_t c = uint32_t(t); c < blockIdx.x; c += NT) before += p.coranks[c];
  const uint64_t ex = block_sum(before);
  if (ex + block_total > p.out_cap) {
    if (t == 0) record_error(p.err, DEV_ERR_CAPACITY);
  } else {
    uint64_t off = ex;
    for (uint32_t j = r0; j < r1; ++j) {
      const uint32_t ck = uint32_t(p.status[j]);  // the same word for every thread
      const uint32_t *src = p.stage + uint64_t(j) * TA;
      for (uint32_t q = uint32_t(t); q < ck; q += NT) p.out[off + q] = src[q];
      off += ck;
    }
    // the last block's end is the total
    if (blockIdx.x == G - 1 && t == 0) *p.out_len = ex + block_total;
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

}  // namespace setops
