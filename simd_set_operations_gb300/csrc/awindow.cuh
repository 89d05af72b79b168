// awindow.cuh -- the window kernel (window.cuh) with its A tiles prefetched
// into shared memory by asynchronous 16-byte copies.  Same result as
// naive_merge (setops/src/intersect/merge.rs:7-33) with the Counter or writer
// visitors (setops/src/visitor.rs:24-49, 759-950): the same elements,
// ascending.
//
// What changes against window.cuh
// -------------------------------
// The window kernel loads each A tile and then each B window into registers,
// one after the other, so a CTA has loads in flight only in those two phases
// and waits out both latencies on every tile; and its materialise mode tests
// every element of a lane's window part to write the (rare) matches.  Here
// both inputs are copied into shared memory by asynchronous 16-byte copies
// (cp.async through L2):
//
//   * A tile k+1 is copied into its buffer as soon as tile k's insertion has
//     read it, so it arrives while tile k's B windows are probed;
//   * the first B window of tile k is copied while tile k's A elements are
//     inserted into T (from shared memory), so its latency overlaps the
//     insertion;
//   * materialise mode walks the set bits of a lane's match mask and reads
//     each matched element back from the window buffer, instead of testing
//     every element; T is cleared with 16-byte stores.
//
// The partition (one A run per resident CTA, its B start from one round of
// probes), the windows (speculative, counted up to the tile's last value),
// the ordered placement and the grid-wide barrier are the window kernel's.
//
// A tile's elements sit in its buffer at [4, 4 + body): the 16-byte aligned
// body of the tile copied whole words at a time; tile 0's head elements
// (before the first aligned word, at most three) go just below it and the
// last tile's tail just above, by plain loads, so the buffer holds the tile
// in order -- the sorted table of a sparse tile.  A window's aligned words
// sit in the window buffer in order; its head and tail elements (at most
// three each) stay in registers of the first / last warp.
#pragma once

#include "tile.cuh"

namespace setops {

// 16-byte copy global -> shared through L2 only (no L1 allocation), in the
// current cp.async group.  Both addresses 16-byte aligned.
__device__ __forceinline__ void cp_async16(void *dst_smem, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst_smem)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
// Waits for every cp.async group this thread committed.
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

template <int NT, int UA, int UB, int VW, bool MAT>
struct AWindowCfg {
  static_assert(NT % 32 == 0 && NT >= 64, "whole warps");
  static_assert(UA >= 1 && UB >= 1 && UB * 4 <= 30, "loads per thread; window hits in one word");
  static constexpr int kTile = 4 * UA * NT;    // A elements per tile (aligned body)
  static constexpr int kWindow = 4 * UB * NT;  // B elements per window (aligned body)
  static_assert((VW & (VW - 1)) == 0 && VW % 4 == 0, "power-of-two bitmap of whole 16-byte words");
  static constexpr uint32_t kSpan = uint32_t(VW) * 32u;
  static constexpr int kTabWords = VW + 8;       // T, with a zero word past its last bit
  static constexpr int kBufWords = kTile + 8;    // the A tile: 4 head slots, body, tail
  static constexpr int kWinWords = kWindow;      // a B window's aligned words
  static constexpr size_t kSmemBytes = size_t(kTabWords + kBufWords + kWinWords) * 4;
};

template <int NT, int UA, int UB, int VW, int MINB, bool MAT>
__global__ void __launch_bounds__(NT, MINB) awindow_kernel(const MergeArgs p) {
  using Cfg = AWindowCfg<NT, UA, UB, VW, MAT>;
  constexpr int NW = NT / 32;
  constexpr uint32_t SPAN = Cfg::kSpan;
  constexpr uint32_t TA = Cfg::kTile;

  extern __shared__ __align__(128) uint32_t smem[];
  uint32_t *tab = smem;                    // T: one bit per value of a dense tile
  uint32_t *abuf = smem + Cfg::kTabWords;  // the A tile: body at abuf + 4 (16-byte aligned)
  uint4 *wbuf = reinterpret_cast<uint4 *>(abuf + Cfg::kBufWords);  // a B window's words
  __shared__ unsigned long long s_b0;
  __shared__ uint32_t s_le[3];      // B elements of a window up to alast (rotating)
  __shared__ uint32_t s_wt[3][NW];  // materialise: matches of each warp in a window
  __shared__ unsigned long long red[NW];

  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;

  // ---- problem (A = smaller set) ----
  uint64_t na = p.na_dev ? *p.na_dev : p.na;
  uint64_t nb = p.nb_dev ? *p.nb_dev : p.nb;
  const uint32_t *A = p.a, *B = p.b;
  if (na > nb) {
    const uint32_t *tp = A; A = B; B = tp;
    const uint64_t tn = na; na = nb; nb = tn;
  }
  if (skip_by_rule(p.skip_rule, p.ratio_thr, na, nb)) return;
  const uint32_t G = gridDim.x;
  const uint64_t ca0 = nb ? uint64_t(blockIdx.x) * na / G : 0;
  const uint64_t ca1 = nb ? (uint64_t(blockIdx.x) + 1) * na / G : 0;

  uint64_t v0, v1;
  aligned_body(A, ca0, ca1, v0, v1);
  const uint32_t ntiles =
      ca1 > ca0 ? uint32_t(v1 > v0 ? (v1 - v0 + TA - 1) / TA : 1) : 0u;
  const uint64_t amis = (reinterpret_cast<uintptr_t>(A) >> 2) & 3;
  const uint64_t bmis = (reinterpret_cast<uintptr_t>(B) >> 2) & 3;
  const uint4 *A4 = reinterpret_cast<const uint4 *>(reinterpret_cast<uintptr_t>(A) & ~uintptr_t(15));
  const uint4 *B4 = reinterpret_cast<const uint4 *>(reinterpret_cast<uintptr_t>(B) & ~uintptr_t(15));

  // the body of tile kk -> abuf + 4, whole 16-byte words, one cp.async group
  auto prefetch = [&](uint32_t kk) {
    const uint64_t body0 = v0 + uint64_t(kk) * TA;
    const uint64_t body1 = (body0 + TA < v1) ? body0 + TA : v1;
    const uint4 *src = A4 + ((amis + body0) >> 2);
    const uint32_t nq = uint32_t((body1 - body0) >> 2);
    uint4 *dst = reinterpret_cast<uint4 *>(abuf + 4);
#pragma unroll
    for (int u = 0; u < UA; ++u) {
      const uint32_t q = uint32_t(u * NT + t);
      if (q < nq) cp_async16(dst + q, src + q);
    }
    cp_async_commit();
  };

  for (int i = t; i < Cfg::kTabWords / 4; i += NT)
    reinterpret_cast<uint4 *>(tab)[i] = make_uint4(0, 0, 0, 0);
  if (t < 3) s_le[t] = 0;
  if (ntiles) prefetch(0);
  // warp 0: where the run starts reading B (as in window.cuh)
  if (ntiles && warp == 0) {
    const uint64_t est = guess_scale(ca0, na, nb);
    const uint64_t r = warp_start_below(B, nb, A + ca0, est);
    if (lane == 0) s_b0 = r;
  }

  uint32_t cnt = 0;     // count mode: this thread's matches
  uint64_t staged = 0;  // materialise: matches staged so far
  uint32_t *dst = MAT ? p.stage + ca0 : nullptr;
  uint64_t b = 0;       // first B element not yet consumed
  uint32_t wc = 0;      // this window's s_le / s_wt slot (windows so far, mod 3)

  // window state: [b, we) with aligned words [qa, qe), head [b, ha), tail
  // [bodyend, we); vb holds the window's words once loaded
  uint64_t we = 0, bodyend = 0;
  uint32_t nqw = 0, nhw = 0, ntw = 0, xe = 0;
  bool fullw = false, is_hw = false, is_tw = false;
  const uint32_t wb0 = uint32_t(warp) * uint32_t(UB * 32);  // this warp's first word
  auto wi = [&](int u) -> uint32_t {
    return MAT ? uint32_t(lane * UB + u) : uint32_t(u * 32 + lane);
  };
  auto load_window = [&]() {
    const uint64_t ab = b + ((4 - ((bmis + b) & 3)) & 3);  // first aligned index >= b
    const uint64_t ha = ab < nb ? ab : nb;
    const uint64_t qa = (bmis + ha) >> 2;
    const uint64_t nbq = (bmis + nb) >> 2;                 // words wholly inside B
    const uint64_t qe = (qa + UB * NT < nbq) ? qa + UB * NT : nbq;
    bodyend = qe > qa ? (qe << 2) - bmis : ha;
    we = (qe == nbq) ? nb : bodyend;
    nqw = uint32_t(qe - qa);
    fullw = nqw == uint32_t(UB * NT);
    // the aligned words, in order, coalesced copies (word u*NT + t)
    const uint4 *wq = B4 + qa;
#pragma unroll
    for (int u = 0; u < UB; ++u) {
      const uint32_t q = uint32_t(u * NT + t);
      if (q < nqw) cp_async16(wbuf + q, wq + q);
    }
    cp_async_commit();
    nhw = uint32_t(ha - b);
    ntw = uint32_t(we - bodyend);
    is_hw = warp == 0 && uint32_t(lane) < nhw;
    is_tw = warp == NW - 1 && uint32_t(lane) < ntw;
    xe = 0;
    if (is_hw) xe = __ldg(B + b + lane);
    else if (is_tw) xe = __ldg(B + bodyend + lane);
  };

  for (uint32_t k = 0; k < ntiles; ++k) {
    // ---- 1. the A tile (its body is arriving in abuf + 4) ----
    const uint64_t body0 = v0 + uint64_t(k) * TA;
    const uint64_t body1 = (body0 + TA < v1) ? body0 + TA : v1;
    const uint64_t e0 = (k == 0) ? ca0 : body0;  // tile [e0, e1)
    const uint64_t e1 = (k + 1 == ntiles) ? ca1 : body1;
    const uint32_t nt = uint32_t(e1 - e0);
    const uint32_t nbody = uint32_t(body1 - body0);
    const uint32_t nh = uint32_t(body0 - e0), ntl = uint32_t(e1 - body1);
    // head (tile 0) and tail (last tile) elements, at most three each, go
    // just below and above the body: the buffer holds the tile in order
    if (uint32_t(t) < nh) abuf[4 - nh + t] = __ldg(A + e0 + t);
    else if (uint32_t(t) >= 32 && uint32_t(t) < 32 + ntl)
      abuf[4 + nbody + (t - 32)] = __ldg(A + body1 + (t - 32));
    cp_async_wait_all();
    __syncthreads();  // the tile in abuf; T clear; (tile 0) s_b0 set
    if (k == 0) b = s_b0;
    const uint32_t *srt = abuf + 4 - nh;  // the sorted tile, nt elements
    const uint32_t w = srt[0], alast = srt[nt - 1];
    const uint32_t span = alast - w;
    const bool dense = span < SPAN;

    // the tile's first B window, in flight while the tile is inserted
    if (b < nb) load_window();

    if (dense) {
      auto ins = [&](uint32_t x) {
        const uint32_t o = min(x - w, span);  // (sorted input: o <= span already)
        atomicOr(&tab[o >> 5], 1u << (o & 31));
      };
      const uint4 *body4 = reinterpret_cast<const uint4 *>(abuf + 4);
      const uint32_t nq = nbody >> 2;
#pragma unroll
      for (int u = 0; u < UA; ++u) {
        const uint32_t q = uint32_t(u * NT + t);
        if (q < nq) {
          const uint4 v = body4[q];
          ins(v.x);
          ins(v.y);
          ins(v.z);
          ins(v.w);
        }
      }
      if (uint32_t(t) < nh) ins(srt[t]);
      else if (uint32_t(t) >= 32 && uint32_t(t) < 32 + ntl) ins(srt[nh + nbody + (t - 32)]);
      cp_async_wait_all();  // this thread's window copies
      __syncthreads();  // T complete; the window in wbuf; abuf read: the next tile may come in
      if (k + 1 < ntiles) prefetch(k + 1);
    } else {
      cp_async_wait_all();
      __syncthreads();  // the window in wbuf
    }

    // ---- 2. B windows from b (window.cuh's scheme) ----
    // T's bit for x (an element outside [w, alast] lands on the zero word
    // past T's last bit)
    auto probe = [&](uint32_t x) -> uint32_t {
      const uint32_t o = min(x - w, span + 1);
      return __funnelshift_r(tab[o >> 5], 0u, o) & 1u;
    };
    // x in the sorted tile (sparse tiles)
    auto in_tile = [&](uint32_t x) -> uint32_t {
      uint32_t lo = 0, len = nt;
      while (len > 0) {
        const uint32_t hh = len >> 1;
        if (srt[lo + hh] < x) {
          lo += hh + 1;
          len -= hh + 1;
        } else {
          len = hh;
        }
      }
      return (lo < nt && srt[lo] == x) ? 1u : 0u;
    };
    bool first = true;
    for (;;) {
      if (b >= nb) break;
      if (!first) {
        __syncthreads();  // every thread done with the last window's buffer
        load_window();
        cp_async_wait_all();
        __syncthreads();  // the window in wbuf
      }
      first = false;
      uint32_t le = 0;  // elements up to alast: head / tail one by one, words x4
      uint32_t hm = 0;  // bit 4u + k = element k of round u matched; bit 30 = xe
      auto run = [&](auto pr) {
#pragma unroll
        for (int u = 0; u < UB; ++u) {
          if (fullw || wb0 + wi(u) < nqw) {
            const uint4 v = wbuf[wb0 + wi(u)];
            hm |= (pr(v.x) | (pr(v.y) << 1) | (pr(v.z) << 2) | (pr(v.w) << 3)) << (4 * u);
            le += v.w <= alast ? 4u : 0u;
          }
        }
        if (is_hw || is_tw) {
          hm |= pr(xe) << 30;
          le += xe <= alast ? 1u : 0u;
        }
      };
      if (dense) run(probe);
      else run(in_tile);
      if (!MAT) cnt += uint32_t(__popc(hm));
      le = __reduce_add_sync(0xffffffffu, le);
      if (lane == 0 && le) atomicAdd(&s_le[wc], le);
      if (MAT) {
        const uint32_t wt = __reduce_add_sync(0xffffffffu, uint32_t(__popc(hm)));
        if (lane == 0) s_wt[wc][warp] = wt;
      }
      __syncthreads();
      const uint32_t used = s_le[wc];
      if (MAT) {
        uint32_t before = 0, wtot = 0;
#pragma unroll
        for (int q = 0; q < NW; ++q) {
          const uint32_t x = s_wt[wc][q];
          before += (q < warp) ? x : 0u;
          wtot += x;
        }
        uint64_t o = staged + before;
        const uint32_t lt = (1u << lane) - 1u;
        if (warp == 0) {  // head first
          const uint32_t hh = is_hw ? (hm >> 30) & 1u : 0u;
          const unsigned pl = __ballot_sync(0xffffffffu, hh);
          if (hh) dst[o + uint32_t(__popc(pl & lt))] = xe;
          o += uint32_t(__popc(pl));
        }
        const uint32_t hb = hm & ((1u << (4 * UB)) - 1u);  // body matches, lane order
        const uint32_t c = uint32_t(__popc(hb));
        // this lane's place among the warp's matches: one ballot when no lane
        // has more than one (the usual case at low selectivity), else a scan
        // of the counts' bit planes
        uint32_t ex, tot;
        const unsigned one = __ballot_sync(0xffffffffu, c != 0);
        if (__ballot_sync(0xffffffffu, c > 1) == 0) {
          ex = uint32_t(__popc(one & lt));
          tot = uint32_t(__popc(one));
        } else {
          ex = 0;
          tot = 0;
#pragma unroll
          for (int bit = 0; bit < 5; ++bit) {
            const unsigned pl = __ballot_sync(0xffffffffu, (c >> bit) & 1u);
            ex += uint32_t(__popc(pl & lt)) << bit;
            tot += uint32_t(__popc(pl)) << bit;
          }
        }
        {
          // bit j = 4u + k of hb is element k of the lane's word u, which
          // sits at element 4 * (wb0 + lane * UB) + j of the window buffer
          const uint32_t *mine =
              reinterpret_cast<const uint32_t *>(wbuf) + 4u * (wb0 + uint32_t(lane) * UB);
          uint64_t q = o + ex;
          for (uint32_t m = hb; m; m &= m - 1u) dst[q++] = mine[__ffs(m) - 1];
        }
        o += tot;
        if (warp == NW - 1) {  // tail last
          const uint32_t th = is_tw ? (hm >> 30) & 1u : 0u;
          const unsigned pl = __ballot_sync(0xffffffffu, th);
          if (th) dst[o + uint32_t(__popc(pl & lt))] = xe;
        }
        staged += wtot;
      }
      if (t == 0) s_le[wc == 0 ? 2 : wc - 1] = 0;  // the slot two windows on
      wc = (wc == 2) ? 0 : wc + 1;
      b += used;
      if (b < we) break;  // an element above alast: the tile is done
    }

    if (dense) {
      // ---- 3. clear the words of T the tile used (16-byte stores) ----
      const uint32_t tq = ((span >> 5) + 4) >> 2;  // 16-byte words covering bits 0..span
      for (uint32_t i = uint32_t(t); i < tq; i += NT)
        reinterpret_cast<uint4 *>(tab)[i] = make_uint4(0, 0, 0, 0);
    } else if (k + 1 < ntiles) {
      // a sparse tile is read in abuf (its ends, its searches) until here
      __syncthreads();
      prefetch(k + 1);
    }
  }

  // ---- combine (window.cuh's) ----
  if (!MAT) {
    uint64_t v = cnt;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (t == 0) {
      unsigned long long sm = 0;
      for (int q = 0; q < NW; ++q) sm += red[q];
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
    if (t == 0) p.coranks[blockIdx.x] = staged;
    if (!grid_barrier(&p.sync->done, G, p.err)) return;
    // counts of CTAs 0..c-1 (plain loads: every CTA published before the
    // barrier): a thread's loads all issued at once, one round trip, for up
    // to 16 * NT CTAs; a larger grid adds a loop for the rest
    uint64_t before = 0;
    {
      constexpr int PL = 16;
      uint64_t w[PL];
#pragma unroll
      for (int j = 0; j < PL; ++j) {
        const uint32_t c = uint32_t(t + j * NT);
        w[j] = c < blockIdx.x ? p.coranks[c] : 0;
      }
#pragma unroll
      for (int j = 0; j < PL; ++j) before += w[j];
      for (uint32_t c = uint32_t(t + PL * NT); c < blockIdx.x; c += NT) before += p.coranks[c];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) before += __shfl_xor_sync(0xffffffffu, before, o);
    if (lane == 0) red[warp] = before;
    __syncthreads();
    uint64_t ex = 0;
#pragma unroll
    for (int q = 0; q < NW; ++q) ex += red[q];
    if (ex + staged > p.out_cap) {
      if (t == 0) record_error(p.err, DEV_ERR_CAPACITY);
    } else {
      for (uint64_t q = uint64_t(t); q < staged; q += NT) p.out[ex + q] = p.stage[ca0 + q];
      if (blockIdx.x == G - 1 && t == 0) *p.out_len = ex + staged;
    }
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
