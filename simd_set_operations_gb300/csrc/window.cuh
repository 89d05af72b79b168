// window.cuh -- tiled bitmap intersection of two large sorted, duplicate-free
// u32 arrays with B read in speculative windows.  Same result as naive_merge
// (setops/src/intersect/merge.rs:7-33) with the Counter or writer visitors
// (setops/src/visitor.rs:24-49, 759-950): the same elements, ascending.
//
// Work layout
// -----------
// A is the smaller input.  CTA c of the G resident CTAs owns the run
// A[c*na/G, (c+1)*na/G); its first B index b0 (the first B value >= the
// run's first value, or a little below it) is found once, by one warp, while
// the other warps load the first A tile.  Then, tile by tile (TA = 4*UA*NT
// elements of A, values [w, alast]):
//
//   1. every thread loads UA 16-byte words of the tile (all loads in flight
//      at once) and sets their bits in bitmap T: one bit per value when the
//      tile's span alast - w is below 32*VW (dense); else (COARSE) one bit
//      per 2^sh values for the least sh that fits, and the tile is also kept
//      as a sorted table in a second shared-memory region (without COARSE
//      the sorted tile takes T's place);
//   2. B is read from the current position b in windows of 4*UB*NT elements
//      (UB 16-byte loads per thread in flight): each element tests its bit in
//      T (an element below w or above alast lands on a zero bit: the index is
//      clamped onto a zero word).  In a dense tile a set bit is a match; in
//      a COARSE sparse one it is a candidate (a few per cent of the elements,
//      since T is at most 1/32 full), and each lane binary-searches the
//      sorted table for its candidates one at a time (without COARSE every
//      element of a sparse tile searches it).  The
//      window is a guess -- the tile's B range is not searched for -- so the
//      elements up to alast are counted: sorted, they are a prefix of the
//      window, b moves past them, and when the whole window was used the
//      next window follows.  An element above alast is read again by the
//      next tile (from L2; it was just loaded);
//   3. count mode counts; materialise mode appends each window's matches,
//      in B's order (= value order), to the CTA's staging run, which starts
//      at the CTA's first A index (an exclusive region): each warp reads a
//      contiguous part of the window, so a ballot per load round places a
//      lane's matches within its warp and the warps' match totals, exchanged
//      at the window's barrier, place the warps -- no bitmap of matches and
//      no extraction pass;
//   4. T is cleared.
//
// So a tile costs two rounds of loads (A, then B) and no search, and every
// thread keeps four 16-byte loads in flight.  Materialise mode then
// publishes each CTA's count, passes one grid-wide barrier (cooperative
// launch: every CTA resident) and copies the CTA's staged run to the sum of
// its predecessors' counts.  Count mode adds per-CTA totals atomically.
//
// 16-byte loads need 16-byte aligned addresses: a tile's or window's at most
// three elements before the first aligned word and after the last are read
// with plain loads, so any 4-byte alignment works and no load reaches past
// either array.
#pragma once

#include "tile.cuh"

namespace setops {

// COARSE: a tile too wide for one bit per value gets one bit per 2^sh values
// and a sorted copy in shared memory (a second region); otherwise the sorted
// tile takes T's place and every B element searches it.
template <int NT, int UA, int UB, int VW, bool MAT, bool COARSE = false>
struct WindowCfg {
  static_assert(NT % 32 == 0 && NT >= 64, "whole warps");
  static_assert(UA >= 1 && UB >= 1, "loads per thread");
  static constexpr int kTile = 4 * UA * NT;    // A elements per tile (aligned body)
  static constexpr int kWindow = 4 * UB * NT;  // B elements per window (aligned body)
  static_assert((VW & (VW - 1)) == 0 && (COARSE || VW >= kTile),
                "power-of-two bitmap; without COARSE a sparse tile (+6 end elements) fits T");
  static constexpr uint32_t kSpan = uint32_t(VW) * 32u;
  static constexpr int kTabWords = VW + 8;
  static constexpr int kSortWords = COARSE ? kTile + 8 : 0;  // the sorted tile (+6 end elements)
  static_assert(UB * 4 <= 30, "a thread's window hits fit one mask word");
  static constexpr size_t kSmemBytes = size_t(kTabWords + kSortWords) * 4;
};

template <int NT, int UA, int UB, int VW, int MINB, bool MAT, bool COARSE = false>
__global__ void __launch_bounds__(NT, MINB) window_kernel(const MergeArgs p) {
  using Cfg = WindowCfg<NT, UA, UB, VW, MAT, COARSE>;
  constexpr int NW = NT / 32;
  constexpr uint32_t SPAN = Cfg::kSpan;
  constexpr uint32_t TA = Cfg::kTile;

  extern __shared__ __align__(128) uint32_t smem[];
  uint32_t *tab = smem;  // T: one bit per 2^sh values of the tile
  uint32_t *srt = COARSE ? smem + Cfg::kTabWords : smem;  // the sorted tile (sparse)
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

  for (int i = t; i < Cfg::kTabWords / 4; i += NT)
    reinterpret_cast<uint4 *>(smem)[i] = make_uint4(0, 0, 0, 0);
  if (t < 3) s_le[t] = 0;
  __syncthreads();  // T zero before any thread inserts

  // the run's aligned body [v0, v1): tile k covers [v0 + k*TA, v0 + (k+1)*TA)
  // of it; the head [ca0, v0) joins tile 0 and the tail [v1, ca1) the last
  uint64_t v0, v1;
  aligned_body(A, ca0, ca1, v0, v1);
  const uint32_t ntiles =
      ca1 > ca0 ? uint32_t(v1 > v0 ? (v1 - v0 + TA - 1) / TA : 1) : 0u;
  // 16-byte words: element i of X is in word (xmis + i) / 4 of X4
  const uint64_t amis = (reinterpret_cast<uintptr_t>(A) >> 2) & 3;
  const uint64_t bmis = (reinterpret_cast<uintptr_t>(B) >> 2) & 3;
  const uint4 *A4 = reinterpret_cast<const uint4 *>(reinterpret_cast<uintptr_t>(A) & ~uintptr_t(15));
  const uint4 *B4 = reinterpret_cast<const uint4 *>(reinterpret_cast<uintptr_t>(B) & ~uintptr_t(15));

  // warp 0: b0 = where the run starts reading B, at or a little below the
  // first B index with a value >= A[ca0] (B elements below A[ca0] match
  // nothing in this run), from a guess at the same fraction of B as ca0 is
  // of A
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

  for (uint32_t k = 0; k < ntiles; ++k) {
    // ---- 1. the A tile ----
    const uint64_t body0 = v0 + uint64_t(k) * TA;
    const uint64_t body1 = (body0 + TA < v1) ? body0 + TA : v1;
    const uint64_t e0 = (k == 0) ? ca0 : body0;  // tile [e0, e1)
    const uint64_t e1 = (k + 1 == ntiles) ? ca1 : body1;
    const uint32_t nt = uint32_t(e1 - e0);
    const uint32_t w = __ldg(A + e0), alast = __ldg(A + e1 - 1);
    const uint32_t span = alast - w;
    // T holds one bit per 2^sh values: sh = 0 (exact) when the tile's span
    // fits (dense), else (COARSE) the least shift that makes it fit; then a
    // set bit is only a candidate, checked against the sorted tile
    const bool dense = span < SPAN;
    const uint32_t sh = (COARSE && !dense) ? 32u - __clz(span / SPAN) : 0u;
    const uint32_t ssp = span >> sh;  // T's last bit
    {
      const uint4 *ta = A4 + ((amis + body0) >> 2);  // the body's 16-byte words
      const uint32_t nq = uint32_t((body1 - body0) >> 2);
      const bool full = nq == uint32_t(UA * NT);
      uint4 va[UA];
      if (full) {
#pragma unroll
        for (int u = 0; u < UA; ++u) va[u] = __ldcs(ta + (u * NT + t));
      } else {
#pragma unroll
        for (int u = 0; u < UA; ++u)
          va[u] = uint32_t(u * NT + t) < nq ? __ldcs(ta + (u * NT + t)) : make_uint4(0, 0, 0, 0);
      }
      // head / tail elements (tile 0 / last tile): plain loads
      const uint32_t nh = uint32_t(body0 - e0), ntl = uint32_t(e1 - body1);
      const bool is_h = uint32_t(t) < nh;
      const bool is_t = uint32_t(t) >= 32 && uint32_t(t) < 32 + ntl;
      uint32_t xe = 0;
      if (is_h) xe = __ldg(A + e0 + t);
      else if (is_t) xe = __ldg(A + body1 + (t - 32));
      if (COARSE || dense) {
        // (sorted input: every offset is at most span; the clamp keeps T's
        // bounds)
        auto ins = [&](uint32_t x) {
          const uint32_t o = min((x - w) >> sh, ssp);
          atomicOr(&tab[o >> 5], 1u << (o & 31));
        };
        auto ins4 = [&](const uint4 &v) {
          ins(v.x);
          ins(v.y);
          ins(v.z);
          ins(v.w);
        };
        if (full) {
#pragma unroll
          for (int u = 0; u < UA; ++u) ins4(va[u]);
        } else {
#pragma unroll
          for (int u = 0; u < UA; ++u)
            if (uint32_t(u * NT + t) < nq) ins4(va[u]);
        }
        if (is_h || is_t) ins(xe);
      }
      if (!dense) {
        // the tile itself, in order
#pragma unroll
        for (int u = 0; u < UA; ++u) {
          const uint32_t qq = uint32_t(u * NT + t);
          if (qq < nq) {  // (tile 0 may start up to three head elements in: 4-byte stores)
            uint32_t *d = srt + nh + 4 * qq;
            d[0] = va[u].x;
            d[1] = va[u].y;
            d[2] = va[u].z;
            d[3] = va[u].w;
          }
        }
        if (is_h) srt[t] = xe;
        else if (is_t) srt[uint32_t(body1 - e0) + (t - 32)] = xe;
      }
    }
    __syncthreads();
    if (k == 0) b = s_b0;

    // ---- 2. B windows from b ----
    // Each element is probed; the elements up to alast are counted in whole
    // 16-byte words (a word counts when its last element is at most alast),
    // so b may stop up to three elements short of the first element above
    // alast.  Those elements are below the next tile's first value: probed
    // again, they match nothing.
    //
    // Warp w takes a contiguous part of the window body, UB*32 16-byte
    // words.  Count mode: round u, lane l loads word u*32 + l of it (32
    // consecutive words per warp load).  Materialise mode: lane l loads words
    // l*UB .. l*UB + UB-1 (consecutive for the lane; the strided warp loads
    // go through L1, so each sector still comes from L2 once), so the
    // window's elements are in the order (head, warp, lane, element, tail),
    // which is B's order.  Matches are written in that order straight to the
    // staging run: one bit-plane ballot scan of the lanes' match counts
    // places them within the warp, and the warps' totals (exchanged at the
    // window's barrier) place the warps.
    // T's bit for x (an element outside [w, alast] lands on a zero bit past
    // T's last; with sh > 0 a set bit is a candidate)
    auto probe = [&](uint32_t x) -> uint32_t {
      const uint32_t o = min((x - w) >> sh, ssp + 1);
      return __funnelshift_r(tab[o >> 5], 0u, o) & 1u;
    };
    // x in the sorted tile
    auto in_tile = [&](uint32_t x) -> bool {
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
      return lo < nt && srt[lo] == x;
    };
    for (;;) {
      if (b >= nb) break;
      // window [b, we): aligned words [qa, qe) plus plain-loaded ends
      const uint64_t ab = b + ((4 - ((bmis + b) & 3)) & 3);  // first aligned index >= b
      const uint64_t ha = ab < nb ? ab : nb;                 // head [b, ha)
      const uint64_t qa = (bmis + ha) >> 2;
      const uint64_t nbq = (bmis + nb) >> 2;                 // words wholly inside B
      const uint64_t qe = (qa + UB * NT < nbq) ? qa + UB * NT : nbq;
      const uint64_t bodyend = qe > qa ? (qe << 2) - bmis : ha;
      // the tail after the last whole word belongs to the window only when
      // the window reaches B's end
      const uint64_t we = (qe == nbq) ? nb : bodyend;
      const uint32_t nq = uint32_t(qe - qa);
      const uint32_t wb0 = uint32_t(warp) * uint32_t(UB * 32);  // this warp's first word
      const uint4 *wq = B4 + qa + wb0;
      const bool full = nq == uint32_t(UB * NT);
      // word of round u within the warp's part
      auto wi = [&](int u) -> uint32_t {
        return MAT ? uint32_t(lane * UB + u) : uint32_t(u * 32 + lane);
      };
      uint32_t le = 0;  // elements up to alast: head / tail one by one, words x4
      uint32_t hm = 0;  // bit 4u + k = element k of round u matched; bit 30 = xe
      uint4 vb[UB];
      auto ld = [&](int u) { return MAT ? __ldg(wq + wi(u)) : __ldcs(wq + wi(u)); };
      if (full) {
#pragma unroll
        for (int u = 0; u < UB; ++u) vb[u] = ld(u);
      } else {
#pragma unroll
        for (int u = 0; u < UB; ++u) vb[u] = wb0 + wi(u) < nq ? ld(u) : make_uint4(0, 0, 0, 0);
      }
      // head elements on warp 0, tail elements on the last warp
      const uint32_t nh = uint32_t(ha - b), ntl = uint32_t(we - bodyend);
      const bool is_h = warp == 0 && uint32_t(lane) < nh;
      const bool is_t = warp == NW - 1 && uint32_t(lane) < ntl;
      uint32_t xe = 0;
      if (is_h) xe = __ldg(B + b + lane);
      else if (is_t) xe = __ldg(B + bodyend + lane);
      auto run = [&](auto pr) {
#pragma unroll
        for (int u = 0; u < UB; ++u) {
          if (full || wb0 + wi(u) < nq) {
            const uint4 v = vb[u];
            hm |= (pr(v.x) | (pr(v.y) << 1) | (pr(v.z) << 2) | (pr(v.w) << 3)) << (4 * u);
            le += v.w <= alast ? 4u : 0u;
          }
        }
        if (is_h || is_t) {
          hm |= pr(xe) << 30;
          le += xe <= alast ? 1u : 0u;
        }
      };
      if (COARSE || dense) run(probe);
      else run([&](uint32_t x) -> uint32_t { return in_tile(x) ? 1u : 0u; });
      if (COARSE && !dense) {
        // candidates, one at a time: the element of bit c (4u + k, or 30 for
        // xe) by selects, then the sorted tile
        uint32_t cand = hm, ok = 0;
        while (cand) {
          const uint32_t c = uint32_t(__ffs(cand)) - 1u;
          cand &= cand - 1u;
          uint32_t x = xe;
#pragma unroll
          for (int u = 0; u < UB; ++u) {
            const uint32_t q = c - 4u * uint32_t(u);
            x = q == 0u ? vb[u].x : x;
            x = q == 1u ? vb[u].y : x;
            x = q == 2u ? vb[u].z : x;
            x = q == 3u ? vb[u].w : x;
          }
          if (in_tile(x)) ok |= 1u << c;
        }
        hm = ok;
      }
      if (!MAT) cnt += uint32_t(__popc(hm));
      // one barrier per window: slot wc%3 sums this window; the slot of two
      // windows on is cleared (its last readers passed this barrier)
      le = __reduce_add_sync(0xffffffffu, le);
      if (lane == 0 && le) atomicAdd(&s_le[wc], le);
      if (MAT) {
        const uint32_t wt = __reduce_add_sync(0xffffffffu, uint32_t(__popc(hm)));
        if (lane == 0) s_wt[wc][warp] = wt;
      }
      __syncthreads();
      const uint32_t used = s_le[wc];
      if (MAT) {
        uint32_t before = 0, wtot = 0;  // matches of the warps before this one; of all
#pragma unroll
        for (int q = 0; q < NW; ++q) {
          const uint32_t x = s_wt[wc][q];
          before += (q < warp) ? x : 0u;
          wtot += x;
        }
        uint64_t o = staged + before;  // this warp's next output position
        const uint32_t lt = (1u << lane) - 1u;
        // one segment's matches: lane counts c (< 32) scanned over the warp by
        // bit-plane ballots; all lanes of the warp call it
        auto place = [&](uint32_t c, uint32_t &ex, uint32_t &tot) {
          ex = 0;
          tot = 0;
#pragma unroll
          for (int bit = 0; bit < 5; ++bit) {
            const unsigned pl = __ballot_sync(0xffffffffu, (c >> bit) & 1u);
            ex += uint32_t(__popc(pl & lt)) << bit;
            tot += uint32_t(__popc(pl)) << bit;
          }
        };
        uint32_t ex, tot;
        if (warp == 0) {  // head first
          const uint32_t hh = is_h ? (hm >> 30) & 1u : 0u;
          const unsigned pl = __ballot_sync(0xffffffffu, hh);
          if (hh) dst[o + uint32_t(__popc(pl & lt))] = xe;
          o += uint32_t(__popc(pl));
        }
        const uint32_t hb = hm & ((1u << (4 * UB)) - 1u);  // body matches, lane order
        place(uint32_t(__popc(hb)), ex, tot);
        {
          uint64_t q = o + ex;
#pragma unroll
          for (int u = 0; u < UB; ++u) {
            const uint4 v = vb[u];
            const uint32_t h = (hb >> (4 * u)) & 0xFu;
            if (h & 1u) dst[q++] = v.x;
            if (h & 2u) dst[q++] = v.y;
            if (h & 4u) dst[q++] = v.z;
            if (h & 8u) dst[q++] = v.w;
          }
        }
        o += tot;
        if (warp == NW - 1) {  // tail last
          const uint32_t th = is_t ? (hm >> 30) & 1u : 0u;
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

    // ---- 3. clear T (the words used; without COARSE a sparse tile's table) ----
    {
      const uint32_t tw = (COARSE || dense) ? (ssp >> 5) + 1 : nt;
      for (uint32_t i = uint32_t(t); i < tw; i += NT) tab[i] = 0;
    }
    __syncthreads();  // T clear before the next tile's insertion
  }

  // ---- combine ----
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
    // barrier), four independent loads per thread per step
    uint64_t before = 0;
    {
      uint32_t c = uint32_t(t);
      for (; c + 3 * NT < blockIdx.x; c += 4 * NT)
        before += (p.coranks[c] + p.coranks[c + NT]) + (p.coranks[c + 2 * NT] + p.coranks[c + 3 * NT]);
      for (; c < blockIdx.x; c += NT) before += p.coranks[c];
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
