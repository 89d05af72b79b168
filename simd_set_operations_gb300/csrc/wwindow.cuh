// wwindow.cuh -- the window intersection with every warp on its own.  Same
// result as naive_merge (setops/src/intersect/merge.rs:7-33) with the
// Counter or writer visitors (setops/src/visitor.rs:24-49, 759-950): the
// same elements, ascending.
//
// Work layout
// -----------
// A is the smaller input, seen as 16-byte words.  Warp g of the G*NW warps
// of the grid owns the run A[g*na/(G*NW), (g+1)*na/(G*NW)) and a bitmap
// region of its own in shared memory; nothing is shared between the warps of
// a CTA until the run is done, so a warp waiting on memory never holds up
// another (no block-wide barrier in the loop).  The warp finds where to start
// reading B once (at most sqrt(nb)/8 elements below the first B index with a
// value >= the run's first value, from one round of probes around a guess;
// the elements read early are below every value of the run and match
// nothing), then walks its run tile by tile (UA*32 words of A):
//
//   1. every lane loads UA words of the tile (coalesced, all in flight at
//      once) together with the tile's first and last values w and alast, and
//      the first B window (UB*32 words from the current B word) goes out with
//      them; the tile's values are set in the bitmap T (dense: alast - w <
//      32*VWW) or stored as a sorted table (sparse);
//   2. each B element tests its bit in T or binary-searches the table.  A
//      window is a guess: the words whose last element is at most alast are
//      counted -- sorted, they are a prefix of the window -- and the B word
//      moves past them; when the whole window was used the next follows;
//   3. count mode counts; materialise mode appends each window's matches, in
//      B's order, to the warp's staging run (at its first A index: an
//      exclusive region), placed within the warp by a ballot scan;
//   4. T is cleared.
//
// Whole words are read: elements of a tile's first and last word outside
// the tile are inserted too, but they lie below w or above alast, so in a
// dense tile they land on alast's bit (set anyway) and a sparse probe
// rejects values outside [w, alast]; B elements before the B word's first
// unconsumed element were consumed by an earlier tile and are below w.  The
// only words read element by element are those that stick out of an array
// (at its start or end when it is not 16-byte aligned): no load reaches
// outside either array.
//
// Materialise mode then publishes each CTA's count (the sum of its warps'),
// passes one grid-wide barrier (cooperative launch) and copies every warp's
// staged run to the sum of the counts before it.  Count mode adds per-CTA
// totals atomically.
#pragma once

#include "tile.cuh"

namespace setops {

template <int NT, int UA, int UB, int VWW, bool MAT>
struct WWindowCfg {
  static_assert(NT % 32 == 0 && NT >= 32, "whole warps");
  static_assert(UA >= 1 && UB >= 1 && UB * 4 <= 30, "a lane's window hits fit one mask word");
  static constexpr int kWarps = NT / 32;
  static constexpr int kTileWords = UA * 32;  // A words per warp tile
  static constexpr int kWinWords = UB * 32;   // B words per window
  static_assert((VWW & (VWW - 1)) == 0 && VWW >= 4 * kTileWords, "a sparse tile fits the region");
  static constexpr uint32_t kSpan = uint32_t(VWW) * 32u;  // values per dense tile
  static constexpr int kRegion = VWW + 8;  // words per warp: dense probes reach word VWW
  static constexpr size_t kSmemBytes = size_t(kWarps) * kRegion * 4;
  // grid sizing unit: a run of at least 32 A elements per warp (every warp
  // streams its own B range, so a skewed pair still spreads over the GPU)
  static constexpr int kTile = 32 * kWarps;
};

// Word q of X (n elements; element i is component (mis + i) & 3 of 16-byte
// word (mis + i) >> 2) for a word that sticks out of X: the elements outside
// X read `before` (ahead of X[0]) or `after` (past X[n-1]); bit c of
// *outside marks component c as outside.
__device__ __forceinline__ uint4 load_edge_word(const uint32_t *X, uint64_t n, uint64_t mis,
                                                uint64_t q, uint32_t before, uint32_t after,
                                                uint32_t *outside) {
  uint32_t e[4];
  uint32_t m = 0;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int64_t i = int64_t(4 * q + uint64_t(c)) - int64_t(mis);
    if (i < 0) {
      e[c] = before;
      m |= 1u << c;
    } else if (uint64_t(i) >= n) {
      e[c] = after;
      m |= 1u << c;
    } else {
      e[c] = __ldg(X + i);
    }
  }
  *outside = m;
  return make_uint4(e[0], e[1], e[2], e[3]);
}

template <int NT, int UA, int UB, int VWW, int MINB, bool MAT>
__global__ void __launch_bounds__(NT, MINB) wwindow_kernel(const MergeArgs p) {
  using Cfg = WWindowCfg<NT, UA, UB, VWW, MAT>;
  constexpr int NW = Cfg::kWarps;
  constexpr uint32_t SPAN = Cfg::kSpan;
  constexpr uint32_t TW = Cfg::kTileWords, WW = Cfg::kWinWords;

  extern __shared__ __align__(128) uint32_t smem[];
  __shared__ unsigned long long s_cnt[NW];  // per warp: its matches
  __shared__ unsigned long long red[NW];

  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  uint32_t *tab = smem + warp * Cfg::kRegion;  // this warp's T / sorted tile

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
  const uint64_t GW = uint64_t(G) * NW;
  const uint64_t gw = uint64_t(blockIdx.x) * NW + uint64_t(warp);
  const uint64_t ra0 = nb ? gw * na / GW : 0, ra1 = nb ? (gw + 1) * na / GW : 0;

  for (int i = lane; i < Cfg::kRegion; i += 32) tab[i] = 0;
  __syncwarp();

  // 16-byte words: element i of X is component (xmis + i) & 3 of word
  // (xmis + i) >> 2 of X4; nwx words touch X; the first sticks out when xmis
  // is non-zero, the last when (xmis + nx) & 3 is
  const uint64_t amis = (reinterpret_cast<uintptr_t>(A) >> 2) & 3;
  const uint64_t bmis = (reinterpret_cast<uintptr_t>(B) >> 2) & 3;
  const uint4 *A4 = reinterpret_cast<const uint4 *>(reinterpret_cast<uintptr_t>(A) & ~uintptr_t(15));
  const uint4 *B4 = reinterpret_cast<const uint4 *>(reinterpret_cast<uintptr_t>(B) & ~uintptr_t(15));
  const uint64_t nwa = (amis + na + 3) >> 2, nwb = (bmis + nb + 3) >> 2;
  const bool a_tail = ((amis + na) & 3) != 0, b_tail = ((bmis + nb) & 3) != 0;

  uint32_t cnt = 0;     // count mode: this lane's matches
  uint64_t staged = 0;  // materialise: this warp's staged matches
  uint32_t *dst = MAT ? p.stage + ra0 : nullptr;

  if (ra1 > ra0) {
    const uint64_t q0 = (amis + ra0) >> 2, q1 = ((amis + ra1 - 1) >> 2) + 1;  // run's A words
    const uint32_t ntiles = uint32_t((q1 - q0 + TW - 1) / TW);

    // ---- A tile k: words [qt, qt + nqa), elements [e0, e1) ----
    uint4 va[UA];
    uint32_t nqa = 0, w = 0, alast = 0;
    auto load_tile = [&](uint32_t k) {
      const uint64_t qt = q0 + uint64_t(k) * TW;
      nqa = uint32_t((q1 - qt < TW) ? q1 - qt : TW);
      const uint64_t e0 = (k == 0) ? ra0 : 4 * qt - amis;
      const uint64_t e1 = (k + 1 == ntiles) ? ra1 : 4 * (qt + TW) - amis;
      w = __ldg(A + e0);
      alast = __ldg(A + e1 - 1);
      const bool edge = (qt == 0 && amis != 0) || (qt + nqa == nwa && a_tail);
      if (!edge && nqa == TW) {
#pragma unroll
        for (int u = 0; u < UA; ++u) va[u] = __ldcs(A4 + qt + uint32_t(u * 32 + lane));
      } else {
#pragma unroll
        for (int u = 0; u < UA; ++u) {
          const uint32_t j = uint32_t(u * 32 + lane);
          uint32_t outside;
          va[u] = j >= nqa ? make_uint4(0, 0, 0, 0)
                  : edge   ? load_edge_word(A, na, amis, qt + j, 0u, 0xffffffffu, &outside)
                           : __ldcs(A4 + qt + j);
        }
      }
    };
    load_tile(0);  // in flight during the search

    // ---- the run's first B word: at or a little below the first B index
    // with a value >= A[ra0] (B elements below it match nothing in this
    // run), from a guess at the same fraction of B as ra0 is of A ----
    uint64_t qb;
    {
      const uint64_t est = guess_scale(ra0, na, nb);
      qb = (bmis + warp_start_below(B, nb, A + ra0, est)) >> 2;
    }

    // ---- B window: words [qb, qb + nqb) ----
    // count mode: round u, lane l holds word u*32 + l (coalesced); materialise:
    // lane l holds words l*UB .. l*UB + UB-1, so (lane, round, component) is
    // B's order
    uint4 vb[UB];
    uint32_t nqb = 0;
    uint32_t outb = 0;  // bit 4u + c: component c of round u lies outside B
    auto wi = [&](int u) -> uint32_t {
      return MAT ? uint32_t(lane * UB + u) : uint32_t(u * 32 + lane);
    };
    auto issue = [&]() {
      nqb = uint32_t((nwb - qb < WW) ? nwb - qb : WW);
      const bool edge = (qb == 0 && bmis != 0) || (qb + nqb == nwb && b_tail);
      outb = 0;
      if (!edge && nqb == WW) {
#pragma unroll
        for (int u = 0; u < UB; ++u) vb[u] = MAT ? __ldg(B4 + qb + wi(u)) : __ldcs(B4 + qb + wi(u));
      } else {
        const uint32_t blast_v = edge ? __ldg(B + nb - 1) : 0u;
#pragma unroll
        for (int u = 0; u < UB; ++u) {
          const uint32_t j = wi(u);
          uint32_t o = 0;
          vb[u] = j >= nqb ? make_uint4(0, 0, 0, 0)
                  : edge   ? load_edge_word(B, nb, bmis, qb + j, 0u, blast_v, &o)
                  : MAT    ? __ldg(B4 + qb + j)
                           : __ldcs(B4 + qb + j);
          outb |= o << (4 * u);
        }
      }
    };

    const uint32_t lt = (1u << lane) - 1u;
    for (uint32_t k = 0; k < ntiles; ++k) {
      if (k > 0) load_tile(k);
      if (qb >= nwb) break;  // B used up: nothing more matches
      issue();               // the tile's first window, with its A loads
      const uint32_t span = alast - w;
      const bool dense = span < SPAN;

      // ---- 1. the tile into T ----
      if (dense) {
        // (values outside [w, alast] clamp onto alast's bit)
        auto ins = [&](uint32_t x) {
          const uint32_t o = min(x - w, span);
          atomicOr(&tab[o >> 5], 1u << (o & 31));
        };
#pragma unroll
        for (int u = 0; u < UA; ++u) {
          if (nqa == TW || uint32_t(u * 32 + lane) < nqa) {
            ins(va[u].x);
            ins(va[u].y);
            ins(va[u].z);
            ins(va[u].w);
          }
        }
      } else {
#pragma unroll
        for (int u = 0; u < UA; ++u) {
          const uint32_t j = uint32_t(u * 32 + lane);
          if (j < nqa) reinterpret_cast<uint4 *>(tab)[j] = va[u];
        }
      }
      __syncwarp();
      const uint32_t ntab = 4 * nqa;  // sparse: sorted entries (edge fills keep the order)

      auto probe_dense = [&](uint32_t x) -> uint32_t {
        const uint32_t o = min(x - w, span + 1);
        return __funnelshift_r(tab[o >> 5], 0u, o) & 1u;
      };
      auto probe_sparse = [&](uint32_t x) -> uint32_t {
        uint32_t lo = 0, len = ntab;
        while (len > 0) {
          const uint32_t hh = len >> 1;
          if (tab[lo + hh] < x) {
            lo += hh + 1;
            len -= hh + 1;
          } else {
            len = hh;
          }
        }
        return (x >= w && x <= alast && lo < ntab && tab[lo] == x) ? 1u : 0u;
      };

      // ---- 2./3. windows ----
      for (;;) {
        uint32_t le = 0;  // this lane's words whose last element is at most alast
        uint32_t hm = 0;  // bit 4u + c: component c of round u matched
        auto run = [&](auto probe) {
#pragma unroll
          for (int u = 0; u < UB; ++u) {
            if (nqb == WW || wi(u) < nqb) {
              const uint4 v = vb[u];
              const uint32_t h =
                  probe(v.x) | (probe(v.y) << 1) | (probe(v.z) << 2) | (probe(v.w) << 3);
              hm |= h << (4 * u);
              le += v.w <= alast ? 1u : 0u;
            }
          }
        };
        if (dense) run(probe_dense);
        else run(probe_sparse);
        hm &= ~outb;
        const uint32_t used = __reduce_add_sync(0xffffffffu, le);
        if (MAT) {
          // lane counts (< 32) scanned over the warp by bit-plane ballots
          const uint32_t c = uint32_t(__popc(hm));
          uint32_t ex = 0, tot = 0;
#pragma unroll
          for (int bit = 0; bit < 5; ++bit) {
            const unsigned pl = __ballot_sync(0xffffffffu, (c >> bit) & 1u);
            ex += uint32_t(__popc(pl & lt)) << bit;
            tot += uint32_t(__popc(pl)) << bit;
          }
          uint64_t q = staged + ex;
#pragma unroll
          for (int u = 0; u < UB; ++u) {
            const uint4 v = vb[u];
            const uint32_t h = (hm >> (4 * u)) & 0xFu;
            if (h & 1u) dst[q++] = v.x;
            if (h & 2u) dst[q++] = v.y;
            if (h & 4u) dst[q++] = v.z;
            if (h & 8u) dst[q++] = v.w;
          }
          staged += tot;
        } else {
          cnt += uint32_t(__popc(hm));
        }
        qb += used;
        // a word above alast, or B's end: the tile is done
        if (used < nqb || qb >= nwb) break;
        issue();
      }

      // ---- 4. clear T (dense: the words used; sparse: the table) ----
      const uint32_t tw = dense ? (span >> 5) + 1 : ntab;
      for (uint32_t i = uint32_t(lane); i < tw; i += 32) tab[i] = 0;
      __syncwarp();
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
    if (lane == 0) s_cnt[warp] = staged;
    __syncthreads();
    uint64_t mine = 0;  // this CTA's matches
#pragma unroll
    for (int q = 0; q < NW; ++q) mine += s_cnt[q];
    if (t == 0) p.coranks[blockIdx.x] = mine;
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
    if (ex + mine > p.out_cap) {
      if (t == 0) record_error(p.err, DEV_ERR_CAPACITY);
    } else {
      uint64_t wo = ex;  // this warp's first output position
      for (int q = 0; q < warp; ++q) wo += s_cnt[q];
      for (uint64_t q = uint64_t(lane); q < staged; q += 32) p.out[wo + q] = p.stage[ra0 + q];
      if (blockIdx.x == G - 1 && t == 0) *p.out_len = ex + mine;
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
