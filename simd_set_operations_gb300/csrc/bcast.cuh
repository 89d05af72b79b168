// bcast.cuh -- BSR 2-set intersection by block broadcast: the scheme of
// broadcast_{sse,avx2,avx512}_bsr (setops/src/intersect/broadcast.rs:163-357)
// with blocks of 32 bases, one per lane of a warp.  Same result as
// branchless_merge_bsr (setops/src/intersect/merge.rs:62-87): for every base
// in both sets, (base, state_a & state_b) when that is non-zero, in base
// order; count mode gives the Counter visitor's popcount sum
// (setops/src/visitor.rs:399-403).
//
// The reference compares a block of W bases of A with a block of W bases of
// B all against all (W broadcasts), ANDs the states of equal bases, visits
// the block, and then advances A's block when its largest base is at most
// B's largest and B's when B's largest is at most A's.  Here:
//
//   * W = 32: lane l holds A block element l and B block element l in
//     registers; each lane finds its A base among the 32 B bases by a
//     five-step binary search over shuffles (the blocks are sorted), which
//     is the broadcast comparison done in log2(W) steps instead of W;
//   * before comparing, the two blocks' base ranges are tested for overlap
//     and a pair of disjoint blocks is only advanced -- the job of
//     qfilter_bsr's byte-check filter (setops/src/intersect/qfilter.rs:92),
//     which rules out block pairs that cannot match;
//   * the grid's warps take contiguous runs of A's blocks (whole 32-word
//     blocks; the last block of A may be short) and the part of B whose
//     bases fall in their run's range, found by a warp-wide search; each
//     warp streams its two runs with the next blocks prefetched in
//     registers (KD blocks ahead);
//   * a warp's non-zero words are compacted by ballot in A order into the
//     stage buffer at its run's first index; materialise then places the
//     runs (per-CTA totals, one grid barrier, each CTA's prefix in one round
//     of loads).  Blocks past the end of a run hold a sentinel above every
//     base (bases are values >> 5, below 2^27).
#pragma once

#include "merge.cuh"
#include "tile.cuh"

namespace setops {

template <int NT>
struct BcastCfg {
  static_assert(NT % 32 == 0 && NT >= 64, "whole warps");
  static constexpr int kTile = (NT / 32) * 64;  // grid sizing: words of both sets per CTA tile
};

template <int NT, int MINB, int KD, bool MAT>
__global__ void __launch_bounds__(NT, MINB) bcast_bsr_kernel(const MergeArgs p) {
  constexpr int NW = NT / 32;
  constexpr uint32_t SENT = 0xffffffffu;  // above every base
  __shared__ unsigned long long s_w[NW];
  __shared__ unsigned long long red[NW];

  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const unsigned lt = (1u << lane) - 1u;

  // ---- problem (A = the set with fewer words) ----
  uint64_t na = p.na_dev ? *p.na_dev : p.na;
  uint64_t nb = p.nb_dev ? *p.nb_dev : p.nb;
  const uint32_t *Ab = p.a, *As = p.sa, *Bb = p.b, *Bs = p.sb;
  if (na > nb) {
    const uint32_t *tb = Ab; Ab = Bb; Bb = tb;
    const uint32_t *ts = As; As = Bs; Bs = ts;
    const uint64_t tn = na; na = nb; nb = tn;
  }
  if (skip_by_rule(p.skip_rule, p.ratio_thr, na, nb)) return;
  const uint32_t G = gridDim.x, c = blockIdx.x;
  const uint64_t WT = uint64_t(G) * NW;
  const uint64_t gw = uint64_t(c) * NW + uint64_t(warp);

  // ---- this warp's runs: A words [ia0, ia1), B words [ib0, ib1) ----
  const uint64_t blocks = (na + 31) / 32;  // A's 32-word blocks (the last may be short)
  const uint64_t k0 = gw * blocks / WT, k1 = (gw + 1) * blocks / WT;
  const uint64_t ia0 = (k0 * 32 < na) ? k0 * 32 : na;
  const uint64_t ia1 = (gw + 1 == WT) ? na : ((k1 * 32 < na) ? k1 * 32 : na);
  uint64_t ib0 = 0, ib1 = 0;
  if (ia0 < ia1 && nb > 0) {
    uint32_t kv;
    const uint64_t e0 = guess_scale(ia0, na, nb);
    ib0 = warp_lower_bound_guess(Bb, nb, Ab + ia0, e0 < nb ? e0 : nb - 1, &kv);
    if (ia1 == na) {
      ib1 = nb;
    } else {
      const uint64_t e1 = guess_scale(ia1, na, nb);
      ib1 = warp_lower_bound_guess(Bb, nb, Ab + ia1, e1 < nb ? e1 : nb - 1, &kv);
    }
  }

  // ---- stream the two runs ----
  uint64_t wn = 0;  // materialise: this warp's words staged
  uint32_t cnt = 0; // count: this lane's popcount sum
  if (ia0 < ia1 && ib0 < ib1) {
    // blocks cur, next 1 .. KD (registers): lane l holds word q + l
    uint32_t ab[KD + 1], as[KD + 1], bb[KD + 1], bs[KD + 1];
    auto ld = [&](const uint32_t *base, const uint32_t *state, uint64_t q, uint64_t end,
                  uint32_t &b, uint32_t &s) {
      const uint64_t i = q + uint64_t(lane);
      b = i < end ? __ldg(base + i) : SENT;
      s = i < end ? __ldg(state + i) : 0u;
    };
    uint64_t ia = ia0, ib = ib0;
#pragma unroll
    for (int d = 0; d <= KD; ++d) {
      ld(Ab, As, ia + 32 * uint64_t(d), ia1, ab[d], as[d]);
      ld(Bb, Bs, ib + 32 * uint64_t(d), ib1, bb[d], bs[d]);
    }
    uint32_t *stg = MAT ? p.stage + ia0 : nullptr;
    uint32_t *stg_s = MAT ? p.stage_s + ia0 : nullptr;
    while (ia < ia1 && ib < ib1) {
      // block extents: first and last valid bases
      const uint32_t la = (ia1 - ia < 32) ? uint32_t(ia1 - ia) - 1 : 31u;
      const uint32_t lb = (ib1 - ib < 32) ? uint32_t(ib1 - ib) - 1 : 31u;
      const uint32_t amin = __shfl_sync(0xffffffffu, ab[0], 0);
      const uint32_t amax = __shfl_sync(0xffffffffu, ab[0], la);
      const uint32_t bmin = __shfl_sync(0xffffffffu, bb[0], 0);
      const uint32_t bmax = __shfl_sync(0xffffffffu, bb[0], lb);
      if (amax >= bmin && bmax >= amin) {  // the blocks' ranges overlap
        // lane: the first of B's 32 bases >= its A base (31 when none)
        const uint32_t x = ab[0];
        uint32_t lo = 0;
#pragma unroll
        for (uint32_t step = 16; step > 0; step >>= 1) {
          const uint32_t v = __shfl_sync(0xffffffffu, bb[0], lo + step - 1);
          lo += (v < x) ? step : 0u;
        }
        const uint32_t vb = __shfl_sync(0xffffffffu, bb[0], lo);
        const uint32_t vs = __shfl_sync(0xffffffffu, bs[0], lo);
        const uint32_t st = (vb == x && x != SENT) ? (as[0] & vs) : 0u;
        if (MAT) {
          const unsigned m = __ballot_sync(0xffffffffu, st != 0);
          if (st) {
            const uint64_t o = wn + uint32_t(__popc(m & lt));
            stg[o] = x;
            stg_s[o] = st;
          }
          wn += uint32_t(__popc(m));
        } else {
          cnt += uint32_t(__popc(st));
        }
      }
      // advance (i_a += W when a_max <= b_max; i_b += W when b_max <= a_max)
      if (amax <= bmax) {
        ia += 32;
#pragma unroll
        for (int d = 0; d < KD; ++d) {
          ab[d] = ab[d + 1];
          as[d] = as[d + 1];
        }
        ld(Ab, As, ia + 32 * uint64_t(KD), ia1, ab[KD], as[KD]);
      }
      if (bmax <= amax) {
        ib += 32;
#pragma unroll
        for (int d = 0; d < KD; ++d) {
          bb[d] = bb[d + 1];
          bs[d] = bs[d + 1];
        }
        ld(Bb, Bs, ib + 32 * uint64_t(KD), ib1, bb[KD], bs[KD]);
      }
    }
  }

  // ---- combine ----
  if (!MAT) {
    unsigned long long v = cnt;
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
    if (lane == 0) s_w[warp] = wn;
    __syncthreads();
    uint64_t before_w = 0, cta = 0;
#pragma unroll
    for (int q = 0; q < NW; ++q) {
      before_w += (q < warp) ? s_w[q] : 0;
      cta += s_w[q];
    }
    if (t == 0) p.coranks[c] = cta;
    if (!grid_barrier(&p.sync->done, G, p.err)) return;
    // the counts of CTAs 0..c-1 and of all CTAs, one round of loads
    constexpr int PL = 16;
    uint64_t bef = 0, all = 0;
    {
      uint64_t v[PL];
#pragma unroll
      for (int j = 0; j < PL; ++j) {
        const uint32_t q = uint32_t(t + j * NT);
        v[j] = q < G ? __ldcg(p.coranks + q) : 0;
      }
#pragma unroll
      for (int j = 0; j < PL; ++j) {
        const uint32_t q = uint32_t(t + j * NT);
        bef += q < c ? v[j] : 0;
        all += v[j];
      }
      for (uint32_t q = uint32_t(t + PL * NT); q < G; q += NT) {
        const uint64_t y = __ldcg(p.coranks + q);
        bef += q < c ? y : 0;
        all += y;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      bef += __shfl_xor_sync(0xffffffffu, bef, o);
      all += __shfl_xor_sync(0xffffffffu, all, o);
    }
    if (lane == 0) red[warp] = bef;
    __syncthreads();  // every warp has read s_w
    if (lane == 0) s_w[warp] = all;
    __syncthreads();
    uint64_t ex = 0, tot = 0;
#pragma unroll
    for (int q = 0; q < NW; ++q) {
      ex += red[q];
      tot += s_w[q];
    }
    if (tot > p.out_cap) {
      if (t == 0) record_error(p.err, DEV_ERR_CAPACITY);
    } else {
      const uint64_t dst0 = ex + before_w;
      for (uint64_t q = uint64_t(lane); q < wn; q += 32) {
        p.out[dst0 + q] = p.stage[ia0 + q];
        p.out_s[dst0 + q] = p.stage_s[ia0 + q];
      }
      if (c + 1 == G && t == 0) *p.out_len = tot;
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
