// gallop.cuh -- search-based intersection for skewed pairs.
//
// Semantics follow the reference's galloping (setops/src/intersect/
// galloping.rs:7-30) and galloping_bsr (galloping.rs:51-76): every element of
// the smaller set is looked up in the larger one; the output is the matching
// elements of the small set in their (ascending) order.
//
// GPU form.  Galloping's exponential phase exists to find a bracket cheaply
// from the previous position; on the GPU all small elements are searched at
// once, so brackets come from cooperative searches instead:
//   * each CTA owns a contiguous run of small elements (one static range per
//     CTA, like the merge kernel's diagonal ranges);
//   * NSAMP > 0: the CTA bounds the large-set bracket of its whole run (two
//     warps, one round of probes around a guess each; a few hundred elements
//     of slack), then loads a shared-memory sample of NSAMP bracket maxima, so
//     each element starts from a narrow block;
//     NSAMP == 0: every element searches the whole large set (no per-CTA
//     preparation; best when a CTA has few elements);
//   * the search inside the block is either GS == 1: one thread per element,
//     branchless binary search, ITEMS interleaved per thread for memory-level
//     parallelism; or GS > 1: GS lanes per element probing GS points per
//     round ((GS+1)-ary narrowing via warp ballot).
// Matches are staged per CTA (block scan per pass, order preserved) in a
// scratch region at the CTA's first element (a CTA cannot emit more matches
// than elements it owns); one warp-parallel look-back per CTA gives its
// output offset.
#pragma once

#include "common.cuh"

namespace setops {

struct GallopArgs {
  const uint32_t *a;   // keys (BSR: bases)
  const uint32_t *b;
  const uint32_t *sa;  // BSR states
  const uint32_t *sb;
  uint64_t na, nb;
  const uint64_t *na_dev;
  const uint64_t *nb_dev;
  uint32_t *stage;    // scratch, >= min(na, nb) words (materialise)
  uint32_t *stage_s;  // scratch states (BSR materialise)
  uint32_t *out;
  uint32_t *out_s;
  uint64_t out_cap;
  uint64_t *out_len;  // elements (count / array) or words (BSR materialise)
  uint64_t *status;   // look-back words, >= gridDim.x entries
  LaunchSync *sync;
  int *err;
  uint32_t epoch;
  // Device-side algorithm choice (k-set steps whose input length is only
  // known on the device): 0 = always run; 1 = run only when
  // max(na,nb)/min(na,nb) >= ratio_thr (search wins); 2 = only when below.
  int skip_rule;
  uint32_t ratio_thr;
};

template <int NT, int GS, int ITEMS, int NSAMP>
struct GallopCfg {
  static_assert(GS == 1 || GS == 2 || GS == 4 || GS == 8 || GS == 16 ||
                    GS == 32,
                "group size must divide a warp");
  static_assert(GS == 1 || ITEMS == 1, "groups search one element at a time");
  static_assert(NSAMP == 0 || NT >= 64, "two warps bound the run's bracket");
  static constexpr int kNG = NT / GS;
  static constexpr int kTile = kNG * ITEMS;  // elements per pass of a CTA
};

// First index k in samp[0..n) with samp[k] >= x (n if none).
__device__ __forceinline__ uint32_t smem_lower_bound(const uint32_t *samp,
                                                     uint32_t n, uint32_t x) {
  uint32_t lo = 0, len = n;
  while (len > 0) {
    const uint32_t half = len >> 1;
    if (samp[lo + half] < x) {
      lo += half + 1;
      len -= half + 1;
    } else {
      len = half;
    }
  }
  return lo;
}

template <int NT, int GS, int ITEMS, int NSAMP, bool BSR, bool MAT>
__global__ void __launch_bounds__(NT) gallop_kernel(const GallopArgs p) {
  using Cfg = GallopCfg<NT, GS, ITEMS, NSAMP>;
  constexpr int TILE = Cfg::kTile;
  constexpr int SAMP = NSAMP > 0 ? NSAMP : 1;

  __shared__ uint32_t samp[SAMP];
  __shared__ uint32_t sHit[TILE];
  __shared__ uint32_t sKey[MAT ? TILE : 1];
  __shared__ uint32_t sSt[(MAT && BSR) ? TILE : 1];
  __shared__ uint32_t warp_sums[NT / 32];
  __shared__ uint32_t s_vid;
  __shared__ uint32_t s_last;
  __shared__ unsigned long long red[NT / 32];

  const int t = threadIdx.x;
  const int lane = t & 31;

  uint64_t ns = p.na_dev ? *p.na_dev : p.na;
  uint64_t nl = p.nb_dev ? *p.nb_dev : p.nb;
  const uint32_t *S = p.a, *L = p.b, *SS = p.sa, *SL = p.sb;
  if (ns > nl) {
    const uint32_t *tp = S; S = L; L = tp;
    tp = SS; SS = SL; SL = tp;
    uint64_t tn = ns; ns = nl; nl = tn;
  }
  if (skip_by_rule(p.skip_rule, p.ratio_thr, ns, nl)) return;

  if (t == 0) s_vid = atomicAdd(&p.sync->ticket, 1u);
  __syncthreads();
  const uint32_t vid = s_vid;
  const uint32_t G = gridDim.x;
  const uint64_t per = (ns + G - 1) / G;
  const uint64_t s0 = (uint64_t(vid) * per < ns) ? uint64_t(vid) * per : ns;
  const uint64_t s1 = (s0 + per < ns) ? s0 + per : ns;

  // ---- bracket of this CTA's run in L, and its sample ----
  uint64_t blo = 0, bhi = nl;  // candidates for S[s0..s1) lie in L[blo, bhi)
  uint64_t st = 1;
  uint32_t nblk = 0;
  if (NSAMP > 0 && s1 > s0 && nl > 0) {
    // bounds, not exact indexes: warp 0 brackets the first element's
    // lower_bound, warp 1 the last one's, at the same time (one round of
    // probes each around a guess at the same fraction of L as of S)
    __shared__ unsigned long long s_br[2];
    const int warp = t >> 5;
    if (warp < 2) {
      const uint64_t i = warp == 0 ? s0 : s1 - 1;
      const uint64_t est = guess_scale(i, ns, nl);
      uint64_t lo, hi;
      warp_bracket_guess(L, nl, S + i, est, &lo, &hi);
      if (lane == 0) s_br[warp] = warp == 0 ? lo : hi;
    }
    __syncthreads();
    blo = s_br[0];
    const uint64_t lbl = s_br[1];   // at or above the last element's lower_bound
    bhi = lbl < nl ? lbl + 1 : nl;  // which is a candidate
    const uint64_t len = bhi > blo ? bhi - blo : 0;
    st = len == 0 ? 1 : (len + SAMP - 1) / SAMP;
    nblk = len == 0 ? 0 : uint32_t((len + st - 1) / st);
    for (uint32_t kb = t; kb < nblk; kb += NT) {
      uint64_t e = blo + uint64_t(kb + 1) * st;
      if (e > bhi) e = bhi;
      samp[kb] = __ldg(L + e - 1);
    }
    __syncthreads();
  }

  // Bracket [lo, lo+len) inside which lower_bound(L, x) lies, or len == 0
  // with lo == nl when x exceeds the candidates.
  auto bracket = [&](uint32_t x, uint64_t &lo, uint64_t &len) {
    if (NSAMP > 0) {
      const uint32_t kb = smem_lower_bound(samp, nblk, x);
      if (kb >= nblk) {
        lo = nl;
        len = 0;
        return;
      }
      lo = blo + uint64_t(kb) * st;
      const uint64_t e = (lo + st < bhi) ? lo + st : bhi;
      len = e - lo;
    } else {
      lo = 0;
      len = nl;
    }
  };

  uint64_t cnt = 0;      // count mode (BSR: elements)
  uint64_t cta_cnt = 0;  // materialise: matches staged so far
  for (uint64_t base = s0; base < s1; base += TILE) {
    if (GS == 1) {
      uint32_t x[ITEMS];
      uint64_t lo[ITEMS], len[ITEMS];
      bool valid[ITEMS];
#pragma unroll
      for (int it = 0; it < ITEMS; ++it) {
        const uint64_t idx = base + uint64_t(t) * ITEMS + it;
        valid[it] = idx < s1;
        x[it] = valid[it] ? __ldg(S + idx) : 0u;
        if (valid[it]) bracket(x[it], lo[it], len[it]);
        else { lo[it] = nl; len[it] = 0; }
      }
      bool more = true;
      while (more) {
        more = false;
#pragma unroll
        for (int it = 0; it < ITEMS; ++it) {
          if (len[it] > 0) {
            const uint64_t half = len[it] >> 1;
            const bool lt = __ldg(L + lo[it] + half) < x[it];
            lo[it] = lt ? lo[it] + half + 1 : lo[it];
            len[it] = lt ? len[it] - half - 1 : half;
            more |= len[it] > 0;
          }
        }
      }
#pragma unroll
      for (int it = 0; it < ITEMS; ++it) {
        const uint64_t idx = base + uint64_t(t) * ITEMS + it;
        bool hit = valid[it] && lo[it] < nl && __ldg(L + lo[it]) == x[it];
        uint32_t stv = 0;
        if (BSR && hit) {
          stv = __ldg(SS + idx) & __ldg(SL + lo[it]);
          hit = stv != 0;
        }
        const int pos = t * ITEMS + it;
        if (MAT) {
          sHit[pos] = hit;
          sKey[pos] = x[it];
          if (BSR) sSt[pos] = stv;
        } else {
          cnt += BSR ? (hit ? __popc(stv) : 0) : (hit ? 1 : 0);
        }
      }
    } else {
      const int g = t / GS, gl = t & (GS - 1);
      const unsigned gbits = (GS == 32) ? 0xffffffffu : ((1u << GS) - 1u);
      const int gshift = lane & ~(GS - 1);
      const unsigned gmask = gbits << gshift;
      const uint64_t idx = base + uint64_t(g);
      bool hit = false;
      uint32_t x = 0, stv = 0;
      if (idx < s1) {
        x = __ldg(S + idx);
        uint64_t lo, len;
        bracket(x, lo, len);
        if (len > 0) {
          uint64_t hi = lo + len;
          while (hi - lo > uint64_t(GS)) {
            const uint64_t span = hi - lo;
            const uint64_t xp = lo + (uint64_t(gl + 1) * span) / (GS + 1);
            const bool pr = __ldg(L + xp) < x;
            const uint64_t c = __popc((__ballot_sync(gmask, pr) >> gshift) & gbits);
            const uint64_t nhi = (c < uint64_t(GS)) ? lo + ((c + 1) * span) / (GS + 1) : hi;
            if (c > 0) lo = lo + (c * span) / (GS + 1) + 1;
            hi = nhi;
          }
          const uint64_t span = hi - lo;
          const bool pr = (uint64_t(gl) < span) && (__ldg(L + lo + gl) < x);
          const uint64_t lb = lo + __popc((__ballot_sync(gmask, pr) >> gshift) & gbits);
          hit = lb < nl && __ldg(L + lb) == x;
          if (BSR && hit) {
            stv = __ldg(SS + idx) & __ldg(SL + lb);
            hit = stv != 0;
          }
        }
      }
      if (gl == 0) {
        if (MAT) {
          sHit[g] = hit;
          sKey[g] = x;
          if (BSR) sSt[g] = stv;
        } else {
          cnt += BSR ? (hit ? __popc(stv) : 0) : (hit ? 1 : 0);
        }
      }
    }

    if (MAT) {
      __syncthreads();
      constexpr int PT = (TILE + NT - 1) / NT;  // positions per thread
      uint32_t mine = 0;
#pragma unroll
      for (int q = 0; q < PT; ++q) {
        const int pos = t * PT + q;
        if (pos < TILE) mine += sHit[pos];
      }
      uint32_t tot;
      const uint32_t ex = block_exclusive_scan<NT>(mine, warp_sums, &tot);
      uint64_t o = s0 + cta_cnt + ex;
#pragma unroll
      for (int q = 0; q < PT; ++q) {
        const int pos = t * PT + q;
        if (pos < TILE && sHit[pos]) {
          p.stage[o] = sKey[pos];
          if (BSR) p.stage_s[o] = sSt[pos];
          ++o;
        }
      }
      cta_cnt += tot;
      __syncthreads();  // sHit / sKey reused by the next pass
    }
  }

  // ---- combine ----
  if (!MAT) {
    uint64_t v = cnt;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[t >> 5] = v;
    __syncthreads();
    if (t == 0) {
      unsigned long long s = 0;
      for (int w = 0; w < NT / 32; ++w) s += red[w];
      if (s) atomicAdd(&p.sync->acc, s);
      __threadfence();
      if (atomicAdd(&p.sync->done, 1u) == G - 1) {
        *p.out_len = atomicExch(&p.sync->acc, 0ull);
        p.sync->ticket = 0;
        p.sync->done = 0;
        __threadfence();
      }
    }
    return;
  }
  // Placement.  Each CTA publishes its match count (p.status[vid]); the last
  // CTA to get here turns the counts into offsets (an exclusive scan, in
  // place, the total in p.status[G]) and raises the flag sync->acc = 1 that
  // the others wait for (the launch is cooperative: all CTAs are resident).
  // Then every CTA copies its staged run.  Matches are few on the pairs that
  // take this kernel, and CTAs finish in any order: a chained look-back would
  // wait on the slowest predecessor once per CTA.
  if (t == 0) {
    p.status[vid] = cta_cnt;
    __threadfence();
    s_last = atomicAdd(&p.sync->done, 1u) == G - 1 ? 1u : 0u;
  }
  __syncthreads();
  if (s_last) {
    __threadfence();
    const uint32_t per_t = (G + NT - 1) / NT;  // thread t scans [t*per_t, t*per_t + per_t)
    const uint32_t i0 = uint32_t(t) * per_t, i1 = (i0 + per_t < G) ? i0 + per_t : G;
    uint32_t sum = 0;
    for (uint32_t i = i0; i < i1; ++i) sum += uint32_t(p.status[i]);
    uint32_t tot;
    uint64_t run_off = block_exclusive_scan<NT>(sum, warp_sums, &tot);
    for (uint32_t i = i0; i < i1; ++i) {
      const uint64_t c = p.status[i];
      p.status[i] = run_off;
      run_off += c;
    }
    if (t == 0) {
      p.status[G] = tot;
      if (tot > p.out_cap) record_error(p.err, DEV_ERR_CAPACITY);
      else *p.out_len = tot;
      __threadfence();
      atomicExch(&p.sync->acc, 1ull);  // the flag
    }
    __syncthreads();
  } else {
    if (t == 0) {
      uint32_t ok = 1;
      const uint64_t t0 = global_ns();
      while (ld_acquire_u64(reinterpret_cast<const uint64_t *>(&p.sync->acc)) == 0) {
        __nanosleep(100);
        if (global_ns() - t0 > wait_limit_ns()) {
          record_error(p.err, DEV_ERR_TIMEOUT_LOOKBACK);
          ok = 0;
          break;
        }
      }
      s_last = ok ? 0u : 2u;
    }
    __syncthreads();
    if (s_last == 2u) return;  // timeout recorded
  }
  {
    const uint64_t ex = p.status[vid], tot = p.status[G];
    if (tot <= p.out_cap) {
      for (uint64_t q = t; q < cta_cnt; q += NT) {
        p.out[ex + q] = p.stage[s0 + q];
        if (BSR) p.out_s[ex + q] = p.stage_s[s0 + q];
      }
    }
  }
  // the last CTA out resets the coordination words for the next launch
  __syncthreads();
  if (t == 0) {
    __threadfence();
    if (atomicAdd(&p.sync->acc, 1ull) == G) {
      p.sync->ticket = 0;
      p.sync->done = 0;
      p.sync->acc = 0;
      __threadfence();
    }
  }
}

}  // namespace setops
