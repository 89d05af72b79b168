// gallop.cuh -- search-based intersection for skewed pairs.
//
// Semantics follow the reference's galloping (setops/src/intersect/
// galloping.rs:7-30) and galloping_bsr (galloping.rs:51-76): every element of
// the smaller set is looked up in the larger one; the output is the matching
// elements of the small set in their (ascending) order.
//
// GPU form: the exponential phase of galloping exists to find a bracket
// cheaply from the previous position.  On the GPU all small elements are
// searched at once, so the bracket comes from a shared-memory sample of the
// large set instead (NSAMP block maxima, loaded once per CTA); the search
// inside the bracket is then either
//   * GS == 1: one thread per element, a branchless binary search, ITEMS
//     independent searches interleaved per thread for memory-level
//     parallelism; or
//   * GS > 1: GS lanes per element, each round probing GS points of the
//     bracket at once and narrowing it (GS+1)-fold (warp ballot), so a
//     2^13-element bracket needs 3 dependent rounds with GS = 32.
// Output order is preserved by tiles (TILE consecutive small elements)
// claimed in order from an atomic ticket and combined with decoupled
// look-back.
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
  uint32_t *out;
  uint32_t *out_s;
  uint64_t out_cap;
  uint64_t *out_len;  // elements (count / array) or words (BSR materialise)
  uint64_t *status;   // look-back words, >= number of tiles
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
  static constexpr int kNG = NT / GS;
  static constexpr int kTile = kNG * ITEMS;
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
  constexpr int PT = (TILE + NT - 1) / NT;  // compaction positions / thread

  __shared__ uint32_t samp[NSAMP];
  __shared__ uint32_t sHit[TILE];
  __shared__ uint32_t sKey[MAT ? TILE : 1];
  __shared__ uint32_t sSt[(MAT && BSR) ? TILE : 1];
  __shared__ uint32_t warp_sums[NT / 32];
  __shared__ uint32_t s_tile;
  __shared__ unsigned long long s_excl;

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
  const uint64_t ntiles = (ns + TILE - 1) / TILE;
  if (skip_by_rule(p.skip_rule, p.ratio_thr, ns, nl)) return;

  // ---- sample of the large set: block maxima ----
  const uint64_t st = nl == 0 ? 1 : (nl + NSAMP - 1) / NSAMP;
  const uint32_t nblk = nl == 0 ? 0 : uint32_t((nl + st - 1) / st);
  for (uint32_t kb = t; kb < nblk; kb += NT) {
    uint64_t e = uint64_t(kb + 1) * st;
    if (e > nl) e = nl;
    samp[kb] = __ldg(L + e - 1);
  }
  __syncthreads();

  uint64_t cnt = 0;
  for (;;) {
    if (t == 0) s_tile = atomicAdd(&p.sync->ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    if (uint64_t(tile) >= ntiles) break;
    const uint64_t base = uint64_t(tile) * TILE;

    if (GS == 1) {
      // ITEMS interleaved branchless searches per thread
      uint32_t x[ITEMS];
      uint64_t lo[ITEMS], len[ITEMS];
      bool valid[ITEMS];
#pragma unroll
      for (int it = 0; it < ITEMS; ++it) {
        const uint64_t idx = base + uint64_t(t) * ITEMS + it;
        valid[it] = idx < ns;
        x[it] = valid[it] ? __ldg(S + idx) : 0u;
        const uint32_t kb = valid[it] ? smem_lower_bound(samp, nblk, x[it]) : nblk;
        if (kb >= nblk) {
          valid[it] = false;
          lo[it] = 0;
          len[it] = 0;
        } else {
          lo[it] = uint64_t(kb) * st;
          const uint64_t e = (lo[it] + st < nl) ? lo[it] + st : nl;
          len[it] = e - lo[it];
        }
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
      // GS lanes per element, (GS+1)-ary narrowing per round
      const int g = t / GS, gl = t & (GS - 1);
      const unsigned gmask =
          (GS == 32) ? 0xffffffffu
                     : (((1u << GS) - 1u) << (lane & ~(GS - 1)));
      const int gshift = lane & ~(GS - 1);
      for (int it = 0; it < ITEMS; ++it) {
        const uint64_t idx = base + uint64_t(g) * ITEMS + it;
        bool hit = false;
        uint32_t x = 0, stv = 0;
        if (idx < ns) {
          x = __ldg(S + idx);
          const uint32_t kb = smem_lower_bound(samp, nblk, x);
          if (kb < nblk) {
            uint64_t lo = uint64_t(kb) * st;
            uint64_t hi = (lo + st < nl) ? lo + st : nl;
            while (hi - lo > uint64_t(GS)) {
              const uint64_t span = hi - lo;
              const uint64_t xp = lo + (uint64_t(gl + 1) * span) / (GS + 1);
              const bool pr = __ldg(L + xp) < x;
              const uint64_t c =
                  __popc((__ballot_sync(gmask, pr) >> gshift) &
                         ((GS == 32) ? 0xffffffffu : ((1u << GS) - 1u)));
              const uint64_t nhi =
                  (c < uint64_t(GS)) ? lo + ((c + 1) * span) / (GS + 1) : hi;
              if (c > 0) lo = lo + (c * span) / (GS + 1) + 1;
              hi = nhi;
            }
            const uint64_t span = hi - lo;
            const bool pr = (uint64_t(gl) < span) && (__ldg(L + lo + gl) < x);
            const uint64_t c =
                __popc((__ballot_sync(gmask, pr) >> gshift) &
                       ((GS == 32) ? 0xffffffffu : ((1u << GS) - 1u)));
            const uint64_t lb = lo + c;
            hit = lb < nl && __ldg(L + lb) == x;
            if (BSR && hit) {
              stv = __ldg(SS + idx) & __ldg(SL + lb);
              hit = stv != 0;
            }
          }
        }
        if (gl == 0) {
          const int pos = g * ITEMS + it;
          if (MAT) {
            sHit[pos] = hit;
            sKey[pos] = x;
            if (BSR) sSt[pos] = stv;
          } else {
            cnt += BSR ? (hit ? __popc(stv) : 0) : (hit ? 1 : 0);
          }
        }
      }
    }

    if (MAT) {
      __syncthreads();
      uint32_t mine = 0;
#pragma unroll
      for (int q = 0; q < PT; ++q) {
        const int pos = t * PT + q;
        if (pos < TILE) mine += sHit[pos];
      }
      uint32_t tot;
      const uint32_t ex = block_exclusive_scan<NT>(mine, warp_sums, &tot);
      if (t == 0) s_excl = lookback_exclusive(p.status, tile, tot, p.epoch, p.err);
      __syncthreads();
      const uint64_t tex = s_excl;
      if (tex == UINT64_MAX) return;  // error recorded; host resets state
      if (tex + tot > p.out_cap) {
        if (t == 0) record_error(p.err, DEV_ERR_CAPACITY);
        return;
      }
      uint64_t o = tex + ex;
#pragma unroll
      for (int q = 0; q < PT; ++q) {
        const int pos = t * PT + q;
        if (pos < TILE && sHit[pos]) {
          p.out[o] = sKey[pos];
          if (BSR) p.out_s[o] = sSt[pos];
          ++o;
        }
      }
      if (tile == ntiles - 1 && t == 0) *p.out_len = tex + tot;
    }
    __syncthreads();  // s_tile / smem tile buffers are reused
  }

  // ---- combine counts, reset coordination words ----
  if (!MAT) {
    uint64_t v = cnt;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __shared__ unsigned long long red[NT / 32];
    if (lane == 0) red[t >> 5] = v;
    __syncthreads();
    if (t == 0) {
      unsigned long long s = 0;
      for (int w = 0; w < NT / 32; ++w) s += red[w];
      if (s) atomicAdd(&p.sync->acc, s);
    }
  }
  if (t == 0) {
    __threadfence();
    const uint32_t prev = atomicAdd(&p.sync->done, 1u);
    if (prev == gridDim.x - 1) {
      if (!MAT) *p.out_len = atomicExch(&p.sync->acc, 0ull);
      else if (ntiles == 0) *p.out_len = 0;
      p.sync->ticket = 0;
      p.sync->done = 0;
      __threadfence();
    }
  }
}

}  // namespace setops
