// merge.cuh -- merge-path intersection of two sorted, duplicate-free u32
// arrays (and of two BSR sets, merging on bases).
//
// Semantics follow the reference's naive_merge (setops/src/intersect/
// merge.rs:7-33) and branchless_merge_bsr (merge.rs:62-87): the output is the
// ascending intersection, with the Counter visitor's count
// (setops/src/visitor.rs:24-49, BSR: sum of popcount(state), visitor.rs:399).
//
// Layout of the work
// ------------------
// Let A be the smaller input.  Merge the two arrays conceptually, taking A
// first on ties; a match is then an A element whose successor in the merge is
// an equal B element.  The merged sequence (length na+nb) is cut into one
// contiguous diagonal range per CTA.  A CTA
//   1. finds the merge-path co-rank of its first diagonal with a cooperative
//      (NT+1)-ary search over global memory (3 rounds for 2^24 elements);
//   2. streams its range in tiles of NV = NT*VT merged elements.  Both inputs
//      are staged in shared-memory rings (R words each) by 1-D bulk copies
//      (cp.async.bulk, completing on one of two mbarriers), issued two tiles
//      ahead of use;
//   3. per tile, every thread binary-searches its own sub-diagonal in the
//      rings and walks VT merge steps, counting (or staging) matches;
//   4. count mode: one atomic add per CTA, the last CTA to finish writes the
//      total.  Materialise mode: matches go to a scratch stage at the CTA's
//      A co-rank (an exclusive region: a CTA can never emit more matches than
//      A elements it consumes), then decoupled look-back over CTAs gives each
//      CTA its output offset and it copies its run to the output.
//
// A match whose A element is the last one a thread/tile/CTA consumes looks
// one element ahead into B; the rings always hold B up to one element past
// the tile window, so no match is lost or counted twice at any boundary.
#pragma once

#include "common.cuh"

namespace setops {

struct MergeArgs {
  const uint32_t *a;   // keys of set A (or BSR bases)
  const uint32_t *b;
  const uint32_t *sa;  // BSR states (BSR kernels only)
  const uint32_t *sb;
  uint64_t na, nb;
  const uint64_t *na_dev;  // optional device-side lengths (override na/nb)
  const uint64_t *nb_dev;
  uint32_t *stage;    // scratch, >= min(na, nb) words (materialise)
  uint32_t *stage_s;  // scratch states (BSR materialise)
  uint32_t *out;      // output keys / bases
  uint32_t *out_s;    // output states (BSR)
  uint64_t out_cap;
  uint64_t *out_len;  // device: element count (count / array), or word count
                      // (BSR materialise)
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

template <int NT, int VT, int RLOG, bool BSR, bool MAT>
struct MergeCfg {
  static constexpr int kNT = NT;
  static constexpr int kVT = VT;
  static constexpr int kNV = NT * VT;
  static constexpr uint32_t kR = 1u << RLOG;
  // Prefetch frontier is two tiles ahead: ring must hold 3*NV+1 words plus
  // 16-byte rounding at both ends.
  static_assert(kR >= 3 * kNV + 16, "ring too small for two-tile lookahead");
  static constexpr size_t kRingWords = (BSR ? 4 : 2) * size_t(kR);
  static constexpr size_t kOutWords = MAT ? (BSR ? 2 : 1) * size_t(kNV) : 0;
  static constexpr size_t kSmemBytes = (kRingWords + kOutWords) * 4;
};

// Producer-side state of one staged array.
struct RingFeed {
  const uint32_t *al;  // 16-byte aligned base (element index -off)
  uint64_t n;          // element count
  uint32_t off;        // misalignment of element 0, in words (0..3)
  uint64_t front;      // aligned coordinate loaded so far (exclusive)
};

__device__ __forceinline__ RingFeed make_feed(const uint32_t *p, uint64_t n,
                                              uint64_t first_elem) {
  RingFeed f;
  const uintptr_t addr = reinterpret_cast<uintptr_t>(p);
  f.off = uint32_t((addr >> 2) & 3);
  f.al = reinterpret_cast<const uint32_t *>(addr & ~uintptr_t(15));
  f.n = n;
  f.front = (first_elem + f.off) & ~uint64_t(3);
  return f;
}

// Bytes the bulk part of a feed step will move (for expect_tx), and the
// aligned range.  Partial 16-byte chunks (only the chunk holding element 0
// when the array is misaligned and the chunk holding the last element) are
// loaded with plain loads by the producer thread instead.
struct FeedPlan {
  uint64_t lo, hi;      // aligned coords [lo, hi) to load this step
  uint64_t blo, bhi;    // bulk sub-range (multiples of 4)
};

__device__ __forceinline__ FeedPlan plan_feed(const RingFeed &f,
                                              uint64_t target_elem) {
  FeedPlan pl;
  const uint64_t end_al = f.n + f.off;
  uint64_t t = (target_elem + f.off + 3) & ~uint64_t(3);
  if (t > end_al) t = end_al;
  pl.lo = f.front;
  pl.hi = t > f.front ? t : f.front;
  pl.blo = (pl.lo + 3) & ~uint64_t(3);
  if (pl.blo < f.off) pl.blo = 4;  // chunk 0 is partial when off > 0
  pl.bhi = pl.hi & ~uint64_t(3);
  if (pl.bhi < pl.blo) pl.bhi = pl.blo;
  return pl;
}

template <uint32_t R>
__device__ __forceinline__ void run_feed(RingFeed &f, const FeedPlan &pl,
                                         uint32_t *ring, uint64_t *bar,
                                         uint64_t pol) {
  constexpr uint32_t RM = R - 1;
  if (pl.hi <= pl.lo) return;
  // Plain loads for the (at most 3 + 3) aligned coords outside the bulk
  // range: the head chunk when element 0 is misaligned, the tail chunk when
  // the array end is.  Coordinates below `off` precede element 0.
  const uint64_t hcut = pl.blo < pl.hi ? pl.blo : pl.hi;
  for (uint64_t c = pl.lo; c < hcut; ++c)
    if (c >= f.off) ring[c & RM] = __ldg(f.al + c);
  const uint64_t tstart = pl.bhi > hcut ? pl.bhi : hcut;
  for (uint64_t c = tstart; c < pl.hi; ++c)
    if (c >= f.off) ring[c & RM] = __ldg(f.al + c);
  if (pl.bhi > pl.blo) {
    const uint32_t words = uint32_t(pl.bhi - pl.blo);
    const uint32_t s0 = uint32_t(pl.blo) & RM;
    const uint32_t first = (s0 + words <= R) ? words : (R - s0);
    bulk_g2s(ring + s0, f.al + pl.blo, first * 4, bar, pol);
    if (first < words)
      bulk_g2s(ring, f.al + pl.blo + first, (words - first) * 4, bar, pol);
  }
  f.front = pl.hi;
}

__device__ __forceinline__ uint32_t plan_bytes(const FeedPlan &pl) {
  return uint32_t(pl.bhi - pl.blo) * 4;
}

template <int NT, int VT, int RLOG, bool BSR, bool MAT>
__global__ void __launch_bounds__(NT)
    merge_kernel(const MergeArgs p) {
  using Cfg = MergeCfg<NT, VT, RLOG, BSR, MAT>;
  constexpr int NV = Cfg::kNV;
  constexpr uint32_t R = Cfg::kR;
  constexpr uint32_t RM = R - 1;

  extern __shared__ __align__(128) uint32_t smem[];
  uint32_t *ringA = smem;
  uint32_t *ringB = smem + R;
  uint32_t *ringSA = BSR ? smem + 2 * R : nullptr;
  uint32_t *ringSB = BSR ? smem + 3 * R : nullptr;
  uint32_t *sOut = smem + Cfg::kRingWords;
  uint32_t *sOutS = sOut + NV;

  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t sCo[NT + 1];
  __shared__ uint32_t warp_sums[NT / 32];
  __shared__ uint32_t s_vid;
  __shared__ int s_abort;

  const int t = threadIdx.x;

  // ---- problem (A = smaller set) ----
  uint64_t na = p.na_dev ? *p.na_dev : p.na;
  uint64_t nb = p.nb_dev ? *p.nb_dev : p.nb;
  const uint32_t *A = p.a, *B = p.b, *SA = p.sa, *SB = p.sb;
  if (na > nb) {
    const uint32_t *tp = A; A = B; B = tp;
    tp = SA; SA = SB; SB = tp;
    uint64_t tn = na; na = nb; nb = tn;
  }
  const uint64_t total = na + nb;
  if (skip_by_rule(p.skip_rule, p.ratio_thr, na, nb)) return;

  if (t == 0) {
    s_vid = atomicAdd(&p.sync->ticket, 1u);
    s_abort = 0;
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  const uint32_t vid = s_vid;
  const uint32_t G = gridDim.x;
  uint64_t D = (total + G - 1) / G;
  D = ((D + NV - 1) / NV) * NV;  // whole tiles per CTA where possible
  const uint64_t d0 = (uint64_t(vid) * D < total) ? uint64_t(vid) * D : total;
  const uint64_t d1 = (d0 + D < total) ? d0 + D : total;

  // ---- 1. co-rank of diagonal d0: smallest i with A[i] > B[d0-1-i] ----
  uint64_t lo = d0 > nb ? d0 - nb : 0;
  uint64_t hi = d0 < na ? d0 : na;
  while (hi > lo) {
    const uint64_t span = hi - lo;
    if (span <= uint64_t(NT)) {
      bool pr = false;
      if (uint64_t(t) < span) {
        const uint64_t x = lo + t;
        pr = __ldg(A + x) <= __ldg(B + (d0 - 1 - x));
      }
      lo += uint64_t(__syncthreads_count(pr));
      break;
    }
    const uint64_t x = lo + (uint64_t(t + 1) * span) / (NT + 1);
    const bool pr = __ldg(A + x) <= __ldg(B + (d0 - 1 - x));
    const uint64_t c = uint64_t(__syncthreads_count(pr));
    const uint64_t nhi = (c < NT) ? lo + ((c + 1) * span) / (NT + 1) : hi;
    if (c > 0) lo = lo + (c * span) / (NT + 1) + 1;
    hi = nhi;
  }
  uint64_t ia = lo, ib = d0 - lo;
  const uint64_t stage_base = ia;  // exclusive stage region of this CTA

  // ---- 2. stream tiles ----
  const uint64_t pol = l2_evict_first_policy();
  RingFeed fA = make_feed(A, na, ia), fB = make_feed(B, nb, ib);
  RingFeed fSA, fSB;
  if (BSR) {
    fSA = make_feed(SA, na, ia);
    fSB = make_feed(SB, nb, ib);
  }
  // state-ring slot = key-ring slot + (state misalignment - key misalignment)
  const uint32_t dSA = BSR ? (fSA.off - fA.off) : 0;
  const uint32_t dSB = BSR ? (fSB.off - fB.off) : 0;

  // Producer: stage everything this CTA needs up to element targets.
  auto issue = [&](int bar_idx, uint64_t ia_n, uint64_t ib_n, uint64_t dn) {
    const uint64_t rem = d1 - dn;  // merged elements left after ia_n/ib_n
    uint64_t ta = ia_n + (rem < 2 * uint64_t(NV) ? rem : 2 * uint64_t(NV)) + 1;
    uint64_t tb = ib_n + (rem < 2 * uint64_t(NV) ? rem : 2 * uint64_t(NV)) + 1;
    if (ta > na) ta = na;
    if (tb > nb) tb = nb;
    FeedPlan pa = plan_feed(fA, ta), pb = plan_feed(fB, tb);
    FeedPlan psa, psb;
    uint32_t bytes = plan_bytes(pa) + plan_bytes(pb);
    if (BSR) {
      psa = plan_feed(fSA, ta);
      psb = plan_feed(fSB, tb);
      bytes += plan_bytes(psa) + plan_bytes(psb);
    }
    mbar_arrive_expect_tx(&mbar[bar_idx], bytes);
    run_feed<R>(fA, pa, ringA, &mbar[bar_idx], pol);
    run_feed<R>(fB, pb, ringB, &mbar[bar_idx], pol);
    if (BSR) {
      run_feed<R>(fSA, psa, ringSA, &mbar[bar_idx], pol);
      run_feed<R>(fSB, psb, ringSB, &mbar[bar_idx], pol);
    }
  };

  uint64_t diag = ia + ib;
  const bool has_work = diag < d1;
  if (has_work && t == 0) issue(0, ia, ib, diag);  // batch -1 -> barrier 0
  __syncthreads();

  uint64_t cnt = 0;      // count mode: this thread's matches
  uint64_t cta_cnt = 0;  // materialise: matches staged by this CTA
  int k = 0;             // tile index
  bool aborted = false;
  while (diag < d1) {
    // wait for the batch that completes this tile's window
    {
      int wb = -2;  // which batch: -1 for tile 0, k-2 for k >= 2
      if (k == 0) wb = -1;
      else if (k >= 2) wb = k - 2;
      if (wb >= -1) {
        const int bi = (wb + 1) & 1;
        const uint32_t par = uint32_t((wb + 1) >> 1) & 1u;
        const bool ok = mbar_wait_bounded(&mbar[bi], par, p.err);
        if (__syncthreads_or(!ok)) {
          aborted = true;
          break;
        }
      }
    }
    const uint64_t rem = d1 - diag;
    const uint32_t nvt = rem < uint64_t(NV) ? uint32_t(rem) : uint32_t(NV);
    const uint32_t la = (na - ia) < nvt ? uint32_t(na - ia) : nvt;
    const uint32_t lb = (nb - ib) < nvt ? uint32_t(nb - ib) : nvt;
    const uint32_t abase = uint32_t(ia + fA.off);
    const uint32_t bbase = uint32_t(ib + fB.off);

    // ---- split: co-rank of each thread's sub-diagonal within the window ----
    {
      // thread 0's own diagonal is 0; it computes the tile end instead
      const uint32_t d = (t == 0) ? nvt : min(uint32_t(t) * VT, nvt);
      uint32_t l = d > lb ? d - lb : 0, h = d < la ? d : la;
      while (l < h) {
        const uint32_t m = (l + h) >> 1;
        const uint32_t av = ringA[(abase + m) & RM];
        const uint32_t bv = ringB[(bbase + d - 1 - m) & RM];
        if (av <= bv) l = m + 1; else h = m;
      }
      if (t == 0) {
        sCo[NT] = l;
        sCo[0] = 0;
      } else {
        sCo[t] = l;
      }
    }
    __syncthreads();
    const uint32_t ca = sCo[NT], cb = nvt - ca;
    // ---- producer: next batch (barrier (k+1)&1) ----
    if (t == 0) issue((k + 1) & 1, ia + ca, ib + cb, diag + nvt);

    // ---- serial merge of this thread's VT steps ----
    const uint32_t dt = min(uint32_t(t) * VT, nvt);
    const uint32_t dn = min(uint32_t(t + 1) * VT, nvt);
    const uint32_t i0 = sCo[t];
    const uint32_t j0 = dt - i0;
    uint32_t as = (abase + i0) & RM, bs = (bbase + j0) & RM;
    uint32_t av = ringA[as], bv = ringB[bs];
    uint32_t c = 0;
    const bool fast = (nvt == uint32_t(NV)) && (ia + NV + 1 <= na) &&
                      (ib + NV + 1 <= nb);
    auto on_match = [&](uint32_t key) {
      if (BSR) {
        const uint32_t st = ringSA[(as + dSA) & RM] & ringSB[(bs + dSB) & RM];
        if (st != 0) {
          if (MAT) {
            sOut[t * VT + c] = key;
            sOutS[t * VT + c] = st;
            ++c;
          } else {
            cnt += __popc(st);
          }
        }
      } else {
        if (MAT) sOut[t * VT + c] = key;
        ++c;
      }
    };
    if (fast) {
#pragma unroll
      for (int s = 0; s < VT; ++s) {
        const bool takeA = av <= bv;
        if (av == bv) on_match(av);
        if (takeA) {
          as = (as + 1) & RM;
          av = ringA[as];
        } else {
          bs = (bs + 1) & RM;
          bv = ringB[bs];
        }
      }
    } else {
      uint64_t gi = ia + i0, gj = ib + j0;
      const uint32_t steps = dn - dt;
#pragma unroll
      for (int s = 0; s < VT; ++s) {
        if (uint32_t(s) < steps) {
          const bool aok = gi < na, bok = gj < nb;
          const bool takeA = aok && (!bok || av <= bv);
          if (takeA && bok && av == bv) on_match(av);
          if (takeA) {
            ++gi;
            as = (as + 1) & RM;
            av = ringA[as];
          } else {
            ++gj;
            bs = (bs + 1) & RM;
            bv = ringB[bs];
          }
        }
      }
    }

    if (MAT) {
      uint32_t tot;
      const uint32_t ex = block_exclusive_scan<NT>(c, warp_sums, &tot);
      uint32_t *dst = p.stage + stage_base + cta_cnt + ex;
      for (uint32_t q = 0; q < c; ++q) dst[q] = sOut[t * VT + q];
      if (BSR) {
        uint32_t *dsts = p.stage_s + stage_base + cta_cnt + ex;
        for (uint32_t q = 0; q < c; ++q) dsts[q] = sOutS[t * VT + q];
      }
      cta_cnt += tot;
    } else {
      if (!BSR) cnt += c;
      __syncthreads();  // sCo is rewritten by the next split
    }
    ia += ca;
    ib += cb;
    diag += nvt;
    ++k;
  }

  // ---- drain: no bulk copy may still target this CTA's shared memory ----
  if (has_work && t == 0) {
    // Batches issued: -1 .. k-1.  Tile 0 waited for -1, tile j >= 2 for j-2,
    // so k-2 .. k-1 (or -1 alone, if tile 0's wait timed out) may still be
    // in flight.  Each barrier has at most one phase outstanding.
    const int first = (k == 0) ? -1 : (k >= 2 ? k - 2 : 0);
    const int last = (k == 0) ? -1 : k - 1;
    for (int wb = first; wb <= last; ++wb) {
      mbar_wait_bounded(&mbar[(wb + 1) & 1], uint32_t((wb + 1) >> 1) & 1u,
                        p.err);
    }
  }
  __syncthreads();
  if (aborted) return;

  // ---- 3. combine ----
  if (!MAT) {
    // block reduction of cnt
    uint64_t v = cnt;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __shared__ unsigned long long red[NT / 32];
    if ((t & 31) == 0) red[t >> 5] = v;
    __syncthreads();
    if (t == 0) {
      unsigned long long s = 0;
      for (int w = 0; w < NT / 32; ++w) s += red[w];
      if (s) atomicAdd(&p.sync->acc, s);
      __threadfence();
      const uint32_t prev = atomicAdd(&p.sync->done, 1u);
      if (prev == G - 1) {
        const unsigned long long tot = atomicExch(&p.sync->acc, 0ull);
        *p.out_len = tot;
        p.sync->ticket = 0;
        p.sync->done = 0;
        __threadfence();
      }
    }
    return;
  }

  // materialise: decoupled look-back over CTA ranges
  __shared__ unsigned long long s_excl;
  if (t == 0) {
    const uint64_t ex = lookback_exclusive(p.status, vid, cta_cnt, p.epoch, p.err);
    s_excl = ex;
    if (ex != UINT64_MAX && ex + cta_cnt > p.out_cap)
      record_error(p.err, DEV_ERR_CAPACITY);
  }
  __syncthreads();
  const uint64_t ex = s_excl;
  if (ex == UINT64_MAX || ex + cta_cnt > p.out_cap) return;
  for (uint64_t q = t; q < cta_cnt; q += NT) {
    p.out[ex + q] = p.stage[stage_base + q];
    if (BSR) p.out_s[ex + q] = p.stage_s[stage_base + q];
  }
  if (t == 0) {
    if (vid == G - 1) *p.out_len = ex + cta_cnt;
    __threadfence();
    const uint32_t prev = atomicAdd(&p.sync->done, 1u);
    if (prev == G - 1) {
      p.sync->ticket = 0;
      p.sync->done = 0;
      __threadfence();
    }
  }
}

}  // namespace setops
