// merge.cuh -- merge-path intersection of two sorted, duplicate-free u32
// arrays (and of two BSR sets, merging on bases).
//
// Semantics follow the reference's naive_merge (setops/src/intersect/
// merge.rs:7-33) and branchless_merge_bsr (merge.rs:62-87): the output is the
// ascending intersection, with the Counter visitor's count
// (setops/src/visitor.rs:24-49; BSR: sum of popcount(state), visitor.rs:399).
//
// Work layout
// -----------
// Let A be the smaller input.  The merged sequence (A first on ties; length
// na+nb) is cut into one contiguous diagonal range per CTA; each CTA finds
// the merge-path co-rank of its end diagonal and takes its start from its
// predecessor.  The CTA owns A[ia0, ia1) and reads B[ib0, ib1] -- B[ib1] is
// the one element past the range that can equal the CTA's last A element; a
// match is counted by the CTA owning its A element, so every match is
// counted once.
//
// Streaming.  Both runs flow through shared memory in fixed chunks of C
// elements (16-byte aligned 1-D TMA bulk copies) into NSA / NSB slots.  Each
// slot has an mbarrier completed by the copy's byte count and a release
// counter: every warp adds one when it is done with the slot's chunk, and
// the warp that completes the count issues the copy of the chunk NS places
// later into the same slot.  Warps therefore never stop at a block-wide
// barrier between chunks, and no thread polls for free slots.
//
// Dense runs (A holds at least one element per 64 values; BSR: per 2 bases)
// are intersected group by group.  A group is a run of consecutive A
// elements of one chunk whose values span less than kSpan.  Its elements set
// their bits in bitmap T (BSR: their state words at their base); then every
// B element in the group's value range probes T.  Matches set their bit in
// bitmap M (indexed by value, so M is in ascending order); after the group
// one warp (a different one each group) writes M's set bits to the output in
// order.  Two T buffers alternate, so the next group's insertion and the last
// group's extraction and clearing share one phase: two barriers per group.
// A B chunk whose last value does not exceed the group's last value is
// released; otherwise the group ends and the chunk's remaining elements
// (found by a binary search for the group's last value) go to the next group.
//
// Sparse runs are intersected chunk pair by chunk pair (binary search of each
// A element in the B chunk, advancing the chunk with the smaller maximum, as
// in the reference's block-wise SIMD algorithms, setops/src/intersect/
// shuffling.rs:69-112).
//
// Count mode adds per-CTA totals atomically; the last CTA writes the total.
// Materialise mode stages a CTA's matches in scratch at its first A index
// (an exclusive region: a CTA cannot emit more matches than A elements it
// owns); each CTA sums its predecessors' published match counts to get its
// output offset.
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
  uint64_t *status;   // per-CTA count words, >= gridDim.x entries
  uint64_t *coranks;  // per-CTA end co-ranks (epoch-tagged), >= gridDim.x
  LaunchSync *sync;
  int *err;
  uint32_t epoch;
  // Device-side algorithm choice (k-set steps whose input length is only
  // known on the device): 0 = always run; 1 = run only when
  // max(na,nb)/min(na,nb) >= ratio_thr (search wins); 2 = only when below.
  int skip_rule;
  uint32_t ratio_thr;
};

// Shapes: NW warps; chunks of C elements; NSA / NSB chunk slots for A / B;
// T buffers of VW words (arrays: one bit per value, so a group spans
// < 32*VW values; BSR: one state word per base).
template <int NW, int C, int NSA, int NSB, int VW, bool BSR, bool MAT>
struct MergeCfg {
  static constexpr int kThreads = NW * 32;
  static_assert(C % 4 == 0 && VW % (4 * NW) == 0, "16-byte groups");
  static_assert(NSA >= 2 && NSB >= 2, "need at least double buffering");
  static_assert((VW & (VW - 1)) == 0, "power-of-two table");
  static constexpr uint32_t kSpan = BSR ? uint32_t(VW) : uint32_t(VW) * 32u;
  // T buffer: VW words plus a zero pad word group, so a probe can clamp an
  // out-of-range offset to the group's span + 1 and read a zero bit there
  static constexpr int kTabWords = VW + 4;
  // match bitmap M: one bit per value (arrays) or per base (BSR), and its
  // summary: one bit per nonzero M word
  static constexpr int kMWords = MAT ? int((kSpan / 32 + 1023) & ~1023u) : 0;
  static constexpr int kSumWords = kMWords / 32;
  static constexpr int kStreams = BSR ? 2 : 1;  // keys (+ states) per input
  static constexpr size_t kSlotWords = size_t(NSA + NSB) * C * kStreams;
  static constexpr size_t kSmemBytes =
      (kSlotWords + 2 * size_t(kTabWords) + size_t(kMWords) + size_t(kSumWords)) * 4;
  static constexpr int kTile = C;  // elements per chunk, for grid sizing
};

// One input's run [s, e) streamed through NS slots of C words.  Chunk c
// holds ring coordinates [c0 + c*C, c0 + (c+1)*C), where coordinate =
// element index + off and off is the misalignment of element 0 within its
// 16-byte group (so every chunk starts on a 16-byte boundary).
struct Stream {
  const uint32_t *al;    // 16-byte aligned base (coordinate 0)
  const uint32_t *al_s;  // states (BSR), same misalignment
  uint64_t n;            // array length
  uint64_t s, e;         // element run of this CTA
  uint64_t c0;           // coordinate of chunk 0
  uint32_t off;
  uint32_t nc;           // chunks covering the run
};

template <int C>
__device__ __forceinline__ Stream make_stream(const uint32_t *keys,
                                              const uint32_t *states,
                                              uint64_t n, uint64_t s,
                                              uint64_t e) {
  Stream x;
  const uintptr_t a = reinterpret_cast<uintptr_t>(keys);
  x.off = uint32_t((a >> 2) & 3);
  x.al = reinterpret_cast<const uint32_t *>(a & ~uintptr_t(15));
  x.al_s = states ? reinterpret_cast<const uint32_t *>(
                        reinterpret_cast<uintptr_t>(states) & ~uintptr_t(15))
                  : nullptr;
  x.n = n;
  x.s = s;
  x.e = e;
  x.c0 = (s + x.off) & ~uint64_t(3);
  x.nc = e > s ? uint32_t((e + x.off - x.c0 + C - 1) / C) : 0u;
  return x;
}

// Loads chunk c of x into slot words `dst` (and `dst_s` for states),
// completing on `bar`.  One thread.  Only the run's 16-byte groups are
// copied; groups that are partly outside the array (first group when the
// array is misaligned, last group at the array end) are loaded with plain
// loads, so nothing outside the array is read.
template <int C>
__device__ __forceinline__ void issue_chunk(const Stream &x, uint32_t c,
                                            uint32_t *dst, uint32_t *dst_s,
                                            uint64_t *bar, uint64_t pol) {
  const uint64_t lo = x.c0 + uint64_t(c) * C;
  uint64_t hi = lo + C;
  const uint64_t need = (x.e + x.off + 3) & ~uint64_t(3);
  if (hi > need) hi = need;
  const uint64_t arr_end = x.n + x.off;
  uint64_t blo = lo;
  if (blo < 4 && x.off > 0) blo = 4;  // group 0 is partial
  uint64_t bhi = arr_end & ~uint64_t(3);
  if (bhi > hi) bhi = hi;
  if (bhi < blo) bhi = blo;
  // head [lo, blo) and tail [bhi, hi): at most 3 + 3 words
  const uint64_t hcut = blo < hi ? blo : hi;
  for (uint64_t q = lo; q < hcut; ++q)
    if (q >= x.off && q < arr_end) {
      dst[q - lo] = __ldg(x.al + q);
      if (dst_s) dst_s[q - lo] = __ldg(x.al_s + q);
    }
  for (uint64_t q = (bhi > hcut ? bhi : hcut); q < hi; ++q)
    if (q >= x.off && q < arr_end) {
      dst[q - lo] = __ldg(x.al + q);
      if (dst_s) dst_s[q - lo] = __ldg(x.al_s + q);
    }
  const uint32_t bytes = uint32_t(bhi - blo) * 4u;
  // order the block's earlier generic-proxy reads of this slot (made visible
  // to this thread by the barrier before the refill) before the async-proxy
  // writes of the bulk copy
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  mbar_arrive_expect_tx(bar, dst_s ? 2 * bytes : bytes);
  if (bytes) {
    bulk_g2s(dst + (blo - lo), x.al + blo, bytes, bar, pol);
    if (dst_s) bulk_g2s(dst_s + (blo - lo), x.al_s + blo, bytes, bar, pol);
  }
}

// Merge-path co-rank of diagonal d: the smallest i with A[i] > B[d-1-i]
// (A first on ties).  All NT threads cooperate.  Round 1 probes exponentially
// spaced points around the proportional estimate d*na/(na+nb) (exact for
// evenly spread values, close for most data), so the later (NT+1)-ary rounds
// narrow a small bracket whose probes stay in a few DRAM pages.
template <int NT>
__device__ __forceinline__ uint64_t corank_search(const uint32_t *A,
                                                  uint64_t na,
                                                  const uint32_t *B,
                                                  uint64_t nb, uint64_t d) {
  __shared__ unsigned long long s_lo, s_hi;
  const int t = threadIdx.x;
  uint64_t lo = d > nb ? d - nb : 0;
  uint64_t hi = d < na ? d : na;  // answer in [lo, hi]
  if (hi - lo > uint64_t(NT)) {
    if (t == 0) {
      s_lo = lo;
      s_hi = hi;
    }
    __syncthreads();
    uint64_t est = guess_scale(d, na + nb, na);
    if (est < lo) est = lo;
    if (est >= hi) est = hi - 1;
    // probes est + (2^k - 1) and est - 2^k, k = 0..47
    if (t < 96) {
      const int k = t % 48;
      const uint64_t off = (k >= 47) ? (uint64_t(1) << 47) : (uint64_t(1) << k);
      bool ok;
      uint64_t x;
      if (t < 48) {
        x = est + off - 1;
        ok = x < hi && x >= est;
      } else {
        x = est - off;
        ok = est >= lo + off;
      }
      if (ok) {
        if (__ldg(A + x) <= __ldg(B + (d - 1 - x))) atomicMax(&s_lo, x + 1);
        else atomicMin(&s_hi, x);
      }
    }
    __syncthreads();
    lo = s_lo;
    hi = s_hi;
    __syncthreads();
  }
  while (hi > lo) {
    const uint64_t span = hi - lo;
    if (span <= uint64_t(NT)) {
      bool pr = false;
      if (uint64_t(t) < span) {
        const uint64_t x = lo + t;
        pr = __ldg(A + x) <= __ldg(B + (d - 1 - x));
      }
      lo += uint64_t(__syncthreads_count(pr));
      break;
    }
    const uint64_t x = lo + (uint64_t(t + 1) * span) / (NT + 1);
    const uint64_t c =
        uint64_t(__syncthreads_count(__ldg(A + x) <= __ldg(B + (d - 1 - x))));
    const uint64_t nhi = (c < uint64_t(NT)) ? lo + ((c + 1) * span) / (NT + 1) : hi;
    if (c > 0) lo = lo + (c * span) / (NT + 1) + 1;
    hi = nhi;
  }
  return lo;
}

// Exclusive scan of one uint32 per thread, synchronising on named barrier 1
// (all NT threads).  `warp_sums` needs NT/32 entries; the caller must pass
// another barrier before the next call.
template <int NT>
__device__ __forceinline__ uint32_t scan_exclusive_nb(uint32_t v,
                                                      uint32_t *warp_sums,
                                                      uint32_t *total) {
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  named_bar_sync<1, NT>();
  uint32_t wpre = 0, tot = 0;
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    const uint32_t s = warp_sums[w];
    wpre += (w < warp) ? s : 0u;
    tot += s;
  }
  *total = tot;
  return wpre + x - v;
}

// Exclusive prefix of per-CTA counts, for blocks whose CTA ids come from an
// atomic ticket (so every predecessor is running or done).  The CTA
// publishes its own count (epoch-tagged), then all threads sum the published
// counts of every predecessor at once: one or two rounds of loads however
// many CTAs precede it, where a chained look-back needs one round per 32
// predecessors when all CTAs finish together.  All NT threads (named
// barrier 1); returns UINT64_MAX after recording a timeout.
template <int NT>
__device__ __forceinline__ uint64_t predecessor_sum(uint64_t *status,
                                                    uint32_t vid,
                                                    uint64_t count,
                                                    uint32_t epoch, int *err,
                                                    unsigned long long *red) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if (t == 0) st_release_u64(&status[vid], pack_status(epoch, kFlagAggregate, count));
  const uint32_t ep = epoch & 0xffffu;
  uint64_t sum = 0;
  bool bad = false;
  for (uint32_t j = uint32_t(t); j < vid && !bad; j += NT) {
    uint64_t w = ld_acquire_u64(&status[j]);
    if (uint32_t(w >> 48) != ep) {
      const uint64_t t0 = global_ns();
      do {
        if (global_ns() - t0 > wait_limit_ns()) {
          record_error(err, DEV_ERR_TIMEOUT_LOOKBACK);
          bad = true;
          break;
        }
        w = ld_acquire_u64(&status[j]);
      } while (uint32_t(w >> 48) != ep);
    }
    sum += w & kValueMask;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  const bool any_bad = __any_sync(0xffffffffu, bad);
  if (lane == 0) red[warp] = any_bad ? ~0ull : sum;
  named_bar_sync<1, NT>();
  uint64_t tot = 0;
  bool fail = false;
#pragma unroll
  for (int w = 0; w < NT / 32; ++w) {
    const unsigned long long v = red[w];
    fail |= (v == ~0ull);
    tot += v;
  }
  return fail ? UINT64_MAX : tot;
}

// Occupancy target for register allocation: the shared-memory footprint
// allows at most this many CTAs per SM anyway.
template <int NW, int C, int NSA, int NSB, int VW, bool BSR, bool MAT>
constexpr int merge_min_blocks() {
  using Cfg = MergeCfg<NW, C, NSA, NSB, VW, BSR, MAT>;
  constexpr size_t smem = Cfg::kSmemBytes + 2048;
  constexpr int by_smem = int((228 * 1024) / smem);
  constexpr int by_threads = 2048 / Cfg::kThreads;
  constexpr int b = by_smem < by_threads ? by_smem : by_threads;
  return b < 1 ? 1 : b;
}

template <int NW, int C, int NSA, int NSB, int VW, bool BSR, bool MAT>
__global__ void __launch_bounds__(
    MergeCfg<NW, C, NSA, NSB, VW, BSR, MAT>::kThreads,
    (merge_min_blocks<NW, C, NSA, NSB, VW, BSR, MAT>()))
    merge_kernel(const MergeArgs p) {
  using Cfg = MergeCfg<NW, C, NSA, NSB, VW, BSR, MAT>;
  constexpr int NT = Cfg::kThreads;
  constexpr uint32_t SPAN = Cfg::kSpan;
  constexpr uint32_t TW = uint32_t(Cfg::kTabWords);

  extern __shared__ __align__(128) uint32_t smem[];
  uint32_t *slotA = smem;            // NSA chunks
  uint32_t *slotB = smem + NSA * C;  // NSB chunks
  uint32_t *slotSA = BSR ? smem + (NSA + NSB) * C : nullptr;
  uint32_t *slotSB = BSR ? slotSA + NSA * C : nullptr;
  uint32_t *tab = smem + Cfg::kSlotWords;  // two T buffers of TW words
  uint32_t *mbits = tab + 2 * TW;          // match bitmap (materialise)
  uint32_t *msum = mbits + Cfg::kMWords;   // its nonzero-word summary

  __shared__ __align__(8) uint64_t fullA[NSA], fullB[NSB];
  __shared__ uint32_t relA[NSA], relB[NSB];    // warps done with the chunk
  __shared__ uint32_t lastA[NSA], lastB[NSB];  // last chunk issued + 1
  __shared__ uint32_t warp_sums[NW];
  __shared__ unsigned long long red[NW];
  __shared__ unsigned long long s_ia0, s_cnt;
  __shared__ uint32_t s_vid, s_abort;
  __shared__ uint32_t s_edge[2];

  const int t = threadIdx.x;
  const int lane = t & 31;
  const int warp = t >> 5;

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
    for (int i = 0; i < NSA; ++i) mbar_init(&fullA[i], 1);
    for (int i = 0; i < NSB; ++i) mbar_init(&fullB[i], 1);
    s_abort = 0;
    s_cnt = 0;
    fence_mbar_init();
  }
  if (t < NSA) { relA[t] = 0; lastA[t] = 0; }
  if (t < NSB) { relB[t] = 0; lastB[t] = 0; }
  for (int i = t; i < int(2 * TW + Cfg::kMWords + Cfg::kSumWords) / 4; i += NT)
    reinterpret_cast<uint4 *>(tab)[i] = make_uint4(0, 0, 0, 0);
  __syncthreads();
  const uint32_t vid = s_vid;
  const uint32_t G = gridDim.x;
  uint64_t D = (total + G - 1) / G;
  D = ((D + C - 1) / C) * C;
  const uint64_t d0 = (uint64_t(vid) * D < total) ? uint64_t(vid) * D : total;
  const uint64_t d1 = (d0 + D < total) ? d0 + D : total;

  // ---- 1. this CTA's runs: A[ia0, ia1) and B[ib0, ib1] ----
  // Each CTA searches the co-rank of its end diagonal and publishes it; its
  // start is its predecessor's end (CTA ids come from an atomic ticket, so
  // the predecessor is running or done).
  const uint64_t ia1 = corank_search<NT>(A, na, B, nb, d1);
  if (t == 0) {
    st_release_u64(&p.coranks[vid], pack_status(p.epoch, kFlagPrefix, ia1));
    uint64_t v0 = 0;
    if (vid > 0) {
      const uint64_t t0 = global_ns();
      for (;;) {
        const uint64_t w = ld_acquire_u64(&p.coranks[vid - 1]);
        if (uint32_t(w >> 48) == (p.epoch & 0xffffu) && ((w >> 46) & 3) == kFlagPrefix) {
          v0 = w & kValueMask;
          break;
        }
        if (global_ns() - t0 > wait_limit_ns()) {
          record_error(p.err, DEV_ERR_TIMEOUT_LOOKBACK);
          v0 = UINT64_MAX;
          break;
        }
      }
    }
    s_ia0 = v0;
  }
  __syncthreads();
  if (s_ia0 == UINT64_MAX) return;  // error recorded; the host resets state
  const uint64_t ia0 = s_ia0;
  const uint64_t ib0 = d0 - ia0;
  const uint64_t ib1 = d1 - ia1;
  // B[ib1] is the one element past the range that can match A[ia1-1]
  const uint64_t be = ib1 < nb ? ib1 + 1 : nb;
  const uint64_t stage_base = ia0;  // matches <= owned A elements
  const uint64_t cap = ia1 > ia0 ? ia1 - ia0 : 0;
  const bool work = ia1 > ia0 && be > ib0;
  const Stream xa = make_stream<C>(A, BSR ? SA : nullptr, na, ia0, work ? ia1 : ia0);
  const Stream xb = make_stream<C>(B, BSR ? SB : nullptr, nb, ib0, work ? be : ib0);
  volatile uint32_t *abortp = &s_abort;
  const uint64_t pol = l2_evict_first_policy();

  // Valid slot-index range of chunk c of stream x.
  auto qrange = [&](const Stream &x, uint32_t c, uint32_t &q0, uint32_t &q1) {
    const uint64_t cs = x.c0 + uint64_t(c) * C;
    const uint64_t vs = x.s + x.off, ve = x.e + x.off;
    q0 = vs > cs ? uint32_t(vs - cs) : 0u;
    q1 = ve < cs + C ? uint32_t(ve - cs) : uint32_t(C);
  };
  // This warp is done with chunk c of A (B): the last warp to say so loads
  // chunk c + NS into the slot.  Call with the whole warp.
  auto release_a = [&](uint32_t c) {
    __syncwarp();
    if (lane == 0) {
      const uint32_t s = c % NSA;
      __threadfence_block();
      if (atomicAdd(&relA[s], 1u) == uint32_t(NW - 1)) {
        relA[s] = 0;
        __threadfence_block();
        const uint32_t nx = c + NSA;
        if (nx < xa.nc) {
          issue_chunk<C>(xa, nx, slotA + s * C, BSR ? slotSA + s * C : nullptr, &fullA[s], pol);
          lastA[s] = nx + 1;
        }
      }
    }
  };
  auto release_b = [&](uint32_t c) {
    __syncwarp();
    if (lane == 0) {
      const uint32_t s = c % NSB;
      __threadfence_block();
      if (atomicAdd(&relB[s], 1u) == uint32_t(NW - 1)) {
        relB[s] = 0;
        __threadfence_block();
        const uint32_t nx = c + NSB;
        if (nx < xb.nc) {
          issue_chunk<C>(xb, nx, slotB + s * C, BSR ? slotSB + s * C : nullptr, &fullB[s], pol);
          lastB[s] = nx + 1;
        }
      }
    }
  };

  uint32_t cnt = 0;      // count mode (BSR: elements)
  uint64_t cta_cnt = 0;  // materialise: matches staged

  if (work) {
    if (t == 0) {
      for (uint32_t c = 0; c < xa.nc && c < uint32_t(NSA); ++c) {
        issue_chunk<C>(xa, c, slotA + c * C, BSR ? slotSA + c * C : nullptr, &fullA[c], pol);
        lastA[c] = c + 1;
      }
      for (uint32_t c = 0; c < xb.nc && c < uint32_t(NSB); ++c) {
        issue_chunk<C>(xb, c, slotB + c * C, BSR ? slotSB + c * C : nullptr, &fullB[c], pol);
        lastB[c] = c + 1;
      }
      s_edge[0] = __ldg(A + ia0);
      s_edge[1] = __ldg(A + ia1 - 1);
    }
    __syncthreads();
    const uint64_t aspan = uint64_t(s_edge[1] - s_edge[0]) + 1;
    // groups pay for themselves when A holds at least one element per 64
    // values (arrays) / per 2 bases (BSR)
    const bool dense = BSR ? (2 * cap >= aspan) : (64 * cap >= aspan);
    uint32_t ca = 0, cb = 0;  // current chunk of each stream
    uint32_t qa0, qa1, qb0, qb1;
    qrange(xa, 0, qa0, qa1);

    if (dense) {
      // ================= dense: groups =================
      uint32_t i0 = qa0;  // first slot index of the next group in chunk ca
      uint32_t g = 0;     // groups run so far
      uint32_t wprev = 0, zprev = 0;  // last group's base value, T words used
      uint32_t bres = 0;  // first unconsumed index of the retained B chunk
      bool more = true;
      for (;;) {
        // ---- phase 1: last group's output and clearing, next insertion ----
        if (g > 0) {
          uint32_t *tp = tab + ((g - 1) & 1u) * TW;
          if (MAT && warp == int((g - 1) % NW)) {
            // this group's extractor.  Lane l owns summary words
            // [l*SPL, l*SPL + SPL), i.e. the M words they flag, in value order.
            constexpr int SPL = Cfg::kSumWords >= 32 ? Cfg::kSumWords / 32 : 1;
            const bool own = lane * SPL < Cfg::kSumWords;
            uint32_t sw[SPL];
            uint32_t pc = 0;
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
              sw[k] = own ? msum[lane * SPL + k] : 0u;
              uint32_t f = sw[k];
              while (f) {
                const uint32_t mi = uint32_t(lane * SPL + k) * 32u + uint32_t(__ffs(f) - 1);
                f &= f - 1;
                pc += __popc(mbits[mi]);
              }
            }
            uint32_t incl = pc;
#pragma unroll
            for (int of = 1; of < 32; of <<= 1) {
              const uint32_t y = __shfl_up_sync(0xffffffffu, incl, of);
              if (lane >= of) incl += y;
            }
            const uint32_t tot = __shfl_sync(0xffffffffu, incl, 31);
            const uint64_t base = s_cnt;  // matches staged by earlier groups
            uint64_t q = base + incl - pc;
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
              uint32_t f = sw[k];
              if (f) msum[lane * SPL + k] = 0;
              while (f) {
                const uint32_t mi = uint32_t(lane * SPL + k) * 32u + uint32_t(__ffs(f) - 1);
                f &= f - 1;
                uint32_t m = mbits[mi];
                mbits[mi] = 0;
                while (m) {
                  const uint32_t off = mi * 32u + uint32_t(__ffs(m) - 1);  // value (base) offset
                  m &= m - 1;
                  if (q < cap) {
                    p.stage[stage_base + q] = wprev + off;
                    if (BSR) p.stage_s[stage_base + q] = tp[off];
                  }
                  ++q;
                }
              }
            }
            __syncwarp();
            if (lane == 0) s_cnt = base + tot;
            if (BSR) {
              // the extractor read T's states: it also clears T
              const uint32_t zr = (zprev + 3u) & ~3u;
              for (uint32_t i = 4u * uint32_t(lane); i < zr; i += 128u)
                *reinterpret_cast<uint4 *>(tp + i) = make_uint4(0, 0, 0, 0);
            }
          }
          if (!MAT || !BSR) {
            // clear the last group's T words, warp by warp
            constexpr uint32_t RW = uint32_t(VW / NW);
            const uint32_t rb = uint32_t(warp) * RW;
            const uint32_t zr = (zprev + 3u) & ~3u;
            const uint32_t re = (rb + RW < zr) ? rb + RW : zr;
            for (uint32_t i = rb + 4u * uint32_t(lane); i < re; i += 128u)
              *reinterpret_cast<uint4 *>(tp + i) = make_uint4(0, 0, 0, 0);
          }
        }
        if (!more) break;

        // ---- group g: A[i0, i1) of chunk ca ----
        mbar_wait_abortable(&fullA[ca % NSA], (ca / NSA) & 1u, p.err, abortp);
        const uint32_t *sa = slotA + (ca % NSA) * C;
        const uint32_t *ssa = BSR ? slotSA + (ca % NSA) * C : nullptr;
        const uint32_t w = sa[i0];
        uint32_t i1 = qa1;
        if (sa[qa1 - 1] - w >= SPAN) {
          // first index past i0 whose value is >= w + SPAN
          uint32_t lo = i0 + 1, len = qa1 - lo;
          while (len > 0) {
            const uint32_t h = len >> 1;
            if (sa[lo + h] - w < SPAN) {
              lo += h + 1;
              len -= h + 1;
            } else {
              len = h;
            }
          }
          i1 = lo;
        }
        const uint32_t alast = sa[i1 - 1];
        const uint32_t span = (alast - w < SPAN) ? alast - w : SPAN - 1;
        uint32_t *tg = tab + (g & 1u) * TW;
        for (uint32_t u = (i0 >> 2) + uint32_t(t); u < ((i1 + 3) >> 2); u += NT) {
          const uint4 v4 = reinterpret_cast<const uint4 *>(sa)[u];
          const uint32_t o[4] = {v4.x - w, v4.y - w, v4.z - w, v4.w - w};
          uint32_t okm = 0xfu;  // slots inside [i0, i1)
          const uint32_t q = 4 * u;
          if (q < i0 || q + 4 > i1) {
#pragma unroll
            for (int e = 0; e < 4; ++e)
              if (q + e < i0 || q + e >= i1) okm &= ~(1u << e);
          }
          if (BSR) {
            const uint4 s4 = reinterpret_cast<const uint4 *>(ssa)[u];
            const uint32_t st[4] = {s4.x, s4.y, s4.z, s4.w};
#pragma unroll
            for (int e = 0; e < 4; ++e)
              if ((okm >> e) & 1u) tg[o[e] & (SPAN - 1)] = st[e];
          } else {
#pragma unroll
            for (int e = 0; e < 4; ++e)
              if ((okm >> e) & 1u) atomicOr(&tg[(o[e] & (SPAN - 1)) >> 5], 1u << (o[e] & 31));
          }
        }
        if (i1 == qa1) {  // chunk used up: release it
          release_a(ca);
          ++ca;
          if (ca < xa.nc) {
            qrange(xa, ca, qa0, qa1);
            i0 = qa0;
          }
        } else {
          i0 = i1;
        }
        const bool a_left = ca < xa.nc;
        __syncthreads();  // T(g) complete; the last group's output written

        // ---- phase 2: probe B chunks against T(g) ----
        const uint32_t oclamp = span + 1;  // offset of a zero bit / word
        bool bdone = false;
        for (;;) {
          mbar_wait_abortable(&fullB[cb % NSB], (cb / NSB) & 1u, p.err, abortp);
          const uint32_t *sb = slotB + (cb % NSB) * C;
          const uint32_t *ssb = BSR ? slotSB + (cb % NSB) * C : nullptr;
          qrange(xb, cb, qb0, qb1);
          const uint32_t qs = bres > qb0 ? bres : qb0;  // skip what is consumed
          const uint32_t bmax = sb[qb1 - 1];
          const bool keep = bmax > alast;  // chunk outlives this group
          uint32_t qe = qb1;
          if (keep) {
            // first index whose value is past the group (exists: bmax > alast)
            uint32_t lo = qs, len = qb1 - qs;
            while (len > 0) {
              const uint32_t h = len >> 1;
              if (sb[lo + h] <= alast) {
                lo += h + 1;
                len -= h + 1;
              } else {
                len = h;
              }
            }
            qe = lo;
          }
          for (uint32_t u = (qs >> 2) + uint32_t(t); u < ((qe + 3) >> 2); u += NT) {
            const uint4 v4 = reinterpret_cast<const uint4 *>(sb)[u];
            uint32_t o[4] = {v4.x - w, v4.y - w, v4.z - w, v4.w - w};
            const uint32_t q = 4 * u;
            if (q < qs || q + 4 > qe) {
#pragma unroll
              for (int e = 0; e < 4; ++e)
                if (q + e < qs || q + e >= qe) o[e] = oclamp;
            }
            uint32_t hit = 0, wd[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              o[e] = o[e] < oclamp ? o[e] : oclamp;
              wd[e] = tg[BSR ? o[e] : (o[e] >> 5)];
            }
            uint32_t st[4] = {0, 0, 0, 0};
            if (BSR) {
              const uint4 s4 = reinterpret_cast<const uint4 *>(ssb)[u];
              st[0] = s4.x; st[1] = s4.y; st[2] = s4.z; st[3] = s4.w;
#pragma unroll
              for (int e = 0; e < 4; ++e) hit |= uint32_t((wd[e] & st[e]) != 0) << e;
            } else {
#pragma unroll
              for (int e = 0; e < 4; ++e) hit |= ((wd[e] >> (o[e] & 31)) & 1u) << e;
            }
            if (hit) {
#pragma unroll
              for (int e = 0; e < 4; ++e) {
                if (!((hit >> e) & 1u)) continue;
                if (MAT) {
                  if (BSR) tg[o[e]] = wd[e] & st[e];
                  const uint32_t mw = o[e] >> 5;
                  if (atomicOr(&mbits[mw], 1u << (o[e] & 31)) == 0u)
                    atomicOr(&msum[mw >> 5], 1u << (mw & 31));  // first bit of the word
                } else {
                  cnt += BSR ? __popc(wd[e] & st[e]) : 1u;
                }
              }
            }
          }
          if (!keep) {  // chunk used up: release it
            release_b(cb);
            bres = 0;
            ++cb;
            if (cb >= xb.nc) {
              bdone = true;
              break;
            }
          } else {
            bres = qe;
          }
          if (bmax >= alast) break;  // group used up
        }
        wprev = w;
        zprev = BSR ? span + 1 : (span >> 5) + 1;
        ++g;
        // one run used up (nothing left in the other can match), or a wait
        // gave up: the next phase 1 is the last
        more = !__syncthreads_or(bdone || !a_left || *abortp != 0u);
      }
      if (MAT) {
        __syncthreads();  // the last extraction's count reaches every warp
        cta_cnt = s_cnt;
      }
    } else {
      // ============ sparse: chunk pairs, binary search of A in B ============
      constexpr uint32_t PER = (C + NT - 1) / NT;
      for (;;) {
        mbar_wait_abortable(&fullA[ca % NSA], (ca / NSA) & 1u, p.err, abortp);
        mbar_wait_abortable(&fullB[cb % NSB], (cb / NSB) & 1u, p.err, abortp);
        const uint32_t *sa = slotA + (ca % NSA) * C;
        const uint32_t *ssa = BSR ? slotSA + (ca % NSA) * C : nullptr;
        const uint32_t *sb = slotB + (cb % NSB) * C;
        const uint32_t *ssb = BSR ? slotSB + (cb % NSB) * C : nullptr;
        qrange(xa, ca, qa0, qa1);
        qrange(xb, cb, qb0, qb1);
        const uint32_t bmin = sb[qb0], bmax = sb[qb1 - 1];
        const uint32_t amax = sa[qa1 - 1];
        // thread t: contiguous A elements [qa0 + t*PER, ...) in order
        const uint32_t my0 = qa0 + uint32_t(t) * PER;
        uint32_t hits = 0;
        auto find = [&](uint32_t v, uint32_t &st) -> bool {
          if (v < bmin || v > bmax) return false;
          uint32_t lo = qb0, len = qb1 - qb0;
          while (len > 0) {
            const uint32_t h = len >> 1;
            if (sb[lo + h] < v) {
              lo += h + 1;
              len -= h + 1;
            } else {
              len = h;
            }
          }
          if (lo >= qb1 || sb[lo] != v) return false;
          if (BSR) st = ssb[lo];
          return true;
        };
        for (uint32_t i = 0; i < PER; ++i) {
          const uint32_t q = my0 + i;
          if (q >= qa1) break;
          uint32_t st = 0;
          if (find(sa[q], st)) {
            if (BSR) {
              st &= ssa[q];
              if (st) {
                if (MAT) ++hits;
                else cnt += __popc(st);
              }
            } else {
              ++hits;
            }
          }
        }
        if (MAT) {
          uint32_t tot;
          const uint32_t ex = scan_exclusive_nb<NT>(hits, warp_sums, &tot);
          if (hits) {
            uint64_t o = cta_cnt + ex;
            for (uint32_t i = 0; i < PER; ++i) {
              const uint32_t q = my0 + i;
              if (q >= qa1) break;
              uint32_t st = 0;
              if (find(sa[q], st)) {
                if (BSR) st &= ssa[q];
                if (!BSR || st) {
                  if (o < cap) {
                    p.stage[stage_base + o] = sa[q];
                    if (BSR) p.stage_s[stage_base + o] = st;
                  }
                  ++o;
                }
              }
            }
          }
          cta_cnt += tot;
        } else if (!BSR) {
          cnt += hits;
        }
        const bool advA = amax <= bmax, advB = bmax <= amax;
        if (advA) {
          release_a(ca);
          ++ca;
        }
        if (advB) {
          release_b(cb);
          ++cb;
        }
        const bool stop = ca >= xa.nc || cb >= xb.nc;
        if (MAT) {
          // the scan above holds barriers: leave together
          if (__syncthreads_or(stop || *abortp != 0u)) break;
        } else if (stop) {
          break;
        }
      }
    }
  }

  // every thread is past its last wait and issue: no copy may still be in
  // flight when the CTA exits
  const bool aborted = __syncthreads_or(*abortp != 0u);
  if (t == 0) {
    for (int s = 0; s < NSA; ++s)
      if (lastA[s]) mbar_wait_bounded(&fullA[s], ((lastA[s] - 1) / NSA) & 1u, p.err);
    for (int s = 0; s < NSB; ++s)
      if (lastB[s]) mbar_wait_bounded(&fullB[s], ((lastB[s] - 1) / NSB) & 1u, p.err);
  }
  if (aborted) return;

  // ---- 3. combine ----
  if (!MAT) {
    uint64_t v = cnt;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (t == 0) {
      unsigned long long s = 0;
      for (int w = 0; w < NW; ++w) s += red[w];
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

  // materialise: output offset = sum of the predecessors' match counts
  const uint64_t ex = predecessor_sum<NT>(p.status, vid, cta_cnt, p.epoch, p.err, red);
  if (ex == UINT64_MAX) return;
  if (ex + cta_cnt > p.out_cap || cta_cnt > cap) {
    if (t == 0) record_error(p.err, DEV_ERR_CAPACITY);
    return;
  }
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
