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
// na+nb) is cut into one contiguous diagonal range per CTA, whose merge-path
// co-ranks (both ends) one block search finds.  The CTA owns A[ia0, ia1) and
// reads B[ib0, ib1] -- B[ib1] is the one element past the range that can
// equal the CTA's last A element; a match is counted by the CTA owning its A
// element, so every match is counted once.
//
// The two runs stream independently through shared memory: fixed chunks of
// C elements, 16-byte aligned, loaded by 1-D TMA bulk copies into NS slots
// per stream, each slot with its own mbarrier; a slot is refilled as soon as
// its chunk is used up.
//
// Dense runs (at least one element per 64 values) are intersected in value
// windows: every element of window [w, w + 32*BMW) sets its bit in its
// set's window bitmap (atomicOr; for BSR the state word is stored at its
// base), the two tables are AND-ed word by word, and the set bits are the
// matches, already in ascending order (one block scan per window orders the
// output).  The next window starts at the smallest value not yet consumed,
// so empty value ranges are skipped.  Sparse runs are intersected chunk pair
// by chunk pair (binary search of each A element in the B chunk, advancing
// the chunk with the smaller maximum, as in the reference's block-wise SIMD
// algorithms, setops/src/intersect/shuffling.rs:69-112).
//
// Count mode adds per-CTA totals atomically; the last CTA writes the total.
// Materialise mode stages a CTA's matches in scratch at its first A index
// (an exclusive region: a CTA cannot emit more matches than A elements it
// owns); decoupled look-back over CTAs gives each CTA its output offset.
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

// Shapes: NT threads, chunks of C elements per stream, NS chunk slots per
// stream, window tables of BMW words per set.
template <int NT, int C, int NS, int BMW, bool BSR, bool MAT>
struct MergeCfg {
  static_assert(C % (4 * NT) == 0 || (4 * NT) % C == 0, "chunk / block shape");
  static_assert(C % 4 == 0 && BMW % (4 * NT) == 0, "16-byte groups");
  static_assert(NS >= 2, "need at least double buffering");
  static constexpr int kSlotWords = NS * C;                    // per stream
  static constexpr int kStreams = BSR ? 4 : 2;                 // keys (+ states)
  static constexpr size_t kSmemBytes =
      (size_t(kStreams) * kSlotWords + 2 * size_t(BMW)) * 4;
  // values (arrays: one bit each) or bases (BSR: one state word each) per window
  static constexpr uint32_t kWindow = BSR ? uint32_t(BMW) : uint32_t(BMW) * 32u;
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
    uint64_t est = uint64_t(double(d) * double(na) / double(na + nb));
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

// Occupancy target for register allocation: the shared-memory footprint
// allows at most this many CTAs per SM anyway.
template <int NT, int C, int NS, int BMW, bool BSR, bool MAT>
constexpr int merge_min_blocks() {
  constexpr size_t smem = MergeCfg<NT, C, NS, BMW, BSR, MAT>::kSmemBytes + 1024;
  constexpr int by_smem = int((228 * 1024) / smem);
  constexpr int by_threads = 2048 / NT;
  constexpr int b = by_smem < by_threads ? by_smem : by_threads;
  return b < 1 ? 1 : b;
}

template <int NT, int C, int NS, int BMW, bool BSR, bool MAT>
__global__ void __launch_bounds__(NT, (merge_min_blocks<NT, C, NS, BMW, BSR, MAT>()))
    merge_kernel(const MergeArgs p) {
  using Cfg = MergeCfg<NT, C, NS, BMW, BSR, MAT>;
  constexpr uint32_t WIN = Cfg::kWindow;

  extern __shared__ __align__(128) uint32_t smem[];
  uint32_t *slotA = smem;
  uint32_t *slotB = smem + Cfg::kSlotWords;
  uint32_t *slotSA = BSR ? smem + 2 * Cfg::kSlotWords : nullptr;
  uint32_t *slotSB = BSR ? smem + 3 * Cfg::kSlotWords : nullptr;
  uint32_t *tabA = smem + Cfg::kStreams * Cfg::kSlotWords;
  uint32_t *tabB = tabA + BMW;

  __shared__ __align__(8) uint64_t barA[NS];
  __shared__ __align__(8) uint64_t barB[NS];
  __shared__ uint32_t warp_sums[NT / 32];
  __shared__ uint32_t s_vid;
  __shared__ uint32_t s_bound[6];  // [pass % 3][stream], triple-buffered
  __shared__ unsigned long long red[NT / 32];
  __shared__ unsigned long long s_excl;
  __shared__ uint32_t s_edge[4];

  const int t = threadIdx.x;
  const int lane = t & 31;

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
    for (int i = 0; i < NS; ++i) {
      mbar_init(&barA[i], 1);
      mbar_init(&barB[i], 1);
    }
    fence_mbar_init();
  }
  for (int i = t; i < 2 * BMW; i += NT) tabA[i] = 0;  // tabA and tabB
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
  __shared__ unsigned long long s_ia0;
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
        if (global_ns() - t0 > kWaitLimitNs) {
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
  const bool work = ia1 > ia0 && be > ib0;

  const uint64_t pol = l2_evict_first_policy();
  Stream xa = make_stream<C>(A, BSR ? SA : nullptr, na, ia0, work ? ia1 : ia0);
  Stream xb = make_stream<C>(B, BSR ? SB : nullptr, nb, ib0, work ? be : ib0);
  uint32_t issuedA = 0, issuedB = 0;  // chunks issued (thread 0's view)
  if (t == 0) {
    for (; issuedA < xa.nc && issuedA < uint32_t(NS); ++issuedA)
      issue_chunk<C>(xa, issuedA, slotA + (issuedA % NS) * C,
                     BSR ? slotSA + (issuedA % NS) * C : nullptr,
                     &barA[issuedA % NS], pol);
    for (; issuedB < xb.nc && issuedB < uint32_t(NS); ++issuedB)
      issue_chunk<C>(xb, issuedB, slotB + (issuedB % NS) * C,
                     BSR ? slotSB + (issuedB % NS) * C : nullptr,
                     &barB[issuedB % NS], pol);
    // first / last values of both runs decide dense vs sparse handling
    if (work) {
      s_edge[0] = __ldg(A + ia0);
      s_edge[1] = __ldg(A + ia1 - 1);
      s_edge[2] = __ldg(B + ib0);
      s_edge[3] = __ldg(B + be - 1);
    }
  }
  __syncthreads();

  uint32_t ca = 0, cb = 0;  // current chunk of each stream
  bool aborted = false;
  uint64_t cnt = 0;      // count mode (BSR: elements)
  uint64_t cta_cnt = 0;  // materialise: matches staged so far

  // Valid slot-index range of chunk c of stream x.
  auto qrange = [&](const Stream &x, uint32_t c, uint32_t &q0, uint32_t &q1) {
    const uint64_t cs = x.c0 + uint64_t(c) * C;
    const uint64_t vs = x.s + x.off, ve = x.e + x.off;
    q0 = vs > cs ? uint32_t(vs - cs) : 0u;
    q1 = ve < cs + C ? uint32_t(ve - cs) : uint32_t(C);
  };
  // Waits (all threads) for chunk c of a stream; false on timeout.
  auto wait_chunk = [&](uint64_t *bars, uint32_t c) -> bool {
    const bool ok = mbar_wait_bounded(&bars[c % NS], (c / NS) & 1u, p.err);
    return !__syncthreads_or(!ok);
  };
  // Releases chunk c's slot (call after a barrier) and loads chunk c + NS.
  auto refill = [&](const Stream &x, uint32_t *slots, uint32_t *slots_s,
                    uint64_t *bars, uint32_t c, uint32_t &issued) {
    if (t == 0 && c + NS < x.nc) {
      const uint32_t nx = c + NS;
      issue_chunk<C>(x, nx, slots + (nx % NS) * C,
                     BSR ? slots_s + (nx % NS) * C : nullptr, &bars[nx % NS],
                     pol);
      issued = nx + 1;
    }
  };

  if (work) {
    const uint32_t a_first = s_edge[0], a_last = s_edge[1];
    const uint32_t b_first = s_edge[2], b_last = s_edge[3];
    const uint32_t vmin = a_first < b_first ? a_first : b_first;
    const uint32_t vmax = a_last > b_last ? a_last : b_last;
    const uint64_t elems = (ia1 - ia0) + (be - ib0);
    // dense when a window table pays for itself: at least one element per
    // 64 values (arrays) / per 2 bases (BSR) over the run's value span
    const bool dense = BSR ? (2 * elems >= uint64_t(vmax - vmin) + 1)
                           : (64 * elems >= uint64_t(vmax - vmin) + 1);
    if (dense) {
      // ================= dense: value windows =================
      // Per stream: current chunk and cursor (slot index of its first
      // unconsumed element).  Window [w, w + wlen) takes a prefix of what is
      // left of each stream, w being the smaller of the two cursor values.
      // One pass inserts from both streams' current chunks (one barrier); a
      // stream is finished for the window once an element past it is seen.
      if (!wait_chunk(barA, 0) || !wait_chunk(barB, 0)) aborted = true;
      uint32_t qa0, qa1, qb0, qb1;
      qrange(xa, 0, qa0, qa1);
      qrange(xb, 0, qb0, qb1);
      uint32_t curA = qa0, curB = qb0;
      bool doneA = false, doneB = false;
      uint32_t pass = 0;
      if (t < 6) s_bound[t] = 0xffffffffu;
      __syncthreads();
      constexpr int NWP = NT / 32;        // warps
      constexpr int WPW = BMW / NWP;      // table words per warp
      constexpr int KW = WPW / 32;        // words per lane
      static_assert(WPW % 32 == 0, "table words per warp must be a multiple of 32");
      while (!aborted) {
        const uint32_t va = slotA[(ca % NS) * C + curA];
        const uint32_t vb = slotB[(cb % NS) * C + curB];
        const uint32_t w = va < vb ? va : vb;
        const uint32_t wlen =
            (uint64_t(w) + WIN > 0x100000000ull) ? uint32_t(0x100000000ull - w) : WIN;
        bool actA = true, actB = true;  // still inserting into this window
        while (actA || actB) {
          uint32_t stopA = 0xffffffffu, stopB = 0xffffffffu;
#pragma unroll
          for (int sidx = 0; sidx < 2; ++sidx) {
            const bool isA = sidx == 0;
            if (!(isA ? actA : actB)) continue;
            const Stream &x = isA ? xa : xb;
            const uint32_t c = isA ? ca : cb;
            const uint32_t cur = isA ? curA : curB;
            const uint32_t *sl = (isA ? slotA : slotB) + (c % NS) * C;
            const uint32_t *sls = BSR ? (isA ? slotSA : slotSB) + (c % NS) * C : nullptr;
            uint32_t *tab = isA ? tabA : tabB;
            uint32_t q0, q1;
            qrange(x, c, q0, q1);
            const uint32_t g0 = cur >> 2, g1 = (q1 + 3) >> 2;
            uint32_t stop = 0xffffffffu;
            for (uint32_t g = g0 + t; g < g1; g += NT) {
              const uint4 v4 = reinterpret_cast<const uint4 *>(sl)[g];
              const uint32_t qb = 4 * g;
              const uint32_t o[4] = {v4.x - w, v4.y - w, v4.z - w, v4.w - w};
              const bool edge = (g == g0) | (g + 1 == g1);
              uint32_t outm = 0;
#pragma unroll
              for (int e2 = 0; e2 < 4; ++e2) {
                const bool valid = !edge || ((qb + e2 >= cur) && (qb + e2 < q1));
                const bool in = valid && (o[e2] < wlen);
                if (in) {
                  if (BSR) tab[o[e2]] = sls[qb + e2];
                  else atomicOr(&tab[o[e2] >> 5], 1u << (o[e2] & 31u));
                }
                outm |= uint32_t(valid && !in) << e2;
              }
              if (outm) {
                stop = qb + uint32_t(__ffs(outm) - 1);
                break;
              }
            }
            if (isA) stopA = stop;
            else stopB = stop;
          }
          const uint32_t wsa = __reduce_min_sync(0xffffffffu, stopA);
          const uint32_t wsb = __reduce_min_sync(0xffffffffu, stopB);
          const uint32_t slot = (pass % 3) * 2;
          if (lane == 0) {
            if (wsa != 0xffffffffu) atomicMin(&s_bound[slot], wsa);
            if (wsb != 0xffffffffu) atomicMin(&s_bound[slot + 1], wsb);
          }
          __syncthreads();  // chunk reads and bounds done
          const uint32_t bA = s_bound[slot], bB = s_bound[slot + 1];
          if (t < 2) s_bound[((pass + 2) % 3) * 2 + t] = 0xffffffffu;
          ++pass;
          bool waitA = false, waitB = false;
#pragma unroll
          for (int sidx = 0; sidx < 2; ++sidx) {
            const bool isA = sidx == 0;
            bool &act = isA ? actA : actB;
            if (!act) continue;
            const uint32_t bnd = isA ? bA : bB;
            if (bnd != 0xffffffffu) {  // the window ends inside this chunk
              (isA ? curA : curB) = bnd;
              act = false;
              continue;
            }
            const Stream &x = isA ? xa : xb;
            uint32_t &c = isA ? ca : cb;
            refill(x, isA ? slotA : slotB, isA ? slotSA : slotSB, isA ? barA : barB,
                   c, isA ? issuedA : issuedB);
            ++c;
            if (c >= x.nc) {
              (isA ? doneA : doneB) = true;
              act = false;
              continue;
            }
            uint32_t n0, n1;
            qrange(x, c, n0, n1);
            (isA ? curA : curB) = n0;
            (isA ? waitA : waitB) = true;
          }
          if (waitA || waitB) {
            bool ok = true;
            if (waitA) ok = mbar_wait_bounded(&barA[ca % NS], (ca / NS) & 1u, p.err);
            if (ok && waitB) ok = mbar_wait_bounded(&barB[cb % NS], (cb / NS) & 1u, p.err);
            if (__syncthreads_or(!ok)) {
              aborted = true;
              break;
            }
          }
        }
        if (aborted) break;
        // AND the two tables.  Warp wp owns words [wp*WPW, (wp+1)*WPW), lane l
        // words wp*WPW + 32k + l (conflict-free); word order = value order.
        const int wp = t >> 5;
        uint32_t *ta = tabA + wp * WPW + lane;
        uint32_t *tb = tabB + wp * WPW + lane;
        uint32_t hits = 0;
#pragma unroll 4
        for (int k = 0; k < KW; ++k) {
          const uint32_t m = ta[32 * k] & tb[32 * k];
          tb[32 * k] = 0;
          ta[32 * k] = MAT ? m : 0u;
          if (BSR) {
            if (MAT) hits += (m != 0);
            else cnt += __popc(m);
          } else {
            hits += __popc(m);
          }
        }
        if (MAT) {
          // warp totals -> block offsets (only when the window has matches)
          uint32_t wt = hits;
#pragma unroll
          for (int of = 16; of > 0; of >>= 1) wt += __shfl_xor_sync(0xffffffffu, wt, of);
          if (__syncthreads_or(hits != 0)) {
            if (lane == 0) warp_sums[wp] = wt;
            __syncthreads();
            uint32_t woff = 0, tot = 0;
#pragma unroll
            for (int i = 0; i < NWP; ++i) {
              const uint32_t v = warp_sums[i];
              woff += (i < wp) ? v : 0u;
              tot += v;
            }
            uint64_t o = stage_base + cta_cnt + woff;
            for (int k = 0; k < KW; ++k) {
              uint32_t m = ta[32 * k];
              if (!__any_sync(0xffffffffu, m != 0)) continue;
              ta[32 * k] = 0;
              const uint32_t pc = BSR ? uint32_t(m != 0) : uint32_t(__popc(m));
              uint32_t incl = pc;
#pragma unroll
              for (int of = 1; of < 32; of <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, of);
                if (lane >= of) incl += y;
              }
              uint64_t q = o + incl - pc;
              const uint32_t wbase = w + uint32_t(wp * WPW + 32 * k + lane) * (BSR ? 1u : 32u);
              if (BSR) {
                if (m) {
                  p.stage[q] = wbase;
                  p.stage_s[q] = m;
                }
              } else {
                while (m) {
                  p.stage[q++] = wbase + uint32_t(__ffs(m) - 1);
                  m &= m - 1;
                }
              }
              o += __shfl_sync(0xffffffffu, incl, 31);
            }
            cta_cnt += tot;
          }
          // every nonzero AND word was extracted and cleared above
        } else if (!BSR) {
          cnt += hits;
        }
        __syncthreads();  // tables clear before the next window's inserts
        // one run used up: nothing left in the other can match
        if (doneA || doneB) break;
        if (uint64_t(w) + wlen >= 0x100000000ull) break;
      }
    } else {
      // ============ sparse: chunk pairs, binary search of A in B ============
      if (!wait_chunk(barA, 0) || !wait_chunk(barB, 0)) aborted = true;
      while (!aborted) {
        const uint32_t *sa = slotA + (ca % NS) * C;
        const uint32_t *ssa = BSR ? slotSA + (ca % NS) * C : nullptr;
        const uint32_t *sb = slotB + (cb % NS) * C;
        const uint32_t *ssb = BSR ? slotSB + (cb % NS) * C : nullptr;
        uint32_t qa0, qa1, qb0, qb1;
        qrange(xa, ca, qa0, qa1);
        qrange(xb, cb, qb0, qb1);
        const uint32_t bmin = sb[qb0], bmax = sb[qb1 - 1];
        const uint32_t amax = sa[qa1 - 1];
        // thread t: contiguous A elements [qa0 + t*per, ...) in order
        constexpr uint32_t PER = (C + NT - 1) / NT;
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
          const uint32_t ex = block_exclusive_scan<NT>(hits, warp_sums, &tot);
          if (hits) {
            uint32_t *dst = p.stage + stage_base + cta_cnt + ex;
            uint32_t *dsts = BSR ? p.stage_s + stage_base + cta_cnt + ex : nullptr;
            uint32_t o = 0;
            for (uint32_t i = 0; i < PER; ++i) {
              const uint32_t q = my0 + i;
              if (q >= qa1) break;
              uint32_t st = 0;
              if (find(sa[q], st)) {
                if (BSR) {
                  st &= ssa[q];
                  if (st) {
                    dst[o] = sa[q];
                    dsts[o] = st;
                    ++o;
                  }
                } else {
                  dst[o++] = sa[q];
                }
              }
            }
          }
          cta_cnt += tot;
        } else if (!BSR) {
          cnt += hits;
        }
        __syncthreads();  // chunk reads done
        const bool advA = amax <= bmax, advB = bmax <= amax;
        if (advA) {
          refill(xa, slotA, slotSA, barA, ca, issuedA);
          ++ca;
        }
        if (advB) {
          refill(xb, slotB, slotSB, barB, cb, issuedB);
          ++cb;
        }
        if (ca >= xa.nc || cb >= xb.nc) break;
        if (advA && !wait_chunk(barA, ca)) { aborted = true; break; }
        if (advB && !wait_chunk(barB, cb)) { aborted = true; break; }
      }
    }
  }

  // ---- drain: every issued chunk must have landed before exit ----
  if (t == 0) {
    // chunks [first unwaited, issued) may still be in flight
    const uint32_t fa = ca, fb = cb;
    for (uint32_t c = fa; c < issuedA; ++c)
      mbar_wait_bounded(&barA[c % NS], (c / NS) & 1u, p.err);
    for (uint32_t c = fb; c < issuedB; ++c)
      mbar_wait_bounded(&barB[c % NS], (c / NS) & 1u, p.err);
  }
  __syncthreads();
  if (aborted) return;

  // ---- 3. combine ----
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

  // materialise: decoupled look-back over CTA ranges (warp 0)
  if (t < 32) {
    const uint64_t ex =
        lookback_exclusive_warp(p.status, vid, cta_cnt, p.epoch, p.err);
    if (t == 0) {
      s_excl = ex;
      if (ex != UINT64_MAX && ex + cta_cnt > p.out_cap)
        record_error(p.err, DEV_ERR_CAPACITY);
    }
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
