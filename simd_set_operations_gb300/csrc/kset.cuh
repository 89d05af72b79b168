// kset.cuh -- the intersection of k sorted, duplicate-free u32 sets in one
// launch.  Same result as svs_generic (setops/src/intersect/svs.rs:50-73)
// with naive_merge steps (setops/src/intersect/merge.rs:7-33): the
// ascending elements present in every set.
//
// The reference (and the step-wise GPU path) intersects smallest-first,
// writing an intermediate result per step.  Here every set is read once and
// nothing intermediate leaves shared memory:
//
//   CTA c owns the run S0[c*n0/G, (c+1)*n0/G) of the smallest set S0 and, for
//   every other set Sj, a cursor bj (first placed by one round of probes per
//   set around a guess, at most sqrt(|Sj|)/8 elements before the first
//   element >= the run's first value; the rounds spread over the warps).  Per tile of the run (TA elements,
//   values [w, alast]):
//     1. the tile sets bits in bitmap X (dense: one bit per value of
//        [w, alast]) or is kept as a sorted table with a bitmap X of its
//        positions (sparse);
//     2. for j = 1 .. k-1: Sj is read from bj in windows (UB 16-byte loads
//        per thread in flight, as in window.cuh); an element whose bit (value
//        or, via a binary search of the table, position) is set in X sets
//        the same bit in Y; elements up to alast are counted to move bj;
//        then X is cleared and the two swap, so X holds the survivors;
//     3. count mode counts X; materialise mode extracts X in value order to
//        the CTA's staging run (its first S0 index onward).
//   Materialise mode then places the runs like window.cuh: per-CTA counts,
//   one grid-wide barrier (cooperative launch), copies to the prefix.
#pragma once

#include "tile.cuh"

namespace setops {

constexpr int kKsetMax = 16;

struct KsetArgs {
  const uint32_t *sets[kKsetMax];  // sorted by length: sets[0] the smallest
  uint64_t lens[kKsetMax];
  int k;
  uint32_t *stage;    // materialise: >= lens[0] words
  uint32_t *out;
  uint64_t out_cap;
  uint64_t *out_len;  // device: result length (count mode: the count)
  uint64_t *coranks;  // >= gridDim.x words
  LaunchSync *sync;
  int *err;
};

template <int NT, int UA, int UB, int VW, bool MAT>
struct KsetCfg {
  static_assert(NT % 32 == 0 && NT >= 64, "whole warps, two at least");
  static constexpr int kTile = 4 * UA * NT;
  static_assert((VW & (VW - 1)) == 0 && VW >= kTile, "a sparse tile fits a buffer");
  static constexpr int kBufWords = VW + 8;                 // each of the two buffers
  static constexpr int kPosWords = (kTile + 8 + 31) / 32;  // sparse: position bitmap
  static_assert(2 * kPosWords <= kBufWords, "two position bitmaps fit a buffer");
  static constexpr uint32_t kSpan = uint32_t(VW) * 32u;
  static constexpr size_t kSmemBytes = size_t(2 * kBufWords) * 4;
};

template <int NT, int UA, int UB, int VW, int MINB, bool MAT>
__global__ void __launch_bounds__(NT, MINB) kset_kernel(const KsetArgs p) {
  using Cfg = KsetCfg<NT, UA, UB, VW, MAT>;
  constexpr int NW = NT / 32;
  constexpr uint32_t SPAN = Cfg::kSpan;
  constexpr uint32_t TA = Cfg::kTile;

  extern __shared__ __align__(128) uint32_t smem[];
  uint32_t *bufU = smem;                   // dense: bitmap; sparse: the sorted tile
  uint32_t *bufV = smem + Cfg::kBufWords;  // dense: bitmap; sparse: two position bitmaps
  __shared__ unsigned long long s_b[kKsetMax];  // cursors of sets 1..k-1
  __shared__ uint32_t s_le[3];
  __shared__ uint32_t warp_sums[NW];
  __shared__ unsigned long long red[NW];

  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int k = p.k;
  const uint32_t *A = p.sets[0];
  const uint64_t na = p.lens[0];
  bool any_empty = false;
  for (int j = 0; j < k; ++j) any_empty |= p.lens[j] == 0;
  const uint32_t G = gridDim.x;
  const uint64_t ca0 = any_empty ? 0 : uint64_t(blockIdx.x) * na / G;
  const uint64_t ca1 = any_empty ? 0 : (uint64_t(blockIdx.x) + 1) * na / G;

  for (int i = t; i < 2 * Cfg::kBufWords / 4; i += NT)
    reinterpret_cast<uint4 *>(smem)[i] = make_uint4(0, 0, 0, 0);
  if (t < 3) s_le[t] = 0;

  uint64_t v0, v1;
  aligned_body(A, ca0, ca1, v0, v1);
  const uint32_t ntiles = ca1 > ca0 ? uint32_t(v1 > v0 ? (v1 - v0 + TA - 1) / TA : 1) : 0u;
  const uint64_t amis = (reinterpret_cast<uintptr_t>(A) >> 2) & 3;
  const uint4 *A4 = reinterpret_cast<const uint4 *>(reinterpret_cast<uintptr_t>(A) & ~uintptr_t(15));

  // cursors: set j's first element >= A[ca0]; warps take sets in turn.
  // A CTA's chain of dependent loads (searches, tiles, windows) is long
  // next to its work, so everything it will read is first requested into L2:
  // its S0 run, and each set's range between the guesses for the run's first
  // and last values (with a margin); the chain then waits on L2, not HBM.
  if (ntiles) {
    const uint32_t key = __ldg(A + ca0), klast = __ldg(A + ca1 - 1);
    if (t == NT - 1)
      prefetch_words_l2(A4, (amis + ca0) >> 2, ((amis + ca1) >> 2) + 1, amis ? 1 : 0,
                        (amis + na) >> 2);
    for (int j = 1 + warp; j < k; j += NW) {
      const uint32_t *B = p.sets[j];
      const uint64_t nb = p.lens[j];
      const uint32_t bfirst = __ldg(B), blast = __ldg(B + nb - 1);
      auto guess = [&](uint32_t v) -> uint64_t {
        return (blast <= bfirst || v <= bfirst)
                   ? 0
                   : guess_scale(v - bfirst, blast - bfirst, nb - 1);
      };
      const uint64_t est = guess(key);
      if (lane == 0) {
        const uint64_t bmis = (reinterpret_cast<uintptr_t>(B) >> 2) & 3;
        const uint4 *B4 = reinterpret_cast<const uint4 *>(reinterpret_cast<uintptr_t>(B) & ~uintptr_t(15));
        const uint64_t q0 = (bmis + est) >> 2, q1 = ((bmis + guess(klast)) >> 2) + 1;
        prefetch_words_l2(B4, q0 > 512 ? q0 - 512 : 0, q1 + 512, bmis ? 1 : 0, (bmis + nb) >> 2);
      }
      // at or a little below the first element >= the run's first value (the
      // elements read early lie below every value of the run: no bit of X)
      const uint64_t r = warp_start_below(B, nb, A + ca0, est);
      if (lane == 0) s_b[j] = r;
    }
  }
  __syncthreads();  // buffers zero, cursors visible

  uint32_t cnt = 0;
  uint64_t staged = 0;
  uint32_t *dst = MAT ? p.stage + ca0 : nullptr;
  uint32_t wc = 0;

  for (uint32_t kt = 0; kt < ntiles; ++kt) {
    // ---- 1. the tile of S0 ----
    const uint64_t body0 = v0 + uint64_t(kt) * TA;
    const uint64_t body1 = (body0 + TA < v1) ? body0 + TA : v1;
    const uint64_t e0 = (kt == 0) ? ca0 : body0;
    const uint64_t e1 = (kt + 1 == ntiles) ? ca1 : body1;
    const uint32_t nt = uint32_t(e1 - e0);
    const uint32_t w = __ldg(A + e0), alast = __ldg(A + e1 - 1);
    const uint32_t span = alast - w;
    const bool dense = span < SPAN;
    // X and Y: dense -> bufU / bufV; sparse -> the two halves of bufV
    uint32_t *X = dense ? bufU : bufV;
    uint32_t *Y = dense ? bufV : bufV + Cfg::kPosWords;
    const uint32_t xw = dense ? (span >> 5) + 1 : (nt + 31) / 32;  // bitmap words in use
    {
      const uint4 *ta = A4 + ((amis + body0) >> 2);
      const uint32_t nq = uint32_t((body1 - body0) >> 2);
      uint4 va[UA];
#pragma unroll
      for (int u = 0; u < UA; ++u)
        va[u] = uint32_t(u * NT + t) < nq ? __ldcs(ta + (u * NT + t)) : make_uint4(0, 0, 0, 0);
      const uint32_t nh = uint32_t(body0 - e0), ntl = uint32_t(e1 - body1);
      const bool is_h = uint32_t(t) < nh;
      const bool is_t = uint32_t(t) >= 32 && uint32_t(t) < 32 + ntl;
      uint32_t xe = 0;
      if (is_h) xe = __ldg(A + e0 + t);
      else if (is_t) xe = __ldg(A + body1 + (t - 32));
      if (dense) {
        auto ins = [&](uint32_t x) {
          const uint32_t o = min(x - w, span);
          atomicOr(&X[o >> 5], 1u << (o & 31));
        };
#pragma unroll
        for (int u = 0; u < UA; ++u)
          if (uint32_t(u * NT + t) < nq) {
            ins(va[u].x);
            ins(va[u].y);
            ins(va[u].z);
            ins(va[u].w);
          }
        if (is_h || is_t) ins(xe);
      } else {
#pragma unroll
        for (int u = 0; u < UA; ++u) {
          const uint32_t qq = uint32_t(u * NT + t);
          if (qq < nq) {
            uint32_t *d = bufU + nh + 4 * qq;
            d[0] = va[u].x;
            d[1] = va[u].y;
            d[2] = va[u].z;
            d[3] = va[u].w;
          }
        }
        if (is_h) bufU[t] = xe;
        else if (is_t) bufU[uint32_t(body1 - e0) + (t - 32)] = xe;
        // every position alive
        for (uint32_t i = uint32_t(t); i < xw; i += NT)
          X[i] = (i + 1 < xw || (nt & 31) == 0) ? 0xffffffffu : ((1u << (nt & 31)) - 1u);
      }
    }
    __syncthreads();

    // ---- 2. every other set against the survivors ----
    for (int j = 1; j < k; ++j) {
      const uint32_t *B = p.sets[j];
      const uint64_t nb = p.lens[j];
      const uint64_t bmis = (reinterpret_cast<uintptr_t>(B) >> 2) & 3;
      const uint4 *B4 = reinterpret_cast<const uint4 *>(reinterpret_cast<uintptr_t>(B) & ~uintptr_t(15));
      uint64_t b = s_b[j];
      auto probe = [&](uint32_t x) {
        if (dense) {
          const uint32_t o = min(x - w, span + 1);
          if (__funnelshift_r(X[o >> 5], 0u, o) & 1u) atomicOr(&Y[o >> 5], 1u << (o & 31));
        } else {
          uint32_t lo = 0, len = nt;
          while (len > 0) {
            const uint32_t hh = len >> 1;
            if (bufU[lo + hh] < x) {
              lo += hh + 1;
              len -= hh + 1;
            } else {
              len = hh;
            }
          }
          if (lo < nt && bufU[lo] == x && ((X[lo >> 5] >> (lo & 31)) & 1u))
            atomicOr(&Y[lo >> 5], 1u << (lo & 31));
        }
      };
      for (;;) {
        if (b >= nb) break;
        const uint64_t ab = b + ((4 - ((bmis + b) & 3)) & 3);
        const uint64_t ha = ab < nb ? ab : nb;
        const uint64_t qa = (bmis + ha) >> 2;
        const uint64_t nbq = (bmis + nb) >> 2;
        const uint64_t qe = (qa + UB * NT < nbq) ? qa + UB * NT : nbq;
        const uint64_t bodyend = qe > qa ? (qe << 2) - bmis : ha;
        const uint64_t we = (qe == nbq) ? nb : bodyend;
        const uint4 *wq = B4 + qa;
        const uint32_t nq = uint32_t(qe - qa);
        uint32_t le = 0;
        {
          uint4 vb[UB];
#pragma unroll
          for (int u = 0; u < UB; ++u)
            vb[u] = uint32_t(u * NT + t) < nq ? __ldcs(wq + (u * NT + t)) : make_uint4(0, 0, 0, 0);
          const uint32_t nh = uint32_t(ha - b), ntl = uint32_t(we - bodyend);
          const bool is_h = uint32_t(t) < nh;
          const bool is_t = uint32_t(t) >= 32 && uint32_t(t) < 32 + ntl;
#pragma unroll
          for (int u = 0; u < UB; ++u)
            if (uint32_t(u * NT + t) < nq) {
              probe(vb[u].x);
              probe(vb[u].y);
              probe(vb[u].z);
              probe(vb[u].w);
              le += vb[u].w <= alast ? 4u : 0u;
            }
          if (is_h || is_t) {
            const uint32_t xe = is_h ? __ldg(B + b + t) : __ldg(B + bodyend + (t - 32));
            probe(xe);
            le += xe <= alast ? 1u : 0u;
          }
        }
        le = __reduce_add_sync(0xffffffffu, le);
        if (lane == 0 && le) atomicAdd(&s_le[wc % 3], le);
        __syncthreads();
        const uint32_t used = s_le[wc % 3];
        if (t == 0) s_le[(wc + 2) % 3] = 0;
        ++wc;
        b += used;
        if (b < we) break;
      }
      if (t == 0) s_b[j] = b;
      // X := Y (survivors); the old X, cleared, is the next Y
      __syncthreads();  // probes done (also: window barriers above may be skipped at B's end)
      for (uint32_t i = uint32_t(t); i < xw; i += NT) X[i] = 0;
      uint32_t *tmp = X;
      X = Y;
      Y = tmp;
      __syncthreads();
    }

    // ---- 3. output ----
    {
      const uint32_t per = (xw + NT - 1) / NT;  // thread t owns X words [m0, m1)
      const uint32_t m0 = uint32_t(t) * per;
      const uint32_t m1 = (m0 + per < xw) ? m0 + per : xw;
      uint32_t pc = 0;
      for (uint32_t i = m0; i < m1; ++i) pc += __popc(X[i]);
      if (!MAT) {
        cnt += pc;
      } else {
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
        for (int q = 0; q < NW; ++q) {
          const uint32_t sm = warp_sums[q];
          before += (q < warp) ? sm : 0u;
          tot += sm;
        }
        uint64_t q = staged + before + incl - pc;
        for (uint32_t i = m0; i < m1; ++i) {
          uint32_t m = X[i];
          while (m) {
            const uint32_t bit = i * 32u + uint32_t(__ffs(m) - 1);
            m &= m - 1;
            dst[q++] = dense ? w + bit : bufU[bit];
          }
        }
        staged += tot;
      }
      __syncthreads();  // X read (and the sparse table); warp sums free
      for (uint32_t i = m0; i < m1; ++i) X[i] = 0;
      if (!dense)  // the table's words (a dense tile's bitmap next, maybe)
        for (uint32_t i = uint32_t(t); i < nt; i += NT) bufU[i] = 0;
      __syncthreads();
    }
  }

  // ---- combine (as window.cuh) ----
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
