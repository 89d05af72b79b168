// batch.cuh -- many independent pairs intersected in one persistent launch.
//
// The reference intersects pairs one call at a time (Intersect2,
// setops/src/intersect.rs:40; the benchmark loops over a dataset's pairs,
// benchmark/src/timer/harness.rs:35-97).  On the GPU one launch per small
// pair costs far more than the pair's work, so this kernel takes a whole
// batch: all sets live in one pool, pair p is pool[a_off[p], +a_len[p]) and
// pool[b_off[p], +b_len[p]), and its intersection goes to
// out[out_off[p], +min(a_len, b_len)) with its length in out_lens[p].
// Results equal naive_merge per pair (setops/src/intersect/merge.rs:7-33).
//
// Persistent CTAs pull pairs from an atomic ticket.  Per pair (A = the
// smaller set):
//   - size ratio >= search_ratio: the search path -- one thread per A
//     element, binary search of B in global memory, an ordered block
//     compaction per NT elements;
//   - otherwise the tile path of tile.cuh: A in tiles as a bitmap (dense) or
//     a sorted tile (sparse) in shared memory, B streamed against it; a pair
//     whose A fits one tile probes all of B, longer pairs search each tile's
//     B range.
// Either way the matches are appended in ascending order directly at the
// pair's output offset: no staging, no second pass.
#pragma once

#include "tile.cuh"

namespace setops {

struct BatchArgs {
  const uint32_t *pool;    // all sets (A sides)
  const uint32_t *pool_b;  // B sides when they live elsewhere (NULL: pool)
  const uint64_t *a_off;  // per pair: offset and length of both sets
  const uint64_t *a_len;
  const uint64_t *b_off;
  const uint64_t *b_len;
  uint64_t npairs;
  const uint64_t *out_off;  // per pair: output offset (materialise)
  uint32_t *out;            // output pool (materialise)
  uint64_t *out_lens;       // per pair: intersection length
  uint32_t search_ratio;    // pairs with max/min >= this take the search path; 0 = never
  uint64_t out_cap;         // materialise: checked on the device when non-zero (graph replays)
  LaunchSync *sync;
  int *err;
};

// Search path: for each element of A[0, na), a binary search of B[0, nb) in
// global memory; hits are compacted in A order (ascending).  Returns the
// match count (materialise: same in every thread) or this thread's share
// (count mode).
template <int NT, bool MAT>
__device__ __forceinline__ uint64_t search_run(const uint32_t *A, uint64_t na,
                                               const uint32_t *B, uint64_t nb, uint32_t *dst,
                                               TileShared<NT> &sh) {
  constexpr int NW = NT / 32;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  uint64_t written = 0;
  uint32_t cnt = 0;
  for (uint64_t c0 = 0; c0 < na; c0 += NT) {
    const uint64_t i = c0 + uint64_t(t);
    bool hit = false;
    uint32_t v = 0;
    if (i < na) {
      v = __ldg(A + i);
      uint64_t lo = 0, len = nb;
      while (len > 0) {
        const uint64_t h = len >> 1;
        if (__ldg(B + lo + h) < v) {
          lo += h + 1;
          len -= h + 1;
        } else {
          len = h;
        }
      }
      hit = lo < nb && __ldg(B + lo) == v;
    }
    if (!MAT) {
      cnt += hit;
      continue;
    }
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    if (lane == 0) sh.warp_sums[warp] = uint32_t(__popc(m));
    __syncthreads();
    uint32_t before = 0, tot = 0;
#pragma unroll
    for (int k = 0; k < NW; ++k) {
      const uint32_t s = sh.warp_sums[k];
      before += (k < warp) ? s : 0u;
      tot += s;
    }
    if (hit) dst[written + before + uint32_t(__popc(m & ((1u << lane) - 1u)))] = v;
    written += tot;
    __syncthreads();  // warp sums reused
  }
  return MAT ? written : uint64_t(cnt);
}

template <int NT, int TA, int VW, int MINB, bool MAT>
__global__ void __launch_bounds__(NT, MINB) batch_kernel(const BatchArgs p) {
  using Cfg = TileCfg<NT, TA, VW, MAT>;
  constexpr int NW = NT / 32;
  extern __shared__ __align__(128) uint32_t smem[];
  uint32_t *tab = smem;
  uint32_t *mbits = smem + Cfg::kTabWords;
  __shared__ TileShared<NT> sh;
  __shared__ unsigned long long red[NW];
  __shared__ uint32_t s_pair;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;

  for (int i = t; i < (Cfg::kTabWords + Cfg::kMWords) / 4; i += NT)
    reinterpret_cast<uint4 *>(smem)[i] = make_uint4(0, 0, 0, 0);

  for (;;) {
    if (t == 0) s_pair = atomicAdd(&p.sync->ticket, 1u);
    __syncthreads();
    const uint64_t k = s_pair;
    __syncthreads();  // everyone has read the ticket before it is reused
    if (k >= p.npairs) break;
    uint64_t na = p.a_len[k], nb = p.b_len[k];
    const uint32_t *A = p.pool + p.a_off[k];
    const uint32_t *B = (p.pool_b ? p.pool_b : p.pool) + p.b_off[k];
    if (na > nb) {
      const uint32_t *tp = A; A = B; B = tp;
      const uint64_t tn = na; na = nb; nb = tn;
    }
    if (MAT && p.out_cap && p.out_off[k] + na > p.out_cap) {  // (na: the smaller length)
      if (t == 0) {
        record_error(p.err, DEV_ERR_CAPACITY);
        p.out_lens[k] = 0;
      }
      continue;
    }
    uint32_t *dst = MAT ? p.out + p.out_off[k] : nullptr;
    uint64_t r = 0;
    if (na > 0) {
      if (p.search_ratio && nb / na >= p.search_ratio)
        r = search_run<NT, MAT>(A, na, B, nb, dst, sh);
      else
        r = tile_run<NT, TA, VW, MAT>(A, 0, na, B, nb, na > uint64_t(TA), dst, tab, mbits, sh);
    }
    if (!MAT) {
      uint64_t v = r;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[warp] = v;
      __syncthreads();
      if (t == 0) {
        uint64_t s = 0;
        for (int q = 0; q < NW; ++q) s += red[q];
        p.out_lens[k] = s;
      }
    } else if (t == 0) {
      p.out_lens[k] = r;
    }
  }
  // the last CTA out resets the ticket for the next launch
  if (t == 0) {
    __threadfence();
    const uint32_t prev = atomicAdd(&p.sync->done, 1u);
    if (prev == gridDim.x - 1) {
      p.sync->ticket = 0;
      p.sync->done = 0;
      __threadfence();
    }
  }
}

// ---- BSR pairs ---------------------------------------------------------------
// The same batch for sets in the reference's BSR form (BsrVec,
// setops/src/bsr.rs:20-30): word i of a set is (bases[i], states[i]), bases
// strictly increasing, states non-zero.  Pair p's result is what
// branchless_merge_bsr (setops/src/intersect/merge.rs:62-87) emits: for every
// base in both sets, (base, state_a & state_b) when non-zero, in base order.
// Count mode gives the Counter visitor's popcount sum
// (setops/src/visitor.rs:399-403).
struct BatchBsrArgs {
  const uint32_t *bases;   // all sets: bases and states, same offsets
  const uint32_t *states;
  const uint64_t *a_off, *a_len, *b_off, *b_len;  // per pair, in words
  uint64_t npairs;
  const uint64_t *out_off;  // per pair: output word offset (materialise)
  uint32_t *out_bases, *out_states;
  uint64_t *out_lens;       // per pair: result words (materialise) or popcount sum (count)
  LaunchSync *sync;
  int *err;
};

// Persistent CTAs pull pairs from a ticket.  Per pair (A = the set with fewer
// words) the longer set is staged in shared memory when it fits CAPW words;
// one thread per A word binary-searches its base there (or in global memory),
// ANDs the states, and the non-zero words are compacted in A order (a warp
// ballot and per-warp sums), which is base order.
template <int NT, int CAPW, bool MAT>
__global__ void __launch_bounds__(NT) batch_bsr_kernel(const BatchBsrArgs p) {
  constexpr int NW = NT / 32;
  __shared__ uint32_t sb[CAPW], ss[CAPW];
  __shared__ uint32_t warp_sums[NW];
  __shared__ unsigned long long red[NW];
  __shared__ uint32_t s_pair;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  for (;;) {
    if (t == 0) s_pair = atomicAdd(&p.sync->ticket, 1u);
    __syncthreads();
    const uint64_t k = s_pair;
    __syncthreads();  // everyone has read the ticket before it is reused
    if (k >= p.npairs) break;
    uint64_t na = p.a_len[k], nb = p.b_len[k];
    uint64_t ao = p.a_off[k], bo = p.b_off[k];
    if (na > nb) {
      const uint64_t tn = na; na = nb; nb = tn;
      const uint64_t to = ao; ao = bo; bo = to;
    }
    const uint32_t *Ab = p.bases + ao, *As = p.states + ao;
    const uint32_t *Bb = p.bases + bo, *Bs = p.states + bo;
    const bool staged = nb <= uint64_t(CAPW);
    if (staged) {
      for (uint32_t i = uint32_t(t); i < uint32_t(nb); i += NT) {
        sb[i] = __ldg(Bb + i);
        ss[i] = __ldg(Bs + i);
      }
    }
    __syncthreads();
    uint64_t written = 0;  // materialise: words written for this pair
    uint64_t pc = 0;       // count: this thread's popcount sum
    for (uint64_t c0 = 0; c0 < na; c0 += NT) {
      const uint64_t i = c0 + uint64_t(t);
      uint32_t base = 0, st = 0;
      if (i < na) {
        base = __ldg(Ab + i);
        uint64_t lo = 0, len = nb;
        if (staged) {
          while (len > 0) {
            const uint64_t h = len >> 1;
            if (sb[lo + h] < base) { lo += h + 1; len -= h + 1; } else { len = h; }
          }
          if (lo < nb && sb[lo] == base) st = __ldg(As + i) & ss[lo];
        } else {
          while (len > 0) {
            const uint64_t h = len >> 1;
            if (__ldg(Bb + lo + h) < base) { lo += h + 1; len -= h + 1; } else { len = h; }
          }
          if (lo < nb && __ldg(Bb + lo) == base) st = __ldg(As + i) & __ldg(Bs + lo);
        }
      }
      if (!MAT) {
        pc += uint64_t(__popc(st));
        continue;
      }
      const unsigned m = __ballot_sync(0xffffffffu, st != 0);
      if (lane == 0) warp_sums[warp] = uint32_t(__popc(m));
      __syncthreads();
      uint32_t before = 0, tot = 0;
#pragma unroll
      for (int q = 0; q < NW; ++q) {
        const uint32_t sm = warp_sums[q];
        before += (q < warp) ? sm : 0u;
        tot += sm;
      }
      if (st) {
        const uint64_t o = p.out_off[k] + written + before + uint32_t(__popc(m & ((1u << lane) - 1u)));
        p.out_bases[o] = base;
        p.out_states[o] = st;
      }
      written += tot;
      __syncthreads();  // warp sums reused
    }
    if (!MAT) {
      uint64_t v = pc;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[warp] = v;
      __syncthreads();
      if (t == 0) {
        uint64_t sm = 0;
        for (int q = 0; q < NW; ++q) sm += red[q];
        p.out_lens[k] = sm;
      }
    } else if (t == 0) {
      p.out_lens[k] = written;
    }
    __syncthreads();  // staged B and red reused by the next pair
  }
  if (t == 0) {
    __threadfence();
    const uint32_t prev = atomicAdd(&p.sync->done, 1u);
    if (prev == gridDim.x - 1) {
      p.sync->ticket = 0;
      p.sync->done = 0;
      __threadfence();
    }
  }
}

// out_off[p] = sum of min(a_len, b_len) over pairs before p (one CTA).
template <int NT>
__global__ void __launch_bounds__(NT) batch_offsets_kernel(const uint64_t *a_len,
                                                           const uint64_t *b_len,
                                                           uint64_t npairs, uint64_t *out_off,
                                                           uint64_t *total) {
  constexpr int NW = NT / 32;
  __shared__ unsigned long long ws[NW];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  unsigned long long base = 0;
  for (uint64_t c0 = 0; c0 < npairs; c0 += NT) {
    const uint64_t i = c0 + uint64_t(t);
    const unsigned long long v = i < npairs ? (a_len[i] < b_len[i] ? a_len[i] : b_len[i]) : 0ull;
    unsigned long long incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) ws[warp] = incl;
    __syncthreads();
    unsigned long long before = 0, tot = 0;
#pragma unroll
    for (int k = 0; k < NW; ++k) {
      before += (k < warp) ? ws[k] : 0ull;
      tot += ws[k];
    }
    if (i < npairs) out_off[i] = base + before + incl - v;
    base += tot;
    __syncthreads();
  }
  if (t == 0) *total = base;
}

}  // namespace setops
