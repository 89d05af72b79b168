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
  // Long pairs split into units (batch_prefix_*); NULL: one unit per pair.
  const uint64_t *ustart;     // per pair: first unit; [npairs] = number of units
  const uint32_t *unit_pair;  // per unit: its pair
  uint64_t *ucount;           // per unit: its matches
  uint32_t *pcount;           // per pair: units finished (zeroed by batch_prefix_global)
  LaunchSync *sync;
  int *err;
};

// Units of at most this many elements of a pair's smaller set: a longer pair
// is intersected by several CTAs at once.
constexpr uint64_t kBatchUnit = 16384;

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

  const uint64_t nunits = p.ustart ? p.ustart[p.npairs] : p.npairs;
  __shared__ uint32_t s_last;
  for (;;) {
    if (t == 0) s_pair = atomicAdd(&p.sync->ticket, 1u);
    __syncthreads();
    const uint64_t un = s_pair;
    __syncthreads();  // everyone has read the ticket before it is reused
    if (un >= nunits) break;
    const uint64_t k = p.ustart ? p.unit_pair[un] : un;  // the pair
    const uint64_t ju = p.ustart ? un - p.ustart[k] : 0;  // unit of the pair
    const uint64_t nu = p.ustart ? p.ustart[k + 1] - p.ustart[k] : 1;
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
    // pair k, or unit ju of its nu units: A[s0, s1) against all of B, the
    // matches at the same offset in the pair's output (a unit's own region)
    const uint64_t s0 = ju * na / nu, s1 = (ju + 1) * na / nu;
    uint32_t *dst = MAT ? p.out + p.out_off[k] + s0 : nullptr;
    uint64_t r = 0;
    if (s1 > s0) {
      if (p.search_ratio && nb / na >= p.search_ratio)
        r = search_run<NT, MAT>(A + s0, s1 - s0, B, nb, dst, sh);
      else
        r = tile_run<NT, TA, VW, MAT>(A, s0, s1, B, nb, nu > 1 || na > uint64_t(TA), dst, tab,
                                      mbits, sh);
    }
    if (!MAT) {  // per-thread shares -> the total, in every thread
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
      if (lane == 0) red[warp] = r;
      __syncthreads();
      r = 0;
      for (int q = 0; q < NW; ++q) r += red[q];
    }
    if (nu == 1) {
      if (t == 0) p.out_lens[k] = r;
      continue;  // (red is next written after the ticket's barriers)
    }
    // the last unit of the pair to finish packs the units' matches left, in
    // unit order, and writes the pair's length
    if (MAT) {
      __threadfence();  // this thread's staged matches, before the count below
      __syncthreads();
    }
    if (t == 0) {
      p.ucount[un] = r;
      __threadfence();
      s_last = atomicAdd(&p.pcount[k], 1u) == uint32_t(nu - 1) ? 1u : 0u;
    }
    __syncthreads();
    if (s_last) {
      __threadfence();
      const uint64_t u0 = p.ustart[k];
      uint64_t wpos = 0;  // packed length so far
      for (uint64_t v = 0; v < nu; ++v) {
        const uint64_t c = __ldcg(p.ucount + u0 + v);  // other CTAs' writes: not via L1
        if (MAT) {
          // move this unit's matches left, block by block: every read of a
          // block before any write of it (the target is never right of the
          // source, so later blocks are not overwritten)
          const uint64_t src = v * na / nu;
          uint32_t *o = p.out + p.out_off[k];
          if (src != wpos) {
            for (uint64_t b0 = 0; b0 < c; b0 += NT) {
              const bool has = b0 + uint64_t(t) < c;
              const uint32_t x = has ? __ldcg(o + src + b0 + t) : 0u;
              __syncthreads();
              if (has) o[wpos + b0 + t] = x;
              __syncthreads();
            }
          }
        }
        wpos += c;
      }
      if (t == 0) p.out_lens[k] = wpos;
    }
    __syncthreads();  // s_last reused
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

// ---- per-pair prefixes: output offsets and the unit map ----------------------
// Two launches over chunks of NT pairs, one pair per thread (G = ceil(npairs /
// NT) CTAs each): batch_prefix_local scans within a chunk and writes the chunk
// sums; batch_prefix_global adds the sums of the chunks before it (each CTA
// reads all G sums) and finishes the arrays.
//   offsets (out_off != NULL): out_off[p] = sum of min(a_len, b_len) over the
//     pairs before p, *out_total = the sum over all pairs;
//   units (ustart != NULL): pair p gets nu = ceil(min / kBatchUnit) units (1
//     for min <= kBatchUnit), ustart[p] = units before p, ustart[npairs] = all
//     units, unit_pair[u] = the pair of unit u, pcount zeroed; when the units
//     exceed unit_cap (the room in unit_pair) every pair gets one unit.

__device__ __forceinline__ uint64_t batch_units_of(uint64_t mn) {
  return mn > kBatchUnit ? (mn + kBatchUnit - 1) / kBatchUnit : 1;
}

// Exclusive 64-bit scan over the block; *total = the block's sum.
template <int NT>
__device__ __forceinline__ unsigned long long block_scan_u64(unsigned long long v,
                                                             unsigned long long *ws,
                                                             unsigned long long *total) {
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[warp] = x;
  __syncthreads();
  unsigned long long before = 0, tot = 0;
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    const unsigned long long s = ws[w];
    before += (w < warp) ? s : 0ull;
    tot += s;
  }
  __syncthreads();  // ws reused by the next scan
  *total = tot;
  return before + x - v;
}

template <int NT>
__global__ void __launch_bounds__(NT) batch_prefix_local(const uint64_t *a_len,
                                                         const uint64_t *b_len, uint64_t npairs,
                                                         uint64_t *out_off, uint64_t *osum,
                                                         uint64_t *ustart, uint64_t *csum) {
  __shared__ unsigned long long ws[NT / 32];
  const uint64_t i = uint64_t(blockIdx.x) * NT + threadIdx.x;
  const bool in = i < npairs;
  const uint64_t mn = in ? (a_len[i] < b_len[i] ? a_len[i] : b_len[i]) : 0;
  unsigned long long tot;
  if (out_off) {
    const unsigned long long x = block_scan_u64<NT>(mn, ws, &tot);
    if (in) out_off[i] = x;
    if (threadIdx.x == 0) osum[blockIdx.x] = tot;
  }
  if (ustart) {
    const unsigned long long x = block_scan_u64<NT>(in ? batch_units_of(mn) : 0ull, ws, &tot);
    if (in) ustart[i] = x;
    if (threadIdx.x == 0) csum[blockIdx.x] = tot;
  }
}

template <int NT>
__global__ void __launch_bounds__(NT) batch_prefix_global(
    const uint64_t *a_len, const uint64_t *b_len, uint64_t npairs, uint64_t *out_off,
    const uint64_t *osum, uint64_t *out_total, uint64_t *ustart, const uint64_t *csum,
    uint32_t *unit_pair, uint32_t *pcount, uint64_t unit_cap) {
  constexpr int NW = NT / 32;
  __shared__ unsigned long long ws[4][NW];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const uint32_t c = blockIdx.x, G = gridDim.x;
  // [0] offsets before this chunk, [1] all offsets, [2] units before, [3] all units
  unsigned long long s[4] = {0, 0, 0, 0};
  for (uint32_t j = uint32_t(t); j < G; j += NT) {
    const unsigned long long o = out_off ? osum[j] : 0ull, u = ustart ? csum[j] : 0ull;
    s[0] += j < c ? o : 0ull;
    s[1] += o;
    s[2] += j < c ? u : 0ull;
    s[3] += u;
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s[q] += __shfl_xor_sync(0xffffffffu, s[q], o);
    if (lane == 0) ws[q][warp] = s[q];
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    s[q] = 0;
    for (int w = 0; w < NW; ++w) s[q] += ws[q][w];
  }
  const uint64_t i = uint64_t(c) * NT + uint64_t(t);
  const bool in = i < npairs;
  const bool last = c == G - 1 && t == 0;
  if (out_off) {
    if (in) out_off[i] += s[0];
    if (last) *out_total = s[1];
  }
  if (ustart) {
    const bool split = s[3] <= unit_cap;
    if (in) {
      pcount[i] = 0;
      if (split) {
        const uint64_t u0 = s[2] + ustart[i];
        const uint64_t nv = batch_units_of(a_len[i] < b_len[i] ? a_len[i] : b_len[i]);
        ustart[i] = u0;
        for (uint64_t u = 0; u < nv; ++u) unit_pair[u0 + u] = uint32_t(i);
      } else {
        ustart[i] = i;
        unit_pair[i] = uint32_t(i);
      }
    }
    if (last) ustart[npairs] = split ? s[3] : npairs;
  }
}

// ---- host side of the prefixes -------------------------------------------------

constexpr int kPrefixNT = 1024;  // pairs per chunk of batch_prefix_*

inline size_t a16(size_t b) { return (b + 15) & ~size_t(15); }

// Scratch of the per-pair prefixes: the chunk sums (2 x G words) and, with
// unit_cap > 0, the unit map: ustart (npairs + 1), ucount and unit_pair
// (unit_cap each), pcount (npairs); each part 16-byte aligned.
inline size_t prefix_bytes(uint64_t npairs, uint64_t unit_cap) {
  const uint64_t G = (npairs + kPrefixNT - 1) / kPrefixNT;
  size_t b = 2 * a16(G * 8);
  if (unit_cap)
    b += a16((npairs + 1) * 8) + a16(unit_cap * 8) + a16(unit_cap * 4) + a16(npairs * 4);
  return b;
}

// Room for the unit map when the pairs' smaller lengths sum to at most
// `words`: a split pair of length m has at most m / kBatchUnit + 1 units.
// 0 (no splitting) when a pair index does not fit unit_pair's 32 bits.
inline uint64_t unit_room(uint64_t npairs, uint64_t words) {
  return npairs > 0xFFFFFFFFull ? 0 : npairs + words / kBatchUnit + 1;
}

// Launches the prefixes of a batch on st (two launches, batch_prefix_*):
// the output offsets when out_off is given (their total into *out_total) and
// the unit map, carved from `scratch` into `a`, when unit_cap > 0 (room for
// max(unit_cap, npairs) units).
inline void launch_prefix(const uint64_t *a_len, const uint64_t *b_len, uint64_t npairs, void *scratch,
                   uint64_t *out_off, uint64_t *out_total, uint64_t unit_cap, BatchArgs *a,
                   cudaStream_t st) {
  const uint64_t G = (npairs + kPrefixNT - 1) / kPrefixNT;
  char *c = static_cast<char *>(scratch);
  uint64_t *osum = reinterpret_cast<uint64_t *>(c);
  c += a16(G * 8);
  uint64_t *csum = reinterpret_cast<uint64_t *>(c);
  c += a16(G * 8);
  uint64_t *ustart = nullptr;
  uint32_t *unit_pair = nullptr, *pcount = nullptr;
  if (unit_cap) {
    unit_cap = std::max<uint64_t>(unit_cap, npairs);
    ustart = reinterpret_cast<uint64_t *>(c);
    c += a16((npairs + 1) * 8);
    a->ucount = reinterpret_cast<uint64_t *>(c);
    c += a16(unit_cap * 8);
    unit_pair = reinterpret_cast<uint32_t *>(c);
    c += a16(unit_cap * 4);
    pcount = reinterpret_cast<uint32_t *>(c);
    a->ustart = ustart;
    a->unit_pair = unit_pair;
    a->pcount = pcount;
  }
  batch_prefix_local<kPrefixNT><<<unsigned(G), kPrefixNT, 0, st>>>(a_len, b_len, npairs, out_off,
                                                                   osum, ustart, csum);
  batch_prefix_global<kPrefixNT><<<unsigned(G), kPrefixNT, 0, st>>>(
      a_len, b_len, npairs, out_off, osum, out_total, ustart, csum, unit_pair, pcount, unit_cap);
}

}  // namespace setops
