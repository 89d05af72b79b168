// adaptive.cuh -- k-set intersection by the small_adaptive scheme
// (setops/src/intersect/adaptive.rs:107-148; Demaine, Lopez-Ortiz and Munro,
// ALENEX 2001): every element of the smallest set is looked up in each other
// set in turn, smallest first, and dropped at the first set that lacks it.
// Same result as svs_generic (setops/src/intersect/svs.rs:50-73): the common
// elements, ascending.
//
// The reference gallops from each set's last position because it walks the
// probe set in order on one core.  Here all elements are looked up at once:
//
//   * the probe set is cut into tiles of NT*IT elements, handed out in order
//     by a ticket (so every earlier tile is running or done);
//   * for each other set, one warp brackets the tile's value range in it
//     (lower bounds of the tile's first and last values, one round of probes
//     around an index guess), and every element then binary-searches only
//     its set's bracket -- the galloping step's job, done once per tile;
//   * an element that a set lacks skips the later sets, so the larger sets
//     are touched only where the survivors lie: a query whose smallest list
//     is short reads a few sectors of its long lists, not the lists;
//   * the survivors of a tile are placed by a block scan and a warp-parallel
//     decoupled look-back over the tiles' counts (tile order = output
//     order), and written in ascending order.
#pragma once

#include "kset.cuh"

namespace setops {

struct AdaptiveArgs {
  const uint32_t *sets[kKsetMax];  // sets[0] the probe set (smallest), then ascending length
  uint64_t lens[kKsetMax];
  int k;
  uint32_t *out;      // NULL: count only
  uint64_t out_cap;
  uint64_t *out_len;  // the result's length (device word)
  uint64_t *status;   // look-back words, >= number of tiles
  LaunchSync *sync;   // ticket, finished CTAs, count accumulator
  int *err;
  uint32_t epoch;
};

template <int NT, int IT>
struct AdaptiveCfg {
  static_assert(NT % 32 == 0 && NT >= 64 && NT <= 1024, "whole warps");
  static constexpr int kTile = NT * IT;  // probe-set elements per tile
};

// First index in [lo, hi) of S with S[i] >= x (hi if none).
__device__ __forceinline__ uint64_t lower_bound_in(const uint32_t *__restrict__ S, uint64_t lo,
                                                   uint64_t hi, uint32_t x) {
  uint64_t n = hi - lo;
  while (n > 0) {
    const uint64_t h = n >> 1;
    if (__ldg(S + lo + h) < x) {
      lo += h + 1;
      n -= h + 1;
    } else {
      n = h;
    }
  }
  return lo;
}

template <int NT, int IT>
__global__ void __launch_bounds__(NT) adaptive_kernel(const AdaptiveArgs p) {
  constexpr int NW = NT / 32;
  constexpr uint32_t TILE = AdaptiveCfg<NT, IT>::kTile;
  __shared__ uint64_t s_lo[kKsetMax], s_hi[kKsetMax];
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_warp[NW];
  __shared__ unsigned long long s_base;

  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const uint32_t *S0 = p.sets[0];
  const uint64_t n0 = p.lens[0];
  const uint32_t ntiles = uint32_t((n0 + TILE - 1) / TILE);
  const bool mat = p.out != nullptr;
  uint64_t my_count = 0;

  for (;;) {
    if (t == 0) s_tile = atomicAdd(&p.sync->ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= ntiles) break;
    const uint64_t e0 = uint64_t(tile) * TILE;
    const uint64_t e1 = (e0 + TILE < n0) ? e0 + TILE : n0;

    // brackets of the tile's values [S0[e0], S0[e1-1]] in each other set
    for (int j = 1 + warp; j < p.k; j += NW) {
      const uint32_t *Sj = p.sets[j];
      const uint64_t nj = p.lens[j];
      uint64_t lo = 0, hi = 0;
      if (nj > 0) {
        uint32_t key;
        const uint64_t est0 = guess_scale(e0, n0, nj);
        const uint64_t est1 = guess_scale(e1, n0, nj);
        lo = warp_lower_bound_guess(Sj, nj, S0 + e0, est0 < nj ? est0 : nj - 1, &key);
        hi = warp_lower_bound_guess(Sj, nj, S0 + e1 - 1, est1 < nj ? est1 : nj - 1, &key);
        hi = (hi < nj) ? hi + 1 : nj;  // include an element equal to the last value
      }
      if (lane == 0) {
        s_lo[j] = lo;
        s_hi[j] = hi;
      }
    }
    __syncthreads();

    // thread t looks up elements e0 + t*IT .. + IT-1 (its own, in order)
    uint32_t x[IT];
    uint32_t alive = 0;
#pragma unroll
    for (int i = 0; i < IT; ++i) {
      const uint64_t idx = e0 + uint64_t(t) * IT + i;
      x[i] = 0;
      if (idx < e1) {
        x[i] = __ldg(S0 + idx);
        alive |= 1u << i;
      }
    }
    for (int j = 1; j < p.k && alive; ++j) {
      const uint32_t *Sj = p.sets[j];
      const uint64_t lo = s_lo[j], hi = s_hi[j];
#pragma unroll
      for (int i = 0; i < IT; ++i) {
        if (alive & (1u << i)) {
          const uint64_t q = lower_bound_in(Sj, lo, hi, x[i]);
          if (q >= hi || __ldg(Sj + q) != x[i]) alive &= ~(1u << i);
        }
      }
    }

    const uint32_t c = uint32_t(__popc(alive));
    if (!mat) {
      my_count += c;
      __syncthreads();  // s_lo / s_hi / s_tile read before the next tile
      continue;
    }
    // placement: block scan of the threads' counts, then the tile's base
    uint32_t total;
    const uint32_t ex = block_exclusive_scan<NT>(c, s_warp, &total);
    if (warp == 0) {
      const uint64_t base = lookback_exclusive_warp(p.status, tile, total, p.epoch, p.err);
      if (lane == 0) s_base = base;
    }
    __syncthreads();
    const uint64_t base = s_base;
    if (base != UINT64_MAX) {
      if (base + total > p.out_cap) {
        if (t == 0) record_error(p.err, DEV_ERR_CAPACITY);
      } else {
        uint64_t o = base + ex;
#pragma unroll
        for (int i = 0; i < IT; ++i)
          if (alive & (1u << i)) p.out[o++] = x[i];
        if (tile == ntiles - 1 && t == 0) *p.out_len = base + total;
      }
    }
    __syncthreads();  // s_base / s_lo / s_hi / s_tile read before the next tile
  }

  // count mode: per-CTA sums; the last CTA to finish writes the total and
  // resets the coordination words (materialise: the last tile wrote it)
  __shared__ unsigned long long s_red[NW];
  if (!mat) {
    unsigned long long v = my_count;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) s_red[warp] = v;
    __syncthreads();
    if (t == 0) {
      unsigned long long sm = 0;
      for (int q = 0; q < NW; ++q) sm += s_red[q];
      if (sm) atomicAdd(&p.sync->acc, sm);
    }
  }
  if (t == 0) {
    __threadfence();
    const uint32_t prev = atomicAdd(&p.sync->done, 1u);
    if (prev == gridDim.x - 1) {
      if (!mat) *p.out_len = atomicExch(&p.sync->acc, 0ull);
      else if (ntiles == 0) *p.out_len = 0;
      p.sync->ticket = 0;
      p.sync->done = 0;
      p.sync->acc = 0;
      __threadfence();
    }
  }
}

}  // namespace setops
