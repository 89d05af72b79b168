// kernels.cu -- instantiation table of the intersection kernels, plus the
// small utility kernels (sortedness check, device BSR encode / decode).
#include "kernels.h"

#include "gallop.cuh"
#include "merge.cuh"
#include "tile.cuh"
#include "window.cuh"
#include "awindow.cuh"
#include "bcast.cuh"
#include "wwindow.cuh"
#include "kset.cuh"

namespace setops {

namespace {

template <int NW, int C, int NSA, int NSB, int VW, bool BSR, bool MAT>
KernelInfo mk_merge(const char *name) {
  using Cfg = MergeCfg<NW, C, NSA, NSB, VW, BSR, MAT>;
  return KernelInfo{reinterpret_cast<const void *>(
                        &merge_kernel<NW, C, NSA, NSB, VW, BSR, MAT>),
                    Cfg::kThreads, Cfg::kSmemBytes, C, name};
}

template <int NT, int GS, int ITEMS, int NSAMP, bool BSR, bool MAT>
KernelInfo mk_gallop(const char *name) {
  // materialise: cooperative (its placement waits on the last CTA's scan)
  return KernelInfo{reinterpret_cast<const void *>(
                        &gallop_kernel<NT, GS, ITEMS, NSAMP, BSR, MAT>),
                    NT, 0, GallopCfg<NT, GS, ITEMS, NSAMP>::kTile, name, MAT};
}

template <int NT, int UA, int UB, int VW, int MINB, bool MAT, bool COARSE = false>
KernelInfo mk_window(const char *name) {
  using Cfg = WindowCfg<NT, UA, UB, VW, MAT, COARSE>;
  return KernelInfo{
      reinterpret_cast<const void *>(&window_kernel<NT, UA, UB, VW, MINB, MAT, COARSE>), NT,
      Cfg::kSmemBytes, Cfg::kTile, name, MAT};
}

template <int NT, int UA, int UB, int VW, int MINB, bool MAT>
KernelInfo mk_awindow(const char *name) {
  using Cfg = AWindowCfg<NT, UA, UB, VW, MAT>;
  return KernelInfo{reinterpret_cast<const void *>(&awindow_kernel<NT, UA, UB, VW, MINB, MAT>),
                    NT, Cfg::kSmemBytes, Cfg::kTile, name, MAT};
}

template <int NT, int MINB, int KD, bool MAT>
KernelInfo mk_bcast(const char *name) {
  // materialise: cooperative (one grid barrier before the runs are placed)
  return KernelInfo{reinterpret_cast<const void *>(&bcast_bsr_kernel<NT, MINB, KD, MAT>), NT, 0,
                    BcastCfg<NT>::kTile, name, MAT};
}

template <int NT, int UA, int UB, int VWW, int MINB, bool MAT>
KernelInfo mk_wwindow(const char *name) {
  using Cfg = WWindowCfg<NT, UA, UB, VWW, MAT>;
  return KernelInfo{reinterpret_cast<const void *>(&wwindow_kernel<NT, UA, UB, VWW, MINB, MAT>),
                    NT, Cfg::kSmemBytes, Cfg::kTile, name, MAT};
}

template <int NT, int TA, int VW, int MINB, bool MAT>
KernelInfo mk_tile(const char *name) {
  using Cfg = TileCfg<NT, TA, VW, MAT>;
  return KernelInfo{reinterpret_cast<const void *>(&tile_kernel<NT, TA, VW, MINB, MAT>), NT,
                    Cfg::kSmemBytes, TA, name, MAT};
}

// [variant][count, materialise]
#define MERGE_ROW(NW, C, NSA, NSB, VW, BSR)                                   \
  {mk_merge<NW, C, NSA, NSB, VW, BSR, false>(                                 \
       "merge_w" #NW "_c" #C "_s" #NSA "x" #NSB "_t" #VW),                    \
   mk_merge<NW, C, NSA, NSB, VW, BSR, true>(                                  \
       "merge_w" #NW "_c" #C "_s" #NSA "x" #NSB "_t" #VW)}
#define GALLOP_ROW(NT, GS, IT, NS, BSR)                                         \
  {mk_gallop<NT, GS, IT, NS, BSR, false>("gallop_" #NT "_g" #GS "_i" #IT "_s" #NS), \
   mk_gallop<NT, GS, IT, NS, BSR, true>("gallop_" #NT "_g" #GS "_i" #IT "_s" #NS)}

// NW warps; C-element chunks in NSA / NSB slots for A / B; T buffers of VW
// words (bitmaps of 32*VW values, or VW BSR states)
const KernelInfo kMergeU32[][2] = {
    MERGE_ROW(8, 2048, 2, 3, 2048, false),   // 0: 64 KB, 3 CTAs/SM
    MERGE_ROW(8, 2048, 3, 3, 2048, false),   // 1: 72 KB, 3 CTAs/SM
    MERGE_ROW(4, 2048, 2, 3, 2048, false),   // 2: 4 warps
    MERGE_ROW(8, 2048, 3, 4, 2048, false),   // 3: 80 KB, 2 CTAs/SM
    MERGE_ROW(4, 1024, 2, 4, 1024, false),   // 4: 36 KB, 5 CTAs/SM
    MERGE_ROW(8, 1024, 3, 4, 2048, false),   // 5: 52 KB, 4 CTAs/SM
};
const KernelInfo kMergeBsr[][2] = {
    MERGE_ROW(8, 1024, 2, 3, 2048, true),  // 0: 56 KB
    MERGE_ROW(8, 2048, 2, 2, 4096, true),  // 1: 96 KB
    MERGE_ROW(8, 1024, 2, 2, 4096, true),  // 2: 64 KB
    {mk_bcast<128, 8, 3, false>("bcast_bsr_128_k3"), mk_bcast<128, 8, 3, true>("bcast_bsr_128_k3")},
    // 3: block broadcast, a warp per run of 32-word blocks (bcast.cuh)
};
// Window kernels: NT threads; UA / UB 16-byte loads per thread for an A tile
// (4*UA*NT elements) / a B window (4*UB*NT); T of VW words (dense tiles span
// < 32*VW values); MINB CTAs per SM.  Tile kernel: A tiles of TA elements,
// B ranges searched per tile.
#define WINDOW_ROW(NT, UA, UB, VW, MINB)                                                     \
  {mk_window<NT, UA, UB, VW, MINB, false>("window_" #NT "_a" #UA "_b" #UB "_t" #VW "_m" #MINB), \
   mk_window<NT, UA, UB, VW, MINB, true>("window_" #NT "_a" #UA "_b" #UB "_t" #VW "_m" #MINB)}
#define WWINDOW_ROW(NT, UA, UB, VWW, MINB)                                                       \
  {mk_wwindow<NT, UA, UB, VWW, MINB, false>("wwindow_" #NT "_a" #UA "_b" #UB "_t" #VWW "_m" #MINB), \
   mk_wwindow<NT, UA, UB, VWW, MINB, true>("wwindow_" #NT "_a" #UA "_b" #UB "_t" #VWW "_m" #MINB)}
#define TILE_ROW(NT, TA, VW, MINB)                                             \
  {mk_tile<NT, TA, VW, MINB, false>("bitmap_" #NT "_a" #TA "_t" #VW "_b" #MINB), \
   mk_tile<NT, TA, VW, MINB, true>("bitmap_" #NT "_a" #TA "_t" #VW "_b" #MINB)}
const KernelInfo kBitmapU32[][2] = {
    WINDOW_ROW(128, 4, 5, 2048, 8),  // 0: 2048-element tiles, 8-9 CTAs/SM
    WINDOW_ROW(256, 4, 6, 4096, 4),  // 1: 4096-element tiles, 4 CTAs/SM
    WINDOW_ROW(256, 4, 5, 4096, 5),  // 2: 5 CTAs/SM
    WINDOW_ROW(256, 4, 4, 4096, 6),  // 3: 6 CTAs/SM
    TILE_ROW(256, 4096, 4096, 8),    // 4: tile kernel (a B search per tile)
    WWINDOW_ROW(128, 4, 5, 512, 8),  // 5: warps on their own, 512-element tiles, 8 CTAs/SM
    WWINDOW_ROW(1024, 4, 5, 512, 1), // 6: the same, one CTA of 32 warps per SM
    {mk_window<128, 4, 5, 2048, 8, false, true>("window_128_a4_b5_t2048_m8_coarse"),
     mk_window<128, 4, 5, 2048, 8, true, true>("window_128_a4_b5_t2048_m8_coarse")},
    // 7: variant 0 with coarse bitmaps for sparse tiles (size ratios 2-31)
    {mk_window<128, 4, 5, 2048, 7, false>("window_128_a4_b5_t2048_m7"),
     mk_awindow<128, 4, 5, 2048, 7, true>("awindow_128_a4_b5_t2048_m7")},
    // 8: materialise with both inputs copied ahead into shared memory
    // (cp.async; 0.045 vs 0.048 ms on the 2^24 pair); count mode keeps
    // variant 0's kernel, which is faster there (0.035 vs 0.037 ms).  Both
    // with a launch bound of 7 CTAs per SM (the shared memory still allows
    // 8): the code generated without the 64-register cap ran 0.0434 against
    // 0.0443-0.0446 ms materialising and 0.0339 against 0.0350 counting
};

// GS lanes per element (1 = thread per element with IT interleaved
// searches); NS = shared-memory sample of the CTA's bracket (0 = none)
const KernelInfo kGallopU32[][2] = {
    GALLOP_ROW(256, 1, 4, 2048, false),  // 0: sampled, thread per element
    GALLOP_ROW(256, 16, 1, 0, false),    // 1: 17-ary over the whole set
    GALLOP_ROW(256, 32, 1, 0, false),    // 2: warp per element, 33-ary
    GALLOP_ROW(256, 8, 1, 0, false),     // 3: 9-ary, 4 elements per warp
    GALLOP_ROW(256, 1, 8, 2048, false),  // 4: sampled, 8 interleaved
    GALLOP_ROW(256, 32, 1, 2048, false), // 5: sampled, warp per element
    GALLOP_ROW(256, 8, 1, 2048, false),  // 6: sampled, 9-ary
    GALLOP_ROW(256, 1, 1, 2048, false),  // 7: sampled, thread per element, 256-element tiles
    GALLOP_ROW(256, 1, 2, 2048, false),  // 8: the same, 512-element tiles (a launch of
                                         //    2^18 elements: 512 CTAs, not 256)
};
const KernelInfo kGallopBsr[][2] = {
    GALLOP_ROW(256, 1, 4, 2048, true),
    GALLOP_ROW(256, 16, 1, 0, true),
    GALLOP_ROW(256, 32, 1, 0, true),
};

template <class T, size_t N>
constexpr int count_of(const T (&)[N]) {
  return int(N);
}

}  // namespace

// NT threads, A tiles of 4*4*NT = 2048 elements, windows of 4*5*NT, bitmaps
// of 4096 words (dense tiles span < 131,072 values), 6 CTAs/SM
const KernelInfo &kset_kernel(bool mat) {
  static const KernelInfo k[2] = {
      KernelInfo{reinterpret_cast<const void *>(&kset_kernel<kKsetThreads, 4, 4, 4096, 3, false>),
                 kKsetThreads, KsetCfg<kKsetThreads, 4, 4, 4096, false>::kSmemBytes,
                 KsetCfg<kKsetThreads, 4, 4, 4096, false>::kTile, "kset_count"},
      KernelInfo{reinterpret_cast<const void *>(&kset_kernel<kKsetThreads, 4, 4, 4096, 3, true>),
                 kKsetThreads, KsetCfg<kKsetThreads, 4, 4, 4096, true>::kSmemBytes,
                 KsetCfg<kKsetThreads, 4, 4, 4096, true>::kTile, "kset_mat", true}};
  return k[mat ? 1 : 0];
}

bool gallop_thread_per_element(int variant) {
  // kGallopU32 rows 0, 4, 7 and 8 are GS = 1
  return variant == 0 || variant == 4 || variant == 7 || variant == 8;
}

int num_variants(Algo algo, bool bsr) {
  if (algo == ALGO_MERGE) return bsr ? count_of(kMergeBsr) : count_of(kMergeU32);
  if (algo == ALGO_BITMAP) return bsr ? 0 : count_of(kBitmapU32);
  return bsr ? count_of(kGallopBsr) : count_of(kGallopU32);
}

const KernelInfo &variant(Algo algo, bool bsr, bool mat, int v) {
  const int n = num_variants(algo, bsr);
  if (v < 0 || v >= n) v = 0;
  const int m = mat ? 1 : 0;
  if (algo == ALGO_MERGE) return bsr ? kMergeBsr[v][m] : kMergeU32[v][m];
  if (algo == ALGO_BITMAP && !bsr) return kBitmapU32[v][m];
  return bsr ? kGallopBsr[v][m] : kGallopU32[v][m];
}

// ---------------------------------------------------------------------------
// Sortedness check: flag := 1 if some a[i] >= a[i+1].
__global__ void validate_sorted_kernel(const uint32_t *a, uint64_t n,
                                       int *flag) {
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  bool bad = false;
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i + 1 < n;
       i += stride)
    bad |= __ldg(a + i) >= __ldg(a + i + 1);
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicExch(flag, 1);
}

cudaError_t launch_validate_sorted(const uint32_t *a, uint64_t n, int *flag,
                                   int sms, cudaStream_t st) {
  uint64_t blocks = (n + kUtilThreads * 8 - 1) / (kUtilThreads * 8);
  if (blocks > uint64_t(sms) * 8) blocks = uint64_t(sms) * 8;
  if (blocks < 1) blocks = 1;
  validate_sorted_kernel<<<unsigned(blocks), kUtilThreads, 0, st>>>(a, n, flag);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// BsrVec::from_sorted (setops/src/bsr.rs:140-163) on the device.  Tiles of
// kBsrEncodeTile elements have their edges moved forward to the next base
// change (a base holds at most 32 elements), so every word belongs to exactly
// one tile; word offsets come from decoupled look-back.
__device__ __forceinline__ uint64_t next_word_start(const uint32_t *in,
                                                    uint64_t n, uint64_t i) {
  if (i == 0 || i >= n) return i < n ? i : n;
  while (i < n && (__ldg(in + i) >> 5) == (__ldg(in + i - 1) >> 5)) ++i;
  return i;
}

__global__ void __launch_bounds__(kUtilThreads)
    bsr_encode_kernel(const uint32_t *in, uint64_t n, uint32_t *bases,
                      uint32_t *states, uint64_t *nwords, uint64_t *status,
                      LaunchSync *sync, int *err, uint32_t epoch) {
  constexpr int NT = kUtilThreads;
  __shared__ uint32_t warp_sums[NT / 32];
  __shared__ uint32_t s_tile;
  __shared__ unsigned long long s_rng[2];
  __shared__ unsigned long long s_excl;
  const int t = threadIdx.x;
  const uint64_t ntiles = (n + kBsrEncodeTile - 1) / kBsrEncodeTile;
  for (;;) {
    if (t == 0) {
      s_tile = atomicAdd(&sync->ticket, 1u);
      if (uint64_t(s_tile) < ntiles) {
        const uint64_t s = uint64_t(s_tile) * kBsrEncodeTile;
        const uint64_t e = s + kBsrEncodeTile < n ? s + kBsrEncodeTile : n;
        s_rng[0] = next_word_start(in, n, s);
        s_rng[1] = next_word_start(in, n, e);
      }
    }
    __syncthreads();
    const uint32_t tile = s_tile;
    if (uint64_t(tile) >= ntiles) break;
    const uint64_t s = s_rng[0], e = s_rng[1];
    const uint64_t len = e > s ? e - s : 0;
    const uint64_t chunk = (len + NT - 1) / NT;
    const uint64_t cs = s + chunk * t < e ? s + chunk * t : e;
    const uint64_t ce = cs + chunk < e ? cs + chunk : e;
    uint32_t starts = 0;
    for (uint64_t i = cs; i < ce; ++i)
      starts += (i == 0) || ((__ldg(in + i) >> 5) != (__ldg(in + i - 1) >> 5));
    uint32_t tot;
    const uint32_t ex = block_exclusive_scan<NT>(starts, warp_sums, &tot);
    if (t < 32) {
      const uint64_t lx = lookback_exclusive_warp(status, tile, tot, epoch, err);
      if (t == 0) s_excl = lx;
    }
    __syncthreads();
    const uint64_t tex = s_excl;
    if (tex == UINT64_MAX) return;
    uint64_t w = tex + ex;
    for (uint64_t i = cs; i < ce; ++i) {
      const uint32_t v = __ldg(in + i);
      if (i != 0 && (v >> 5) == (__ldg(in + i - 1) >> 5)) continue;
      const uint32_t base = v >> 5;
      uint32_t state = 1u << (v & 31u);
      for (uint64_t j = i + 1; j < e; ++j) {
        const uint32_t u = __ldg(in + j);
        if ((u >> 5) != base) break;
        state |= 1u << (u & 31u);
      }
      bases[w] = base;
      states[w] = state;
      ++w;
    }
    if (tile == ntiles - 1 && t == 0) *nwords = tex + tot;
    __syncthreads();
  }
  if (t == 0) {
    __threadfence();
    if (atomicAdd(&sync->done, 1u) == gridDim.x - 1) {
      if (ntiles == 0) *nwords = 0;
      sync->ticket = 0;
      sync->done = 0;
      __threadfence();
    }
  }
}

// BsrVec::to_sorted_set (setops/src/bsr.rs:77-88) on the device.
__global__ void __launch_bounds__(kUtilThreads)
    bsr_decode_kernel(const uint32_t *bases, const uint32_t *states,
                      uint64_t n, uint32_t *out, uint64_t out_cap,
                      uint64_t *out_len, uint64_t *status, LaunchSync *sync,
                      int *err, uint32_t epoch) {
  constexpr int NT = kUtilThreads;
  constexpr int WPT = kBsrDecodeTile / NT;
  __shared__ uint32_t warp_sums[NT / 32];
  __shared__ uint32_t s_tile;
  __shared__ unsigned long long s_excl;
  const int t = threadIdx.x;
  const uint64_t ntiles = (n + kBsrDecodeTile - 1) / kBsrDecodeTile;
  for (;;) {
    if (t == 0) s_tile = atomicAdd(&sync->ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    if (uint64_t(tile) >= ntiles) break;
    const uint64_t w0 = uint64_t(tile) * kBsrDecodeTile + uint64_t(t) * WPT;
    uint32_t mine = 0;
#pragma unroll
    for (int q = 0; q < WPT; ++q)
      if (w0 + q < n) mine += __popc(__ldg(states + w0 + q));
    uint32_t tot;
    const uint32_t ex = block_exclusive_scan<NT>(mine, warp_sums, &tot);
    if (t < 32) {
      const uint64_t lx = lookback_exclusive_warp(status, tile, tot, epoch, err);
      if (t == 0) s_excl = lx;
    }
    __syncthreads();
    const uint64_t tex = s_excl;
    if (tex == UINT64_MAX) return;
    if (tex + tot > out_cap) {
      if (t == 0) record_error(err, DEV_ERR_CAPACITY);
      return;
    }
    uint64_t o = tex + ex;
#pragma unroll
    for (int q = 0; q < WPT; ++q) {
      if (w0 + q >= n) break;
      const uint32_t hi = __ldg(bases + w0 + q) << 5;
      uint32_t s = __ldg(states + w0 + q);
      while (s) {
        out[o++] = hi | uint32_t(__ffs(s) - 1);
        s &= s - 1;
      }
    }
    if (tile == ntiles - 1 && t == 0) *out_len = tex + tot;
    __syncthreads();
  }
  if (t == 0) {
    __threadfence();
    if (atomicAdd(&sync->done, 1u) == gridDim.x - 1) {
      if (ntiles == 0) *out_len = 0;
      sync->ticket = 0;
      sync->done = 0;
      __threadfence();
    }
  }
}

const void *bsr_encode_fn() {
  return reinterpret_cast<const void *>(&bsr_encode_kernel);
}
const void *bsr_decode_fn() {
  return reinterpret_cast<const void *>(&bsr_decode_kernel);
}

cudaError_t launch_bsr_encode(const uint32_t *in, uint64_t n, uint32_t *bases,
                              uint32_t *states, uint64_t *nwords,
                              uint64_t *status, LaunchSync *sync, int *err,
                              uint32_t epoch, int grid, cudaStream_t st) {
  bsr_encode_kernel<<<grid, kUtilThreads, 0, st>>>(in, n, bases, states,
                                                   nwords, status, sync, err,
                                                   epoch);
  return cudaGetLastError();
}

cudaError_t launch_bsr_decode(const uint32_t *bases, const uint32_t *states,
                              uint64_t n, uint32_t *out, uint64_t out_cap,
                              uint64_t *out_len, uint64_t *status,
                              LaunchSync *sync, int *err, uint32_t epoch,
                              int grid, cudaStream_t st) {
  bsr_decode_kernel<<<grid, kUtilThreads, 0, st>>>(
      bases, states, n, out, out_cap, out_len, status, sync, err, epoch);
  return cudaGetLastError();
}

// One warp runs the look-back of tile 1 with tag `epoch`, whose predecessor
// (tile 0) never publishes: status[0] holds no word of this tag.  The wait
// therefore ends only by its time limit, which records
// DEV_ERR_TIMEOUT_LOOKBACK; *waited gets the time the warp waited.
__global__ void __launch_bounds__(32) wait_check_kernel(uint64_t *status, uint32_t epoch,
                                                        int *err, uint64_t *waited) {
  const uint64_t t0 = global_ns();
  const uint64_t r = lookback_exclusive_warp(status, 1u, 1u, epoch, err);
  if (threadIdx.x == 0) *waited = (r == UINT64_MAX) ? global_ns() - t0 : 0;
}

cudaError_t launch_wait_check(uint64_t *status, uint32_t epoch, int *err, uint64_t *waited,
                              cudaStream_t st) {
  wait_check_kernel<<<1, 32, 0, st>>>(status, epoch, err, waited);
  return cudaGetLastError();
}

}  // namespace setops
