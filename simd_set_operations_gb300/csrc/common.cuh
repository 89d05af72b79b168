// common.cuh -- device helpers shared by the set-intersection kernels.
//
// * mbarrier + cp.async.bulk (1-D TMA) wrappers for staging input windows in
//   shared memory (sm_90+ PTX; this library is built for sm_103a only);
// * bounded spin-waits: every wait has a time limit (GPU global timer),
//   after which the kernel records an error code in global memory and
//   returns instead of hanging the GPU;
// * decoupled look-back over an epoch-tagged status array, used to turn
//   per-tile match counts into global output offsets in a single pass.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace setops {

// Error codes a kernel can record in its error word (first writer wins).
enum DeviceError : int {
  DEV_OK = 0,
  DEV_ERR_TIMEOUT_MBAR = 1,      // a bulk-copy barrier never completed
  DEV_ERR_TIMEOUT_LOOKBACK = 2,  // a predecessor tile never published
  DEV_ERR_CAPACITY = 3,          // output would exceed its capacity
};

// Wait limits, in nanoseconds of the GPU's global timer.  A bulk copy of a
// few KB or a predecessor tile publishing its count takes microseconds; a
// wait that reaches the limit records an error and the kernel returns.
constexpr uint64_t kDefaultWaitLimitNs = 2000000000ull;  // 2 s

// The limit in force.  Without relocatable device code every translation
// unit has its own copy (per device); setops_gpu_set_wait_limit_ns writes
// all of them through the setters registered below.
static __device__ uint64_t g_wait_limit_ns = kDefaultWaitLimitNs;

__device__ __forceinline__ uint64_t wait_limit_ns() { return g_wait_limit_ns; }

// Host side: each translation unit that includes this header registers a
// setter of its own copy at static initialisation (the registry is in
// runtime.cu).  A setter writes the copy on the current device.
using WaitLimitSetter = cudaError_t (*)(uint64_t ns);
void register_wait_limit_setter(WaitLimitSetter fn);

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// floor(x / den * num) as an index guess, at most num (den > 0).  Single
// precision: this GPU's double-precision rate is a small fraction of its
// single-precision one, and every guess here is followed by an exact search,
// so a few significant digits are enough.
__device__ __forceinline__ uint64_t guess_scale(uint64_t x, uint64_t den, uint64_t num) {
  const float g = float(x) / float(den) * float(num);
  return g <= 0.0f ? 0 : (g >= float(num) ? num : uint64_t(g));
}

__device__ __forceinline__ void record_error(int *err, int code) {
  if (err) atomicCAS(err, 0, code);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---- mbarrier ------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar,
                                                      uint32_t bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
          smem_u32(bar)),
      "r"(bytes)
      : "memory");
}

// Plain arrival (no bytes expected): completes a phase whose copy is empty.
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Orders this thread's earlier generic-proxy shared-memory accesses (and
// those it has synchronised with) before later async-proxy ones: used before
// a bulk copy overwrites a buffer that threads have been reading.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Non-blocking test: has phase `parity` of `bar` completed?
__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Named barrier `ID` over N threads (N a multiple of 32).
template <int ID, int N>
__device__ __forceinline__ void named_bar_sync() {
  asm volatile("bar.sync %0, %1;" ::"n"(ID), "n"(N) : "memory");
}

// Waits for phase `parity` of `bar` to complete.  Returns false (and records
// DEV_ERR_TIMEOUT_MBAR) if the limit is reached.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar,
                                                  uint32_t parity, int *err) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > wait_limit_ns()) break;
  }
  record_error(err, DEV_ERR_TIMEOUT_MBAR);
  return false;
}

// As mbar_wait_bounded, for blocks whose threads share an abort flag in
// shared memory: a timeout sets the flag, and a wait that sees the flag set
// gives up at once, so one failed copy costs one time limit, not one per
// later wait.
__device__ __forceinline__ bool mbar_wait_abortable(uint64_t *bar,
                                                    uint32_t parity, int *err,
                                                    volatile uint32_t *abort) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort) return false;
    if (global_ns() - t0 > wait_limit_ns()) {
      record_error(err, DEV_ERR_TIMEOUT_MBAR);
      *abort = 1u;
      return false;
    }
  }
}

// 1-D bulk copy global -> shared, completing `bytes` on `bar`.  dst, src and
// bytes must be multiples of 16.  The evict-first L2 policy marks the
// streamed inputs as read-once.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src,
                                         uint32_t bytes, uint64_t *bar,
                                         uint64_t policy) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes."
      "L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(policy)
      : "memory");
}

// Asks the L2 to fetch global [p, p + bytes) ahead of the loads that will
// read it (1-D bulk prefetch: no registers, nothing to wait for).  p and
// bytes must be multiples of 16 and the range inside the allocation.
__device__ __forceinline__ void bulk_prefetch_l2(const void *p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Prefetch (as above) of the whole 16-byte words [q0, q1) of x4, clipped to
// [qlo, qhi) (the words wholly inside the array), in pieces of 64 KB.
__device__ __forceinline__ void prefetch_words_l2(const uint4 *x4, uint64_t q0, uint64_t q1,
                                                  uint64_t qlo, uint64_t qhi) {
  q0 = q0 > qlo ? q0 : qlo;
  q1 = q1 < qhi ? q1 : qhi;
  for (; q0 < q1; q0 += 4096) {
    const uint64_t n = (q1 - q0 < 4096) ? q1 - q0 : 4096;
    bulk_prefetch_l2(x4 + q0, uint32_t(n) * 16u);
  }
}

__device__ __forceinline__ uint64_t l2_evict_first_policy() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;"
               : "=l"(pol));
  return pol;
}

// ---- global status words -------------------------------------------------
__device__ __forceinline__ uint64_t ld_acquire_u64(const uint64_t *p) {
  uint64_t v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];"
               : "=l"(v)
               : "l"(p)
               : "memory");
  return v;
}

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_u64(uint64_t *p, uint64_t v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v)
               : "memory");
}

// Look-back status word: [63:48] epoch (launch tag), [47:46] flag,
// [45:0] value.  Entries from earlier launches carry another epoch and read
// as "not yet published", so the array never needs clearing between launches.
constexpr uint64_t kFlagAggregate = 1;
constexpr uint64_t kFlagPrefix = 2;
constexpr uint64_t kValueMask = (uint64_t(1) << 46) - 1;

__device__ __forceinline__ uint64_t pack_status(uint32_t epoch, uint64_t flag,
                                                uint64_t value) {
  return (uint64_t(epoch & 0xffffu) << 48) | (flag << 46) | (value & kValueMask);
}

// Decoupled look-back (single thread).  Publishes `aggregate` for `tile`,
// walks predecessors until an inclusive prefix is found, publishes this
// tile's inclusive prefix and returns the exclusive prefix.  Tiles must have
// been started in increasing order (tile ids come from an atomic ticket), so
// every predecessor is running or finished and the walk terminates; the spin
// is bounded anyway.  Returns UINT64_MAX on timeout (error recorded).
__device__ __forceinline__ uint64_t lookback_exclusive(uint64_t *status,
                                                       uint32_t tile,
                                                       uint64_t aggregate,
                                                       uint32_t epoch,
                                                       int *err) {
  if (tile == 0) {
    st_release_u64(&status[0], pack_status(epoch, kFlagPrefix, aggregate));
    return 0;
  }
  st_release_u64(&status[tile], pack_status(epoch, kFlagAggregate, aggregate));
  uint64_t excl = 0;
  int64_t t = int64_t(tile) - 1;
  uint64_t t0 = 0;
  while (t >= 0) {
    uint64_t w = ld_acquire_u64(&status[t]);
    uint32_t e = uint32_t(w >> 48);
    uint64_t flag = (w >> 46) & 3;
    if (e != (epoch & 0xffffu) || flag == 0) {
      if (t0 == 0) {
        t0 = global_ns();
      } else if (global_ns() - t0 > wait_limit_ns()) {
        record_error(err, DEV_ERR_TIMEOUT_LOOKBACK);
        return UINT64_MAX;
      }
      continue;
    }
    excl += (w & kValueMask);
    if (flag == kFlagPrefix) break;
    --t;
  }
  st_release_u64(&status[tile],
                 pack_status(epoch, kFlagPrefix, excl + aggregate));
  return excl;
}

// Warp-parallel decoupled look-back: call with all 32 lanes of one warp.
// Each round reads the status words of the 32 preceding tiles at once; the
// nearest inclusive prefix ends the walk, otherwise the 32 aggregates are
// added and the window moves back.  Returns the exclusive prefix in every
// lane (UINT64_MAX on timeout, error recorded).
__device__ __forceinline__ uint64_t lookback_exclusive_warp(
    uint64_t *status, uint32_t tile, uint64_t aggregate, uint32_t epoch,
    int *err) {
  const int lane = threadIdx.x & 31;
  if (tile == 0) {
    if (lane == 0)
      st_release_u64(&status[0], pack_status(epoch, kFlagPrefix, aggregate));
    return 0;
  }
  if (lane == 0)
    st_release_u64(&status[tile], pack_status(epoch, kFlagAggregate, aggregate));
  const uint32_t ep = epoch & 0xffffu;
  uint64_t excl = 0;
  int64_t base = int64_t(tile);  // window covers tiles base-1 .. base-32
  uint64_t t0 = 0;
  for (;;) {
    const int64_t idx = base - 1 - lane;
    uint64_t val = 0;
    uint32_t flag = uint32_t(kFlagPrefix);  // before tile 0: prefix 0
    if (idx >= 0) {
      const uint64_t w = ld_acquire_u64(&status[idx]);
      flag = (uint32_t(w >> 48) == ep) ? uint32_t((w >> 46) & 3) : 0u;
      val = w & kValueMask;
    }
    const unsigned pre = __ballot_sync(0xffffffffu, flag == kFlagPrefix);
    const unsigned nrd = __ballot_sync(0xffffffffu, flag == 0);
    const int p = pre ? __ffs(pre) - 1 : 32;
    const unsigned need = (p >= 31) ? 0xffffffffu : ((2u << p) - 1u);
    if (nrd & need) {
      if (t0 == 0) {
        t0 = global_ns();
      } else if (global_ns() - t0 > wait_limit_ns()) {
        if (lane == 0) record_error(err, DEV_ERR_TIMEOUT_LOOKBACK);
        return UINT64_MAX;
      }
      continue;
    }
    uint64_t c = (lane <= p) ? val : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    excl += c;
    if (p < 32) break;
    base -= 32;
  }
  if (lane == 0)
    st_release_u64(&status[tile], pack_status(epoch, kFlagPrefix, excl + aggregate));
  return excl;
}

// True when a kernel with device-side choice rule `rule` should not run for
// lengths (na, nb): rule 1 runs only when max/min >= thr, rule 2 only below.
// An empty input counts as "search" (either kernel returns 0).
__device__ __forceinline__ bool skip_by_rule(int rule, uint32_t thr,
                                             uint64_t na, uint64_t nb) {
  if (rule == 0) return false;
  const uint64_t mn = na < nb ? na : nb, mx = na < nb ? nb : na;
  const bool search = (mn == 0) || (mx / mn >= uint64_t(thr));
  return (rule == 1) ? !search : search;
}

// Per-launch coordination words kept in scratch (zeroed once at allocation;
// the last CTA of every launch restores them to zero).
struct LaunchSync {
  uint32_t ticket;  // next virtual CTA / tile id
  uint32_t done;    // CTAs finished
  unsigned long long acc;  // count accumulator (count-only kernels)
};

// Block-wide exclusive scan of one uint32 per thread.  `warp_sums` needs
// NT/32 entries of shared memory.  Returns the exclusive prefix; *total gets
// the block total.  Contains __syncthreads(); call from all threads.
template <int NT>
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v,
                                                         uint32_t *warp_sums,
                                                         uint32_t *total) {
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  uint32_t wpre = 0, tot = 0;
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    uint32_t s = warp_sums[w];
    wpre += (w < warp) ? s : 0u;
    tot += s;
  }
  __syncthreads();
  *total = tot;
  return wpre + x - v;
}

// First index i in [0, n) with B[i] >= *keyp (n when none), n > 0; all lanes
// of the calling warp take part and get the result, and the key in *key_out.
// `est` guesses the index.  Round 1 loads the key together with 128 probes
// S = max(1, sqrt(n)/16) apart around est (for two sets drawn from the same
// distribution the index error is O(sqrt(n))); when the probes bracket the
// key to at most 256 elements, one more round reads the bracket and counts
// the elements below the key.  Otherwise round 2 probes the same way around
// an interpolation of the key's value between B's first and last values
// (loaded in round 1), and after that 129-ary rounds narrow what is left.
__device__ __forceinline__ uint64_t warp_lower_bound_guess(const uint32_t *__restrict__ B,
                                                           uint64_t n, const uint32_t *keyp,
                                                           uint64_t est, uint32_t *key_out) {
  const int lane = threadIdx.x & 31;
  const uint32_t key = __ldg(keyp);
  const uint32_t bfirst = __ldg(B), blast = __ldg(B + n - 1);
  uint64_t lo = 0, hi = n;  // answer in [lo, hi]
  // 128 probes at positions p(k), k = 4*lane + j, clamped into [lo, hi)
  auto narrow = [&](auto pos) {
    uint64_t l = lo, h = hi;
    uint64_t x[4];
    uint32_t v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int64_t q = pos(4 * lane + j);
      q = q < int64_t(lo) ? int64_t(lo) : q;
      q = q > int64_t(hi) - 1 ? int64_t(hi) - 1 : q;
      x[j] = uint64_t(q);
      v[j] = __ldg(B + x[j]);
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (v[j] < key) l = x[j] + 1 > l ? x[j] + 1 : l;
      else h = x[j] < h ? x[j] : h;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const uint64_t l2 = __shfl_xor_sync(0xffffffffu, l, o);
      const uint64_t h2 = __shfl_xor_sync(0xffffffffu, h, o);
      l = l2 > l ? l2 : l;
      h = h2 < h ? h2 : h;
    }
    lo = l;
    hi = h;
  };
  if (n > 256) {
    const int64_t S = int64_t(sqrtf(float(n)) * (1.0f / 16.0f)) > 1
                          ? int64_t(sqrtf(float(n)) * (1.0f / 16.0f))
                          : 1;
    const int64_t g1 = int64_t(est < n ? est : n - 1);
    narrow([&](int k) { return g1 + int64_t(k - 64) * S; });
    if (hi - lo > 256) {
      const uint64_t g2 =
          (blast <= bfirst || key <= bfirst)
              ? lo
              : guess_scale(key - bfirst, blast - bfirst, n - 1);
      const int64_t gg = int64_t(g2);
      narrow([&](int k) { return gg + int64_t(k - 64) * S; });
    }
    while (hi - lo > 256) {
      const uint64_t l0 = lo, span = hi - lo;
      narrow([&](int k) { return int64_t(l0 + uint64_t(k + 1) * span / 129); });
    }
  }
  // the bracket [lo, hi), at most 256 elements: count those below the key
  uint32_t c = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const uint64_t i = lo + uint64_t(lane + 32 * j);
    c += (i < hi && __ldg(B + i) < key) ? 1u : 0u;
  }
  *key_out = key;
  return lo + __reduce_add_sync(0xffffffffu, c);
}

// A bracket [*lo, *hi] of the first index i with B[i] >= *keyp, n > 0, at
// most S = max(1, sqrt(n)/8) wide, for callers that only need bounds: one
// round in which the key and 64 probes S apart around the guess `est` are
// loaded together; the largest probe below the key and the smallest one not
// below it bound the index.  When the probes do not bracket it (the guess was
// far off) the exact index, by warp_lower_bound_guess (*lo == *hi).  All
// lanes take part and get the result.
__device__ __forceinline__ void warp_bracket_guess(const uint32_t *__restrict__ B, uint64_t n,
                                                   const uint32_t *keyp, uint64_t est,
                                                   uint64_t *lo, uint64_t *hi) {
  const int lane = threadIdx.x & 31;
  if (n > 64) {
    const uint32_t key = __ldg(keyp);
    const float r = sqrtf(float(n)) * 0.125f;
    const int64_t S = r > 1.0f ? int64_t(r) : 1;
    const int64_t g = int64_t(est < n ? est : n - 1);
    uint64_t below = 0;  // largest probe below the key, + 1 (0: none)
    uint64_t above = n;  // smallest probe not below the key (n: none)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      int64_t q = g + int64_t(2 * lane + j - 32) * S;
      q = q < 0 ? 0 : (q > int64_t(n) - 1 ? int64_t(n) - 1 : q);
      if (__ldg(B + q) < key) below = uint64_t(q) + 1 > below ? uint64_t(q) + 1 : below;
      else above = uint64_t(q) < above ? uint64_t(q) : above;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const uint64_t b2 = __shfl_xor_sync(0xffffffffu, below, o);
      const uint64_t a2 = __shfl_xor_sync(0xffffffffu, above, o);
      below = b2 > below ? b2 : below;
      above = a2 < above ? a2 : above;
    }
    // bracketed from both sides (no probe below: the lowest probe is index 0)
    if (above < n && (below > 0 || above == 0)) {
      *lo = below;
      *hi = above;
      return;
    }
  }
  uint32_t k;
  const uint64_t x = warp_lower_bound_guess(B, n, keyp, est, &k);
  *lo = x;
  *hi = x;
}

// A start index for reading B from the key *keyp on: some s <= the first
// index i with B[i] >= key, at most sqrt(n)/8 below it (warp_bracket_guess's
// lower end) -- for callers that discard B elements below the key by value.
__device__ __forceinline__ uint64_t warp_start_below(const uint32_t *__restrict__ B, uint64_t n,
                                                     const uint32_t *keyp, uint64_t est) {
  if (n == 0) return 0;
  uint64_t lo, hi;
  warp_bracket_guess(B, n, keyp, est, &lo, &hi);
  return lo;
}

static cudaError_t set_wait_limit_this_unit(uint64_t ns) {
  return cudaMemcpyToSymbol(g_wait_limit_ns, &ns, sizeof ns);
}
[[maybe_unused]] static const bool g_wait_limit_setter_registered =
    (register_wait_limit_setter(&set_wait_limit_this_unit), true);

}  // namespace setops
