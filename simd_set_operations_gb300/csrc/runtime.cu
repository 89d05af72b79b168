// runtime.cu -- host runtime behind the C ABI (include/setops_gpu.h):
// context, scratch pool, algorithm choice, kernel launches, and the k-set
// SvS driver that keeps intermediates on the device.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/setops_gpu.h"
#include "gallop.cuh"
#include "kernels.h"
#include "kset.cuh"
#include "merge.cuh"
#include "runtime.h"

using namespace setops;

// ---------------------------------------------------------------------------
// context helpers

namespace {

const char *kStatusText[] = {
    "ok",          "invalid argument", "output capacity too small",
    "CUDA error",  "out of memory",    "device wait timed out",
    "unsorted input", "busy",          "input too large",
    "not ready"};

}  // namespace

// Setters of the per-unit copies of the device wait limit (common.cuh).  A
// function-local registry: units register during static initialisation.
static std::vector<WaitLimitSetter> &wait_limit_setters() {
  static std::vector<WaitLimitSetter> v;
  return v;
}

void setops::register_wait_limit_setter(WaitLimitSetter fn) {
  wait_limit_setters().push_back(fn);
}

int ctx_fail(setops_ctx *ctx, int status, const std::string &what) {
  if (ctx) ctx->err = what;
  return status;
}

int ctx_cuda(setops_ctx *ctx, cudaError_t e, const char *what) {
  if (e == cudaSuccess) return SETOPS_OK;
  std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation)
    return ctx_fail(ctx, SETOPS_ERR_NOMEM, msg);
  return ctx_fail(ctx, SETOPS_ERR_CUDA, msg);
}

#define CK(call)                                                     \
  do {                                                               \
    cudaError_t e_ = (call);                                         \
    if (e_ != cudaSuccess) return ctx_cuda(ctx, e_, #call);          \
  } while (0)
#define RK(call)                 \
  do {                           \
    int r_ = (call);             \
    if (r_ != SETOPS_OK) return r_; \
  } while (0)

int buf_reserve(setops_ctx *ctx, DevBuf &b, size_t bytes) {
  if (bytes <= b.cap) return SETOPS_OK;
  size_t want = std::max<size_t>(bytes, 4096);
  want = std::max(want, b.cap + b.cap / 2);  // grow geometrically
  if (b.p) {
    CK(cudaStreamSynchronize(ctx->st));
    CK(cudaFree(b.p));
    b.p = nullptr;
    b.cap = 0;
  }
  cudaError_t e = cudaMalloc(&b.p, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    e = cudaMalloc(&b.p, bytes);  // retry at the exact size
    if (e != cudaSuccess) {
      cudaGetLastError();
      b.p = nullptr;
      return ctx_fail(ctx, SETOPS_ERR_NOMEM,
                      "device allocation of " + std::to_string(bytes) +
                          " bytes failed");
    }
    want = bytes;
  }
  b.cap = want;
  return SETOPS_OK;
}

// Blocks per SM of a kernel at its launch shape (cached), also raising the
// dynamic shared-memory limit the first time.
int ctx_occupancy(setops_ctx *ctx, const KernelInfo &k, int *blocks) {
  auto it = ctx->occ.find(k.fn);
  if (it != ctx->occ.end()) {
    *blocks = it->second;
    return SETOPS_OK;
  }
  // opt in whenever dynamic shared memory is used: static plus dynamic
  // shared memory above 48 KB needs it
  if (k.dyn_smem > 0)
    CK(cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            int(k.dyn_smem)));
  int n = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k.fn, k.nt, k.dyn_smem));
  if (n < 1) n = 1;
  ctx->occ[k.fn] = n;
  *blocks = n;
  return SETOPS_OK;
}

// Next launch tag for look-back status words; wraps within 16 bits, and the
// status array is cleared whenever the tag wraps so that stale words of an
// earlier launch with the same tag cannot be mistaken for fresh ones.
int ctx_next_epoch(setops_ctx *ctx, uint32_t *epoch) {
  ctx->epoch = (ctx->epoch + 1) & 0xffffu;
  if (ctx->epoch == 0) {
    if (ctx->status.p)
      CK(cudaMemsetAsync(ctx->status.p, 0, ctx->status.cap, ctx->st));
    ctx->epoch = 1;
  }
  *epoch = ctx->epoch;
  return SETOPS_OK;
}

int ctx_status_words(setops_ctx *ctx, uint64_t n) {
  const size_t need = size_t(std::max<uint64_t>(n, 1)) * sizeof(uint64_t);
  if (need <= ctx->status.cap) return SETOPS_OK;
  const size_t old = ctx->status.cap;
  RK(buf_reserve(ctx, ctx->status, need));
  (void)old;
  CK(cudaMemsetAsync(ctx->status.p, 0, ctx->status.cap, ctx->st));
  return SETOPS_OK;
}

// Device error word -> status; clears device state after an error so the
// next call starts clean.
int ctx_check_device(setops_ctx *ctx) {
  CK(cudaMemcpyAsync(&ctx->hres[15], ctx->derr, sizeof(int),
                     cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  int code = 0;
  std::memcpy(&code, &ctx->hres[15], sizeof(int));
  if (code == 0) return SETOPS_OK;
  CK(cudaMemsetAsync(ctx->derr, 0, sizeof(int), ctx->st));
  CK(cudaMemsetAsync(ctx->sync, 0, sizeof(LaunchSync) * kSyncSlots, ctx->st));
  if (ctx->status.p)
    CK(cudaMemsetAsync(ctx->status.p, 0, ctx->status.cap, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  switch (code) {
    case DEV_ERR_CAPACITY:
      return ctx_fail(ctx, SETOPS_ERR_CAPACITY,
                      "device: output would exceed its capacity");
    case DEV_ERR_TIMEOUT_MBAR:
      return ctx_fail(ctx, SETOPS_ERR_TIMEOUT,
                      "device: bulk-copy barrier wait hit its limit");
    case DEV_ERR_TIMEOUT_LOOKBACK:
      return ctx_fail(ctx, SETOPS_ERR_TIMEOUT,
                      "device: look-back wait hit its limit");
    default:
      return ctx_fail(ctx, SETOPS_ERR_CUDA,
                      "device error code " + std::to_string(code));
  }
}

// Reads a device u64 into *out (synchronises) and checks the error word.
int ctx_read_u64(setops_ctx *ctx, const uint64_t *dev, uint64_t *out) {
  CK(cudaMemcpyAsync(&ctx->hres[0], dev, sizeof(uint64_t),
                     cudaMemcpyDeviceToHost, ctx->st));
  RK(ctx_check_device(ctx));
  *out = ctx->hres[0];
  return SETOPS_OK;
}

// ---------------------------------------------------------------------------
// algorithm choice

Choice ctx_choose(const setops_ctx *ctx, uint64_t na, uint64_t nb, bool bsr,
                  unsigned flags) {
  Choice c;
  const unsigned algo = (flags & SETOPS_ALGO_MASK);
  const int var = int((flags & SETOPS_VARIANT_MASK) >> SETOPS_VARIANT_SHIFT);
  if (algo == SETOPS_ALGO_MERGE) {
    c.algo = ALGO_MERGE;
    c.variant = var;
    return c;
  }
  if (algo == SETOPS_ALGO_GALLOP) {
    c.algo = ALGO_GALLOP;
    c.variant = var;
    return c;
  }
  if (algo == SETOPS_ALGO_BITMAP) {
    // arrays only; BSR sets take the merge kernel
    c.algo = bsr ? ALGO_MERGE : ALGO_BITMAP;
    c.variant = bsr ? 0 : var;
    return c;
  }
  const uint64_t mn = std::min(na, nb), mx = std::max(na, nb);
  if (mn == 0) {
    c.algo = ALGO_GALLOP;
    c.variant = 0;
    return c;
  }
  int band = 0;
  for (uint64_t r = mx / mn; r > 1 && band < kRatioBands - 1; r >>= 1) ++band;
  const unsigned pol = ctx->policy[bsr ? 1 : 0][band][size_class(mn)];
  const unsigned pa = pol & SETOPS_ALGO_MASK;
  c.algo = (pa == SETOPS_ALGO_GALLOP)               ? ALGO_GALLOP
           : (pa == SETOPS_ALGO_BITMAP && !bsr)     ? ALGO_BITMAP
                                                    : ALGO_MERGE;
  c.variant = int((pol & SETOPS_VARIANT_MASK) >> SETOPS_VARIANT_SHIFT);
  return c;
}

// Smallest power-of-two ratio at which the policy switches to the search
// kernel (used for device-side choices).
uint32_t ctx_search_threshold(const setops_ctx *ctx, bool bsr) {
  for (int band = 0; band < kRatioBands; ++band)
    if ((ctx->policy[bsr ? 1 : 0][band][kSizeClasses - 1] & SETOPS_ALGO_MASK) ==
        SETOPS_ALGO_GALLOP)
      return 1u << band;
  return 0xffffffffu;
}

void ctx_default_policy(setops_ctx *ctx) {
  for (int b = 0; b < kRatioBands; ++b) {
    // arrays: ratio < 32: tiled bitmap with coarse
    // bitmaps for sparse tiles (variant 7); 32..511: sampled
    // thread-per-element search; 512..8191: 8 lanes per element (4 elements
    // a warp); >= 8192: a warp per element.  BSR: block broadcast below 32.
    // (Measured on 2^10 / 2^14 / 2^18 / 2^20-2^23 x 2^24 pairs: each band's
    // choice was the fastest variant there.)
    unsigned v = (b < 5)    ? (SETOPS_ALGO_MERGE | SETOPS_VARIANT(0))
                 : (b < 9)  ? (SETOPS_ALGO_GALLOP | SETOPS_VARIANT(0))
                 : (b < 13) ? (SETOPS_ALGO_GALLOP | SETOPS_VARIANT(3))
                            : (SETOPS_ALGO_GALLOP | SETOPS_VARIANT(2));
    unsigned u = (b < 5) ? (SETOPS_ALGO_BITMAP | SETOPS_VARIANT(kCoarseBitmap)) : v;
    // BSR below 32: the block-broadcast kernel (0.042-0.045 ms against
    // 0.09-0.16 ms for the merge-path kernels materialising 2^20-word pairs);
    // above, the BSR search variants that exist: sampled thread per element,
    // then a warp per element from 8192
    unsigned w = (b < 5)    ? (SETOPS_ALGO_MERGE | SETOPS_VARIANT(kBcastBsr))
                 : (b < 13) ? (SETOPS_ALGO_GALLOP | SETOPS_VARIANT(0))
                            : (SETOPS_ALGO_GALLOP | SETOPS_VARIANT(2));
    for (int c = 0; c < kSizeClasses; ++c) {
      ctx->policy[0][b][c] = u;
      ctx->policy[1][b][c] = w;
    }
  }
  // the balanced band's largest pairs: the window kernel with both inputs
  // staged in shared memory (the coarse-bitmap variant's second table costs
  // a few per cent on dense pairs there; below 2^22 the two are equal on
  // dense pairs and the coarse one about twice as fast on sparse ones)
  ctx->policy[0][0][kSizeClasses - 1] = SETOPS_ALGO_BITMAP | SETOPS_VARIANT(kStagedWindow);
  // ratios 32-511 with a smaller input of 2^16 to 2^22 elements: the sampled
  // search with 512-element tiles, so a launch has more CTAs to hide its
  // probes' latency (2^18 x 2^24: 0.0213 against 0.0234 ms with 1024)
  for (int b = 5; b < 9; ++b) ctx->policy[0][b][2] = SETOPS_ALGO_GALLOP | SETOPS_VARIANT(8);
}

// ---------------------------------------------------------------------------
// one 2-set launch (device pointers)

int ctx_launch_pair(setops_ctx *ctx, const PairJob &j) {
  const uint64_t na_ub = j.na, nb_ub = j.nb;
  const uint64_t mn = std::min(na_ub, nb_ub);
  const bool mat = j.out != nullptr;
  const KernelInfo &k = variant(j.choice.algo, j.bsr, mat, j.choice.variant);
  int occ = 1;
  RK(ctx_occupancy(ctx, k, &occ));
  const uint64_t full = uint64_t(occ) * uint64_t(ctx->sms);
  uint64_t grid = 1, status_words = 1;
  uint64_t ntiles = 0;
  if (j.choice.algo == ALGO_MERGE) {
    const uint64_t total = na_ub + nb_ub;
    const uint64_t per = uint64_t(k.tile) * kMinTilesPerCta;
    grid = std::max<uint64_t>(1, std::min(full, (total + per - 1) / per));
    status_words = grid;
  } else if (j.choice.algo == ALGO_BITMAP) {
    // persistent grid: a CTA per two tiles' worth of both inputs (a balanced
    // pair: a CTA per tile of the smaller set; a skewed one spreads the
    // longer set's stream over the whole GPU)
    ntiles = (na_ub + nb_ub + 2 * uint64_t(k.tile) - 1) / (2 * uint64_t(k.tile));
    grid = std::max<uint64_t>(1, std::min(full, ntiles));
    status_words = std::max<uint64_t>(ntiles, 1);
  } else {
    const uint64_t ntiles = (mn + k.tile - 1) / k.tile;
    grid = std::max<uint64_t>(1, std::min(full, ntiles));
    status_words = grid + 1;  // per-CTA counts, then the total
  }
  if (j.grid_cap && grid > j.grid_cap) grid = j.grid_cap;
  uint32_t epoch = 0;
  // merge kernels publish per-CTA co-ranks after the look-back words
  const bool merge = j.choice.algo == ALGO_MERGE || j.choice.algo == ALGO_BITMAP;
  RK(ctx_status_words(ctx, merge ? status_words + grid : status_words));
  RK(ctx_next_epoch(ctx, &epoch));
  LaunchSync *sync = ctx->sync + j.sync_slot;

  uint32_t *stage = nullptr, *stage_s = nullptr;
  if (mat) {
    RK(buf_reserve(ctx, ctx->stage0, std::max<uint64_t>(mn, 1) * 4));
    stage = static_cast<uint32_t *>(ctx->stage0.p);
    if (j.bsr) {
      RK(buf_reserve(ctx, ctx->stage1, std::max<uint64_t>(mn, 1) * 4));
      stage_s = static_cast<uint32_t *>(ctx->stage1.p);
    }
  }
  if (j.choice.algo == ALGO_MERGE || j.choice.algo == ALGO_BITMAP) {
    MergeArgs a{};
    a.a = j.a;
    a.b = j.b;
    a.sa = j.sa;
    a.sb = j.sb;
    a.na = j.na;
    a.nb = j.nb;
    a.na_dev = j.na_dev;
    a.nb_dev = j.nb_dev;
    a.stage = stage;
    a.stage_s = stage_s;
    a.out = j.out;
    a.out_s = j.out_s;
    a.out_cap = j.out_cap;
    a.out_len = j.len_dev;
    a.status = static_cast<uint64_t *>(ctx->status.p);
    a.coranks = static_cast<uint64_t *>(ctx->status.p) + status_words;
    a.sync = sync;
    a.err = ctx->derr;
    a.epoch = epoch;
    a.skip_rule = j.skip_rule;
    a.ratio_thr = j.ratio_thr;
    void *args[] = {&a};
    RK(ctx_launch(ctx, k, grid, args));
  } else {
    GallopArgs a{};
    a.a = j.a;
    a.b = j.b;
    a.sa = j.sa;
    a.sb = j.sb;
    a.na = j.na;
    a.nb = j.nb;
    a.na_dev = j.na_dev;
    a.nb_dev = j.nb_dev;
    a.stage = stage;
    a.stage_s = stage_s;
    a.out = j.out;
    a.out_s = j.out_s;
    a.out_cap = j.out_cap;
    a.out_len = j.len_dev;
    a.status = static_cast<uint64_t *>(ctx->status.p);
    a.sync = sync;
    a.err = ctx->derr;
    a.epoch = epoch;
    a.skip_rule = j.skip_rule;
    a.ratio_thr = j.ratio_thr;
    void *args[] = {&a};
    RK(ctx_launch(ctx, k, grid, args));
  }
  ctx->launches++;
  return SETOPS_OK;
}

// Launches kernel k with one argument block; errors name the launch shape.
int ctx_launch(setops_ctx *ctx, const KernelInfo &k, uint64_t grid,
               void **args) {
  const cudaError_t e =
      k.coop ? cudaLaunchCooperativeKernel(k.fn, dim3(unsigned(grid)), dim3(k.nt), args,
                                           k.dyn_smem, ctx->st)
             : cudaLaunchKernel(k.fn, dim3(unsigned(grid)), dim3(k.nt), args, k.dyn_smem,
                                ctx->st);
  if (e == cudaSuccess) return SETOPS_OK;
  char buf[256];
  std::snprintf(buf, sizeof buf, "launch of %s (grid %llu, block %d, %zu B shared)",
                k.name, (unsigned long long)grid, k.nt, k.dyn_smem);
  return ctx_cuda(ctx, e, buf);
}

// Copies host arrays into staging slot `slot` and returns the device pointer.
int ctx_stage_in(setops_ctx *ctx, int slot, const uint32_t *h, size_t n,
                 const uint32_t **d) {
  if (n == 0) {
    *d = nullptr;
    return SETOPS_OK;
  }
  RK(buf_reserve(ctx, ctx->in[slot], n * 4));
  CK(cudaMemcpyAsync(ctx->in[slot].p, h, n * 4, cudaMemcpyHostToDevice,
                     ctx->st));
  *d = static_cast<const uint32_t *>(ctx->in[slot].p);
  return SETOPS_OK;
}

// ---------------------------------------------------------------------------
// C ABI

extern "C" {

const char *setops_status_string(int status) {
  if (status > 0 || status < -9) return "unknown status";
  return kStatusText[-status];
}

int setops_gpu_create(setops_ctx **out, int device) {
  if (!out) return SETOPS_ERR_INVALID;
  *out = nullptr;
  setops_ctx *ctx = new (std::nothrow) setops_ctx();
  if (!ctx) return SETOPS_ERR_NOMEM;
  ctx->device = device;
  int rc = SETOPS_OK;
  do {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) { rc = ctx_cuda(ctx, e, "cudaSetDevice"); break; }
    e = cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) { rc = ctx_cuda(ctx, e, "sm count"); break; }
    e = cudaStreamCreateWithFlags(&ctx->own, cudaStreamNonBlocking);
    if (e != cudaSuccess) { rc = ctx_cuda(ctx, e, "stream"); break; }
    ctx->st = ctx->own;
    // device scalars: [sync slots][err + flag][len words]
    const size_t bytes = sizeof(LaunchSync) * kSyncSlots + 64 +
                         sizeof(uint64_t) * kLenWords;
    e = cudaMalloc(&ctx->dsmall, bytes);
    if (e != cudaSuccess) { rc = ctx_cuda(ctx, e, "scalars"); break; }
    e = cudaMemset(ctx->dsmall, 0, bytes);
    if (e != cudaSuccess) { rc = ctx_cuda(ctx, e, "memset"); break; }
    char *p = static_cast<char *>(ctx->dsmall);
    ctx->sync = reinterpret_cast<LaunchSync *>(p);
    p += sizeof(LaunchSync) * kSyncSlots;
    ctx->derr = reinterpret_cast<int *>(p);
    ctx->dflag = reinterpret_cast<int *>(p + 32);
    p += 64;
    ctx->dlen = reinterpret_cast<uint64_t *>(p);
    e = cudaMallocHost(&ctx->hres, sizeof(uint64_t) * 16);
    if (e != cudaSuccess) { rc = ctx_cuda(ctx, e, "pinned scalars"); break; }
    ctx_default_policy(ctx);
  } while (0);
  if (rc != SETOPS_OK) {
    std::fprintf(stderr, "setops_gpu_create: %s\n", ctx->err.c_str());
    setops_gpu_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return SETOPS_OK;
}

int setops_gpu_destroy(setops_ctx *ctx) {
  if (!ctx) return SETOPS_ERR_INVALID;
  if (ctx->st) cudaStreamSynchronize(ctx->st);
  for (DevBuf *b : ctx->all_bufs())
    if (b->p) cudaFree(b->p);
  if (ctx->aux) cudaStreamSynchronize(ctx->aux);
  if (ctx->dsmall) cudaFree(ctx->dsmall);
  if (ctx->hres) cudaFreeHost(ctx->hres);
  if (ctx->hlens) cudaFreeHost(ctx->hlens);
  if (ctx->ev_main) cudaEventDestroy(ctx->ev_main);
  if (ctx->ev_aux) cudaEventDestroy(ctx->ev_aux);
  if (ctx->aux) cudaStreamDestroy(ctx->aux);
  if (ctx->own) cudaStreamDestroy(ctx->own);
  delete ctx;
  return SETOPS_OK;
}

int setops_gpu_set_stream(setops_ctx *ctx, void *stream) {
  if (!ctx) return SETOPS_ERR_INVALID;
  CK(cudaStreamSynchronize(ctx->st));
  ctx->st = stream ? static_cast<cudaStream_t>(stream) : ctx->own;
  return SETOPS_OK;
}

void *setops_gpu_get_stream(setops_ctx *ctx) {
  return ctx ? static_cast<void *>(ctx->st) : nullptr;
}

int setops_gpu_synchronize(setops_ctx *ctx) {
  if (!ctx) return SETOPS_ERR_INVALID;
  CK(cudaStreamSynchronize(ctx->st));
  return ctx_check_device(ctx);
}

const char *setops_gpu_last_error(const setops_ctx *ctx) {
  return ctx ? ctx->err.c_str() : "no context";
}

int setops_gpu_num_variants(unsigned algo, int bsr) {
  if ((algo & SETOPS_ALGO_MASK) == SETOPS_ALGO_MERGE)
    return num_variants(ALGO_MERGE, bsr != 0);
  if ((algo & SETOPS_ALGO_MASK) == SETOPS_ALGO_GALLOP)
    return num_variants(ALGO_GALLOP, bsr != 0);
  if ((algo & SETOPS_ALGO_MASK) == SETOPS_ALGO_BITMAP)
    return num_variants(ALGO_BITMAP, bsr != 0);
  return 0;
}

uint64_t setops_gpu_launch_count(const setops_ctx *ctx) {
  return ctx ? ctx->launches : 0;
}

int setops_gpu_set_wait_limit_ns(setops_ctx *ctx, uint64_t ns) {
  if (!ctx) return SETOPS_ERR_INVALID;
  if (ns == 0) ns = kDefaultWaitLimitNs;
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->st));
  for (WaitLimitSetter fn : wait_limit_setters()) CK(fn(ns));
  CK(cudaDeviceSynchronize());
  return SETOPS_OK;
}

int setops_gpu_check_wait_limit(setops_ctx *ctx, uint64_t *waited_ns) {
  if (!ctx || !waited_ns) return SETOPS_ERR_INVALID;
  *waited_ns = 0;
  CK(cudaSetDevice(ctx->device));
  RK(ctx_status_words(ctx, 2));
  uint32_t epoch = 0;
  RK(ctx_next_epoch(ctx, &epoch));  // a fresh tag: no status word carries it
  uint64_t *status = static_cast<uint64_t *>(ctx->status.p);
  CK(launch_wait_check(status, epoch, ctx->derr, ctx->dlen, ctx->st));
  ++ctx->launches;
  CK(cudaMemcpyAsync(&ctx->hres[1], ctx->dlen, sizeof(uint64_t), cudaMemcpyDeviceToHost,
                     ctx->st));
  const int rc = ctx_check_device(ctx);  // synchronises; clears the error state
  *waited_ns = ctx->hres[1];
  return rc;
}

int setops_gpu_set_policy(setops_ctx *ctx, int bsr, int ratio_band,
                          unsigned algo_flags) {
  if (!ctx || ratio_band < 0 || ratio_band >= kRatioBands) return SETOPS_ERR_INVALID;
  const unsigned a = algo_flags & SETOPS_ALGO_MASK;
  if (a != SETOPS_ALGO_MERGE && a != SETOPS_ALGO_GALLOP && a != SETOPS_ALGO_BITMAP)
    return SETOPS_ERR_INVALID;
  const int v = int((algo_flags & SETOPS_VARIANT_MASK) >> SETOPS_VARIANT_SHIFT);
  const Algo al = a == SETOPS_ALGO_MERGE ? ALGO_MERGE : a == SETOPS_ALGO_GALLOP ? ALGO_GALLOP : ALGO_BITMAP;
  if (v >= num_variants(al, bsr != 0)) return SETOPS_ERR_INVALID;
  for (int c = 0; c < kSizeClasses; ++c)
    ctx->policy[bsr ? 1 : 0][ratio_band][c] = algo_flags & (SETOPS_ALGO_MASK | SETOPS_VARIANT_MASK);
  return SETOPS_OK;
}

int setops_gpu_set_policy_class(setops_ctx *ctx, int bsr, int ratio_band, int size_class,
                                unsigned algo_flags) {
  if (!ctx || size_class < 0 || size_class >= kSizeClasses) return SETOPS_ERR_INVALID;
  unsigned keep[kSizeClasses];
  std::memcpy(keep, ctx->policy[bsr ? 1 : 0][ratio_band < 0 ? 0 : ratio_band % kRatioBands],
              sizeof keep);
  RK(setops_gpu_set_policy(ctx, bsr, ratio_band, algo_flags));  // validates
  const unsigned f = ctx->policy[bsr ? 1 : 0][ratio_band][size_class];
  std::memcpy(ctx->policy[bsr ? 1 : 0][ratio_band], keep, sizeof keep);
  ctx->policy[bsr ? 1 : 0][ratio_band][size_class] = f;
  return SETOPS_OK;
}

int setops_gpu_get_policy_class(const setops_ctx *ctx, int bsr, int ratio_band, int size_class,
                                unsigned *algo_flags) {
  if (!ctx || !algo_flags || ratio_band < 0 || ratio_band >= kRatioBands || size_class < 0 ||
      size_class >= kSizeClasses)
    return SETOPS_ERR_INVALID;
  *algo_flags = ctx->policy[bsr ? 1 : 0][ratio_band][size_class];
  return SETOPS_OK;
}

int setops_gpu_get_policy(const setops_ctx *ctx, int bsr, int ratio_band,
                          unsigned *algo_flags) {
  if (!ctx || !algo_flags || ratio_band < 0 || ratio_band >= kRatioBands)
    return SETOPS_ERR_INVALID;
  *algo_flags = ctx->policy[bsr ? 1 : 0][ratio_band][kSizeClasses - 1];
  return SETOPS_OK;
}

// ---- 2-set arrays ----

// The device address of host memory the GPU can read in place (pinned by
// cudaHostAlloc or registered, so mapped into the device's address space),
// else nullptr (pageable memory).
static void *device_view(const void *h) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, h) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  return (at.type == cudaMemoryTypeHost) ? at.devicePointer : nullptr;
}

// Host inputs a search reads in place instead of copying them first.  On
// this machine the host link (NVLink-C2C) moves about 210 GB/s, by copy or by
// a kernel reading pinned memory, so a host-pointer call is bound by the
// bytes it moves: a search reads only the sectors its probes touch (2^10 to
// 2^18 elements against 2^24: 0.04-0.28 ms in place against 0.31-0.37 ms
// with the 64 MB larger set copied first), while a balanced pair reads both
// inputs whole and the window kernel streams host memory slower than a copy
// (0.89 against 0.66 ms for 2^24 x 2^24).  So: search-band pairs whose
// inputs are both device-readable host memory are read in place; everything
// else is copied.
static bool read_in_place(const Choice &c) { return c.algo == ALGO_GALLOP; }

static int intersect_impl(setops_ctx *ctx, const uint32_t *a, size_t na,
                          const uint32_t *b, size_t nb, uint32_t *out,
                          size_t out_cap, uint64_t *len_host,
                          uint64_t *len_dev_user, unsigned flags) {
  if (!ctx) return SETOPS_ERR_INVALID;
  if ((na && !a) || (nb && !b))
    return ctx_fail(ctx, SETOPS_ERR_INVALID, "NULL input with non-zero length");
  const bool host = (flags & SETOPS_HOST) != 0;
  const bool mat = out != nullptr;
  const uint64_t mn = std::min<uint64_t>(na, nb);
  if (mat && out_cap < mn)
    return ctx_fail(ctx, SETOPS_ERR_CAPACITY,
                    "out_cap " + std::to_string(out_cap) + " < min(na, nb) " +
                        std::to_string(mn));
  CK(cudaSetDevice(ctx->device));
  const uint32_t *da = a, *db = b;
  uint32_t *dout = out;
  Choice choice = ctx_choose(ctx, na, nb, false, flags);
  bool out_in_place = false;
  if (host) {
    if (len_dev_user) return ctx_fail(ctx, SETOPS_ERR_INVALID, "async call with host pointers");
    void *va = mn ? device_view(a) : nullptr, *vb = mn ? device_view(b) : nullptr;
    if (va && vb && read_in_place(choice)) {
      da = static_cast<const uint32_t *>(va);
      db = static_cast<const uint32_t *>(vb);
      // a search over host memory waits on the link for every probe round:
      // under the default policy the thread-per-element variants give way to
      // nine-way rounds with eight lanes per element (0.28 against 0.37 ms
      // for 2^18 against 2^24 in place)
      if ((flags & SETOPS_ALGO_MASK) == SETOPS_ALGO_AUTO && gallop_thread_per_element(choice.variant))
        choice.variant = kGallopNineWay;
    } else if (mn > 0) {
      RK(ctx_stage_in(ctx, 0, a, na, &da));
      RK(ctx_stage_in(ctx, 1, b, nb, &db));
    }
    if (mat) {
      void *vo = mn ? device_view(out) : nullptr;
      if (vo) {  // the kernel writes the result straight into host memory
        dout = static_cast<uint32_t *>(vo);
        out_in_place = true;
      } else {
        RK(buf_reserve(ctx, ctx->out0, std::max<uint64_t>(mn, 1) * 4));
        dout = static_cast<uint32_t *>(ctx->out0.p);
      }
    }
  }
  uint64_t *len_dev = len_dev_user ? len_dev_user : &ctx->dlen[0];
  if (mn == 0) {
    if (len_dev_user) {
      CK(cudaMemsetAsync(len_dev_user, 0, sizeof(uint64_t), ctx->st));
      return SETOPS_OK;
    }
    *len_host = 0;
    return SETOPS_OK;
  }
  PairJob j;
  j.a = da;
  j.b = db;
  j.na = na;
  j.nb = nb;
  j.out = mat ? dout : nullptr;
  j.out_cap = mat ? out_cap : 0;
  j.len_dev = len_dev;
  j.choice = choice;
  RK(ctx_launch_pair(ctx, j));
  if (len_dev_user) return SETOPS_OK;
  uint64_t n = 0;
  RK(ctx_read_u64(ctx, len_dev, &n));
  if (host && mat && n > 0 && !out_in_place) {
    CK(cudaMemcpyAsync(out, dout, n * 4, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
  }
  *len_host = n;
  return SETOPS_OK;
}

int setops_gpu_intersect_count(setops_ctx *ctx, const uint32_t *a, size_t na,
                               const uint32_t *b, size_t nb, uint64_t *count,
                               unsigned flags) {
  if (!count) return ctx_fail(ctx, SETOPS_ERR_INVALID, "count is NULL");
  return intersect_impl(ctx, a, na, b, nb, nullptr, 0, count, nullptr, flags);
}

int setops_gpu_intersect(setops_ctx *ctx, const uint32_t *a, size_t na,
                         const uint32_t *b, size_t nb, uint32_t *out,
                         size_t out_cap, size_t *out_len, unsigned flags) {
  if (!out_len || (!out && std::min(na, nb) > 0))
    return ctx_fail(ctx, SETOPS_ERR_INVALID, "out / out_len is NULL");
  uint64_t n = 0;
  uint32_t dummy = 0;
  int rc = intersect_impl(ctx, a, na, b, nb, out ? out : &dummy, out_cap, &n,
                          nullptr, flags);
  if (rc == SETOPS_OK) *out_len = size_t(n);
  return rc;
}

int setops_gpu_intersect_async(setops_ctx *ctx, const uint32_t *a, size_t na,
                               const uint32_t *b, size_t nb, uint32_t *out,
                               size_t out_cap, uint64_t *len_dev,
                               unsigned flags) {
  if (!len_dev) return ctx_fail(ctx, SETOPS_ERR_INVALID, "len_dev is NULL");
  if (flags & SETOPS_HOST)
    return ctx_fail(ctx, SETOPS_ERR_INVALID, "async call with host pointers");
  return intersect_impl(ctx, a, na, b, nb, out, out_cap, nullptr, len_dev,
                        flags);
}

// ---- many pairs with host inputs ----
//
// One call for npairs independent pairs in host memory, results to host
// memory, each result what setops_gpu_intersect gives for the pair.  A
// search-band pair whose inputs and output are device-readable (pinned)
// host memory is read in place (as in the one-pair call); here those pairs
// run on a second stream while the other pairs' inputs are copied over the
// host link, so the copies and the in-place searches overlap.  Kernels never
// overlap each other: the copied pairs' kernels wait for the in-place ones
// (two cooperative launches sharing the GPU could each wait for CTAs the
// other holds).  All scratch is reserved before any work is queued, so no
// buffer is reallocated while work is in flight.  Pairs with a pageable
// output take the one-pair call afterwards.

namespace {
enum PairKind { kEmpty = 0, kInPlace = 1, kCopied = 2, kOnePairCall = 3 };
constexpr int kCopySlots = 3;  // copied pairs whose inputs may be in flight at once
}  // namespace

int setops_gpu_intersect_pairs(setops_ctx *ctx, size_t npairs,
                               const uint32_t *const *a, const size_t *na,
                               const uint32_t *const *b, const size_t *nb,
                               uint32_t *const *out, const size_t *out_cap,
                               size_t *out_len, unsigned flags) {
  if (!ctx) return SETOPS_ERR_INVALID;
  if (npairs == 0) return SETOPS_OK;
  if (!a || !na || !b || !nb || !out || !out_cap || !out_len)
    return ctx_fail(ctx, SETOPS_ERR_INVALID, "NULL pair array");
  if (!(flags & SETOPS_HOST))
    return ctx_fail(ctx, SETOPS_ERR_INVALID,
                    "setops_gpu_intersect_pairs takes host pointers (SETOPS_HOST)");
  for (size_t i = 0; i < npairs; ++i) {
    const uint64_t mn = std::min<uint64_t>(na[i], nb[i]);
    if ((na[i] && !a[i]) || (nb[i] && !b[i]) || (mn && !out[i]))
      return ctx_fail(ctx, SETOPS_ERR_INVALID, "pair " + std::to_string(i) + ": NULL pointer");
    if (out_cap[i] < mn)
      return ctx_fail(ctx, SETOPS_ERR_CAPACITY,
                      "pair " + std::to_string(i) + ": out_cap " + std::to_string(out_cap[i]) +
                          " < min(na, nb) " + std::to_string(mn));
  }
  CK(cudaSetDevice(ctx->device));

  // ---- plan ----
  struct Plan {
    int kind = kEmpty;
    Choice c;
    const uint32_t *da = nullptr, *db = nullptr;
    uint32_t *dout = nullptr;
    int slot = 0;
  };
  std::vector<Plan> plan(npairs);
  uint64_t max_mn = 1, max_status = 1;
  uint64_t slot_a[kCopySlots] = {}, slot_b[kCopySlots] = {};
  int n_in_place = 0, n_copied = 0;
  for (size_t i = 0; i < npairs; ++i) {
    Plan &q = plan[i];
    const uint64_t mn = std::min<uint64_t>(na[i], nb[i]);
    if (mn == 0) continue;
    q.c = ctx_choose(ctx, na[i], nb[i], false, flags);
    void *vo = device_view(out[i]);
    void *va = device_view(a[i]), *vb = device_view(b[i]);
    if (!vo) {
      q.kind = kOnePairCall;
      continue;
    }
    q.dout = static_cast<uint32_t *>(vo);
    if (va && vb && read_in_place(q.c)) {
      q.kind = kInPlace;
      q.da = static_cast<const uint32_t *>(va);
      q.db = static_cast<const uint32_t *>(vb);
      if ((flags & SETOPS_ALGO_MASK) == SETOPS_ALGO_AUTO && gallop_thread_per_element(q.c.variant))
        q.c.variant = kGallopNineWay;
      ++n_in_place;
    } else {
      q.kind = kCopied;
      q.slot = n_copied % kCopySlots;
      slot_a[q.slot] = std::max<uint64_t>(slot_a[q.slot], na[i]);
      slot_b[q.slot] = std::max<uint64_t>(slot_b[q.slot], nb[i]);
      ++n_copied;
    }
    max_mn = std::max(max_mn, mn);
    // at least what any kernel's launch reserves: tiles of the pair plus
    // per-CTA words for a full grid (at most 64 CTAs per SM)
    max_status = std::max<uint64_t>(max_status,
                                    (na[i] + nb[i]) / 1024 + 2 + 2 * 64 * uint64_t(ctx->sms));
  }

  // ---- scratch, before anything is queued ----
  RK(buf_reserve(ctx, ctx->stage0, max_mn * 4));
  RK(ctx_status_words(ctx, max_status));
  RK(buf_reserve(ctx, ctx->plen, npairs * sizeof(uint64_t)));
  for (int s = 0; s < kCopySlots; ++s) {
    if (slot_a[s]) RK(buf_reserve(ctx, ctx->in[2 * s], slot_a[s] * 4));
    if (slot_b[s]) RK(buf_reserve(ctx, ctx->in[2 * s + 1], slot_b[s] * 4));
  }
  if (ctx->hlens_cap < npairs) {
    if (ctx->hlens) {
      CK(cudaStreamSynchronize(ctx->st));
      CK(cudaFreeHost(ctx->hlens));
      ctx->hlens = nullptr;
      ctx->hlens_cap = 0;
    }
    const size_t want = std::max<size_t>(npairs, 64);
    CK(cudaMallocHost(&ctx->hlens, want * sizeof(uint64_t)));
    ctx->hlens_cap = want;
  }
  if (!ctx->aux) {
    CK(cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&ctx->ev_main, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ctx->ev_aux, cudaEventDisableTiming));
  }
  uint64_t *plen = static_cast<uint64_t *>(ctx->plen.p);
  const cudaStream_t main_st = ctx->st;
  auto job = [&](size_t i, const uint32_t *da, const uint32_t *db) {
    PairJob j;
    j.a = da;
    j.b = db;
    j.na = na[i];
    j.nb = nb[i];
    j.out = plan[i].dout;
    j.out_cap = out_cap[i];
    j.len_dev = plen + i;
    j.choice = plan[i].c;
    return j;
  };

  // ---- in-place pairs on the second stream (after the main stream's queued work) ----
  int rc = SETOPS_OK;
  CK(cudaEventRecord(ctx->ev_main, main_st));
  CK(cudaStreamWaitEvent(ctx->aux, ctx->ev_main, 0));
  if (n_in_place) {
    ctx->st = ctx->aux;  // launches, and their epoch clears, go to the second stream
    for (size_t i = 0; i < npairs && rc == SETOPS_OK; ++i)
      if (plan[i].kind == kInPlace) rc = ctx_launch_pair(ctx, job(i, plan[i].da, plan[i].db));
    ctx->st = main_st;
  }
  if (rc == SETOPS_OK) {
    const cudaError_t e = cudaEventRecord(ctx->ev_aux, ctx->aux);
    if (e != cudaSuccess) rc = ctx_cuda(ctx, e, "cudaEventRecord");
  }

  // ---- copied pairs on the main stream: the first kCopySlots pairs' copies
  // start at once; every kernel waits for the in-place pairs ----
  std::vector<size_t> copied;
  for (size_t i = 0; i < npairs; ++i)
    if (plan[i].kind == kCopied) copied.push_back(i);
  auto copy_in = [&](size_t i) -> int {
    const int s = plan[i].slot;
    CK(cudaMemcpyAsync(ctx->in[2 * s].p, a[i], na[i] * 4, cudaMemcpyHostToDevice, main_st));
    CK(cudaMemcpyAsync(ctx->in[2 * s + 1].p, b[i], nb[i] * 4, cudaMemcpyHostToDevice, main_st));
    return SETOPS_OK;
  };
  for (size_t k = 0; k < copied.size() && k < size_t(kCopySlots) && rc == SETOPS_OK; ++k)
    rc = copy_in(copied[k]);
  if (rc == SETOPS_OK) {
    const cudaError_t e = cudaStreamWaitEvent(main_st, ctx->ev_aux, 0);
    if (e != cudaSuccess) rc = ctx_cuda(ctx, e, "cudaStreamWaitEvent");
  }
  for (size_t k = 0; k < copied.size() && rc == SETOPS_OK; ++k) {
    const size_t i = copied[k];
    // a slot is refilled only after the kernel that read it (stream order)
    if (k >= size_t(kCopySlots)) rc = copy_in(i);
    if (rc != SETOPS_OK) break;
    const int s = plan[i].slot;
    rc = ctx_launch_pair(ctx, job(i, static_cast<const uint32_t *>(ctx->in[2 * s].p),
                                  static_cast<const uint32_t *>(ctx->in[2 * s + 1].p)));
  }
  if (rc != SETOPS_OK) {
    cudaStreamSynchronize(ctx->aux);
    cudaStreamSynchronize(main_st);
    return rc;
  }

  // ---- every length in one copy; the main stream has waited for the second ----
  if (n_in_place + n_copied > 0)
    CK(cudaMemcpyAsync(ctx->hlens, plen, npairs * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                       main_st));
  RK(ctx_check_device(ctx));  // synchronises the main stream, reads the error word
  for (size_t i = 0; i < npairs; ++i) {
    if (plan[i].kind == kEmpty) out_len[i] = 0;
    else if (plan[i].kind != kOnePairCall) out_len[i] = size_t(ctx->hlens[i]);
  }
  // pairs with a pageable output: one call each
  for (size_t i = 0; i < npairs; ++i)
    if (plan[i].kind == kOnePairCall)
      RK(setops_gpu_intersect(ctx, a[i], na[i], b[i], nb[i], out[i], out_cap[i], &out_len[i],
                              flags));
  return SETOPS_OK;
}

// ---- 2-set BSR ----

static int bsr_impl(setops_ctx *ctx, const uint32_t *ba, const uint32_t *sa,
                    size_t na, const uint32_t *bb, const uint32_t *sb,
                    size_t nb, uint32_t *ob, uint32_t *os, size_t out_cap,
                    uint64_t *len_host, unsigned flags) {
  if (!ctx) return SETOPS_ERR_INVALID;
  if ((na && (!ba || !sa)) || (nb && (!bb || !sb)))
    return ctx_fail(ctx, SETOPS_ERR_INVALID, "NULL input with non-zero length");
  const bool host = (flags & SETOPS_HOST) != 0;
  const bool mat = ob != nullptr;
  const uint64_t mn = std::min<uint64_t>(na, nb);
  if (mat && out_cap < mn)
    return ctx_fail(ctx, SETOPS_ERR_CAPACITY, "out_cap < min(na, nb)");
  if (mn == 0) {
    *len_host = 0;
    return SETOPS_OK;
  }
  CK(cudaSetDevice(ctx->device));
  const uint32_t *dba = ba, *dsa = sa, *dbb = bb, *dsb = sb;
  uint32_t *dob = ob, *dos = os;
  if (host) {
    RK(ctx_stage_in(ctx, 0, ba, na, &dba));
    RK(ctx_stage_in(ctx, 1, bb, nb, &dbb));
    RK(ctx_stage_in(ctx, 2, sa, na, &dsa));
    RK(ctx_stage_in(ctx, 3, sb, nb, &dsb));
    if (mat) {
      RK(buf_reserve(ctx, ctx->out0, mn * 4));
      RK(buf_reserve(ctx, ctx->out1, mn * 4));
      dob = static_cast<uint32_t *>(ctx->out0.p);
      dos = static_cast<uint32_t *>(ctx->out1.p);
    }
  }
  PairJob j;
  j.a = dba;
  j.b = dbb;
  j.sa = dsa;
  j.sb = dsb;
  j.na = na;
  j.nb = nb;
  j.bsr = true;
  j.out = mat ? dob : nullptr;
  j.out_s = mat ? dos : nullptr;
  j.out_cap = mat ? out_cap : 0;
  j.len_dev = &ctx->dlen[0];
  j.choice = ctx_choose(ctx, na, nb, true, flags);
  RK(ctx_launch_pair(ctx, j));
  uint64_t n = 0;
  RK(ctx_read_u64(ctx, j.len_dev, &n));
  if (host && mat && n > 0) {
    CK(cudaMemcpyAsync(ob, dob, n * 4, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(os, dos, n * 4, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
  }
  *len_host = n;
  return SETOPS_OK;
}

int setops_gpu_intersect_bsr_count(setops_ctx *ctx, const uint32_t *bases_a,
                                   const uint32_t *states_a, size_t na,
                                   const uint32_t *bases_b,
                                   const uint32_t *states_b, size_t nb,
                                   uint64_t *count, unsigned flags) {
  if (!count) return ctx_fail(ctx, SETOPS_ERR_INVALID, "count is NULL");
  return bsr_impl(ctx, bases_a, states_a, na, bases_b, states_b, nb, nullptr,
                  nullptr, 0, count, flags);
}

int setops_gpu_intersect_bsr(setops_ctx *ctx, const uint32_t *bases_a,
                             const uint32_t *states_a, size_t na,
                             const uint32_t *bases_b, const uint32_t *states_b,
                             size_t nb, uint32_t *out_bases,
                             uint32_t *out_states, size_t out_cap,
                             size_t *out_len, unsigned flags) {
  if (!out_len) return ctx_fail(ctx, SETOPS_ERR_INVALID, "out_len is NULL");
  if (std::min(na, nb) > 0 && (!out_bases || !out_states))
    return ctx_fail(ctx, SETOPS_ERR_INVALID, "output arrays are NULL");
  uint32_t dummy[2];
  uint64_t n = 0;
  int rc = bsr_impl(ctx, bases_a, states_a, na, bases_b, states_b, nb,
                    out_bases ? out_bases : &dummy[0],
                    out_states ? out_states : &dummy[1], out_cap, &n, flags);
  if (rc == SETOPS_OK) *out_len = size_t(n);
  return rc;
}

int setops_gpu_bsr_from_sorted(setops_ctx *ctx, const uint32_t *in, size_t n,
                               uint32_t *bases, uint32_t *states,
                               size_t *nwords, unsigned flags) {
  if (!ctx || !nwords || (n && (!in || !bases || !states)))
    return ctx_fail(ctx, SETOPS_ERR_INVALID, "NULL argument");
  if (n == 0) {
    *nwords = 0;
    return SETOPS_OK;
  }
  CK(cudaSetDevice(ctx->device));
  const bool host = (flags & SETOPS_HOST) != 0;
  const uint32_t *din = in;
  uint32_t *dbs = bases, *dst = states;
  if (host) {
    RK(ctx_stage_in(ctx, 0, in, n, &din));
    RK(buf_reserve(ctx, ctx->out0, n * 4));
    RK(buf_reserve(ctx, ctx->out1, n * 4));
    dbs = static_cast<uint32_t *>(ctx->out0.p);
    dst = static_cast<uint32_t *>(ctx->out1.p);
  }
  const uint64_t ntiles = (n + kBsrEncodeTile - 1) / kBsrEncodeTile;
  int occ = 1;
  RK(ctx_occupancy(ctx, KernelInfo{bsr_encode_fn(), kUtilThreads, 0, kBsrEncodeTile, "bsr_encode"}, &occ));
  const uint64_t grid = std::max<uint64_t>(1, std::min<uint64_t>(ntiles, uint64_t(occ) * ctx->sms));
  RK(ctx_status_words(ctx, ntiles));
  uint32_t epoch;
  RK(ctx_next_epoch(ctx, &epoch));
  CK(launch_bsr_encode(din, n, dbs, dst, &ctx->dlen[0],
                       static_cast<uint64_t *>(ctx->status.p), ctx->sync,
                       ctx->derr, epoch, int(grid), ctx->st));
  ctx->launches++;
  uint64_t w = 0;
  RK(ctx_read_u64(ctx, &ctx->dlen[0], &w));
  if (host && w) {
    CK(cudaMemcpyAsync(bases, dbs, w * 4, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(states, dst, w * 4, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
  }
  *nwords = size_t(w);
  return SETOPS_OK;
}

int setops_gpu_bsr_to_sorted(setops_ctx *ctx, const uint32_t *bases,
                             const uint32_t *states, size_t n, uint32_t *out,
                             size_t out_cap, size_t *out_len, unsigned flags) {
  if (!ctx || !out_len || (n && (!bases || !states || !out)))
    return ctx_fail(ctx, SETOPS_ERR_INVALID, "NULL argument");
  if (n == 0) {
    *out_len = 0;
    return SETOPS_OK;
  }
  CK(cudaSetDevice(ctx->device));
  const bool host = (flags & SETOPS_HOST) != 0;
  const uint32_t *dbs = bases, *dst = states;
  uint32_t *dout = out;
  if (host) {
    RK(ctx_stage_in(ctx, 0, bases, n, &dbs));
    RK(ctx_stage_in(ctx, 1, states, n, &dst));
    RK(buf_reserve(ctx, ctx->out0, std::max<size_t>(out_cap, 1) * 4));
    dout = static_cast<uint32_t *>(ctx->out0.p);
  }
  const uint64_t ntiles = (n + kBsrDecodeTile - 1) / kBsrDecodeTile;
  int occ = 1;
  RK(ctx_occupancy(ctx, KernelInfo{bsr_decode_fn(), kUtilThreads, 0, kBsrDecodeTile, "bsr_decode"}, &occ));
  const uint64_t grid = std::max<uint64_t>(1, std::min<uint64_t>(ntiles, uint64_t(occ) * ctx->sms));
  RK(ctx_status_words(ctx, ntiles));
  uint32_t epoch;
  RK(ctx_next_epoch(ctx, &epoch));
  CK(launch_bsr_decode(dbs, dst, n, dout, out_cap, &ctx->dlen[0],
                       static_cast<uint64_t *>(ctx->status.p), ctx->sync,
                       ctx->derr, epoch, int(grid), ctx->st));
  ctx->launches++;
  uint64_t m = 0;
  RK(ctx_read_u64(ctx, &ctx->dlen[0], &m));
  if (host && m) {
    CK(cudaMemcpyAsync(out, dout, m * 4, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
  }
  *out_len = size_t(m);
  return SETOPS_OK;
}

// ---- k-set SvS ----

// len_dev != NULL: asynchronous form (device arrays only): the result length
// goes to the device word *len_dev and nothing waits for the GPU.
static int svs_impl(setops_ctx *ctx, const uint32_t *const *sets,
                    const size_t *lens, size_t k, uint32_t *out,
                    size_t out_cap, uint64_t *len_host, unsigned flags,
                    uint64_t *len_dev = nullptr) {
  if (!ctx) return SETOPS_ERR_INVALID;
  if (!sets || !lens || k < 2)
    return ctx_fail(ctx, SETOPS_ERR_INVALID, "svs needs k >= 2 sets");
  for (size_t i = 0; i < k; ++i)
    if (lens[i] && !sets[i])
      return ctx_fail(ctx, SETOPS_ERR_INVALID, "NULL set with non-zero length");
  if (k > kLenWords - 2)
    return ctx_fail(ctx, SETOPS_ERR_TOO_LARGE,
                    "svs supports up to " + std::to_string(kLenWords - 2) + " sets");
  const bool host = (flags & SETOPS_HOST) != 0;
  const bool mat = out != nullptr;
  std::vector<size_t> order(k);
  std::iota(order.begin(), order.end(), size_t(0));
  std::stable_sort(order.begin(), order.end(),
                   [&](size_t x, size_t y) { return lens[x] < lens[y]; });
  const uint64_t mn = lens[order[0]];
  if (mat && out_cap < mn)
    return ctx_fail(ctx, SETOPS_ERR_CAPACITY, "out_cap < smallest set");
  if (len_dev && host)
    return ctx_fail(ctx, SETOPS_ERR_INVALID, "the asynchronous k-set call takes device arrays");
  if (mn == 0) {
    if (len_dev) {
      CK(cudaSetDevice(ctx->device));
      CK(cudaMemsetAsync(len_dev, 0, sizeof(uint64_t), ctx->st));
    } else {
      *len_host = 0;
    }
    return SETOPS_OK;
  }
  CK(cudaSetDevice(ctx->device));
  std::vector<const uint32_t *> d(k);
  if (host) {
    size_t total = 0;
    for (size_t i = 0; i < k; ++i) total += lens[i];
    RK(buf_reserve(ctx, ctx->in[4], total * 4));
    size_t off = 0;
    for (size_t i = 0; i < k; ++i) {
      uint32_t *dst = static_cast<uint32_t *>(ctx->in[4].p) + off;
      if (lens[i])
        CK(cudaMemcpyAsync(dst, sets[i], lens[i] * 4, cudaMemcpyHostToDevice,
                           ctx->st));
      d[i] = dst;
      off += lens[i];
    }
  } else {
    for (size_t i = 0; i < k; ++i) d[i] = sets[i];
  }
  uint32_t *final_out = out;
  if (host && mat) {
    RK(buf_reserve(ctx, ctx->out0, mn * 4));
    final_out = static_cast<uint32_t *>(ctx->out0.p);
  }
  uint64_t *lens_dev0 = &ctx->dlen[2];
  // k >= 3 sets of sizes within 16x of the smallest: one fused launch reads
  // every set once and keeps the survivors in shared memory (kset.cuh)
  if ((flags & SETOPS_ALGO_MASK) == SETOPS_ALGO_AUTO && k >= 3 && k <= size_t(kKsetMax) &&
      lens[order[k - 1]] / mn < 16) {
    const KernelInfo &kk = kset_kernel(mat);
    int occ = 1;
    RK(ctx_occupancy(ctx, kk, &occ));
    // a CTA per two tiles' worth of all the sets (not of the smallest alone:
    // each CTA's chain of windows through the other sets stays short)
    uint64_t total = 0;
    for (size_t i = 0; i < k; ++i) total += lens[i];
    const uint64_t ntiles = (total + 2 * uint64_t(kk.tile) - 1) / (2 * uint64_t(kk.tile));
    const uint64_t grid = std::max<uint64_t>(1, std::min<uint64_t>(uint64_t(occ) * ctx->sms, ntiles));
    RK(ctx_status_words(ctx, grid));
    KsetArgs a{};
    for (size_t i = 0; i < k; ++i) {
      a.sets[i] = d[order[i]];
      a.lens[i] = lens[order[i]];
    }
    a.k = int(k);
    if (mat) {
      RK(buf_reserve(ctx, ctx->stage0, mn * 4));
      a.stage = static_cast<uint32_t *>(ctx->stage0.p);
      a.out = final_out;
      a.out_cap = out_cap;
    }
    a.out_len = len_dev ? len_dev : lens_dev0;
    a.coranks = static_cast<uint64_t *>(ctx->status.p);
    a.sync = ctx->sync;
    a.err = ctx->derr;
    void *args[] = {&a};
    RK(ctx_launch(ctx, kk, grid, args));
    ++ctx->launches;
    if (len_dev) return SETOPS_OK;  // errors surface at the next synchronising call
    uint64_t n = 0;
    RK(ctx_read_u64(ctx, lens_dev0, &n));  // (also reports device-side errors)
    if (host && mat && n > 0) {
      CK(cudaMemcpyAsync(out, final_out, n * 4, cudaMemcpyDeviceToHost, ctx->st));
      CK(cudaStreamSynchronize(ctx->st));
    }
    *len_host = n;
    return SETOPS_OK;
  }
  RK(buf_reserve(ctx, ctx->inter[0], mn * 4));
  RK(buf_reserve(ctx, ctx->inter[1], mn * 4));
  uint32_t *inter[2] = {static_cast<uint32_t *>(ctx->inter[0].p),
                        static_cast<uint32_t *>(ctx->inter[1].p)};
  uint64_t *lens_dev = &ctx->dlen[2];
  const uint32_t thr = ctx_search_threshold(ctx, false);
  // step 0: the two smallest sets (lengths known on the host)
  uint64_t ub = mn;
  {
    PairJob j;
    j.a = d[order[0]];
    j.na = lens[order[0]];
    j.b = d[order[1]];
    j.nb = lens[order[1]];
    const bool last = (k == 2);
    j.out = last ? (mat ? final_out : nullptr) : inter[0];
    j.out_cap = last ? (mat ? out_cap : 0) : mn;
    j.len_dev = &lens_dev[0];
    j.choice = ctx_choose(ctx, j.na, j.nb, false, flags);
    RK(ctx_launch_pair(ctx, j));
  }
  for (size_t s = 1; s + 1 < k; ++s) {
    const bool last = (s + 2 == k);
    const uint64_t nb = lens[order[s + 1]];
    PairJob j;
    j.a = inter[(s - 1) & 1];
    j.na = ub;
    j.na_dev = &lens_dev[s - 1];
    j.b = d[order[s + 1]];
    j.nb = nb;
    j.out = last ? (mat ? final_out : nullptr) : inter[s & 1];
    j.out_cap = last ? (mat ? out_cap : 0) : mn;
    j.len_dev = &lens_dev[s];
    if ((flags & SETOPS_ALGO_MASK) != SETOPS_ALGO_AUTO) {
      j.choice = ctx_choose(ctx, ub, nb, false, flags);
      RK(ctx_launch_pair(ctx, j));
    } else {
      // The intermediate length is only known on the device: launch both
      // kernels; each checks the actual length ratio and only one runs.
      j.ratio_thr = thr;
      j.skip_rule = 2;
      j.choice.algo = ALGO_BITMAP;  // tiles, coarse bitmaps for sparse ones
      j.choice.variant = kCoarseBitmap;
      RK(ctx_launch_pair(ctx, j));
      j.skip_rule = 1;
      j.choice.algo = ALGO_GALLOP;
      int band = 0;
      while (band < kRatioBands - 1 && (1u << band) < thr) ++band;
      const unsigned pol = ctx->policy[0][band][size_class(ub)];
      j.choice.variant = int((pol & SETOPS_VARIANT_MASK) >> SETOPS_VARIANT_SHIFT);
      if ((pol & SETOPS_ALGO_MASK) != SETOPS_ALGO_GALLOP) j.choice.variant = 0;
      RK(ctx_launch_pair(ctx, j));
    }
    ub = std::min(ub, nb);
  }
  if (len_dev) {
    CK(cudaMemcpyAsync(len_dev, &lens_dev[k - 2], sizeof(uint64_t), cudaMemcpyDeviceToDevice,
                       ctx->st));
    return SETOPS_OK;
  }
  uint64_t n = 0;
  RK(ctx_read_u64(ctx, &lens_dev[k - 2], &n));
  if (host && mat && n > 0) {
    CK(cudaMemcpyAsync(out, final_out, n * 4, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
  }
  *len_host = n;
  return SETOPS_OK;
}

int setops_gpu_svs(setops_ctx *ctx, const uint32_t *const *sets,
                   const size_t *lens, size_t k, uint32_t *out,
                   size_t out_cap, size_t *out_len, unsigned flags) {
  if (!out_len) return ctx_fail(ctx, SETOPS_ERR_INVALID, "out_len is NULL");
  uint32_t dummy = 0;
  uint64_t n = 0;
  int rc = svs_impl(ctx, sets, lens, k, out ? out : &dummy, out ? out_cap : 0,
                    &n, flags);
  if (rc == SETOPS_OK) *out_len = size_t(n);
  return rc;
}

int setops_gpu_svs_async(setops_ctx *ctx, const uint32_t *const *sets,
                         const size_t *lens, size_t k, uint32_t *out,
                         size_t out_cap, uint64_t *len_dev, unsigned flags) {
  if (!len_dev) return ctx_fail(ctx, SETOPS_ERR_INVALID, "len_dev is NULL");
  return svs_impl(ctx, sets, lens, k, out, out_cap, nullptr, flags, len_dev);  // out NULL: count
}

int setops_gpu_svs_count(setops_ctx *ctx, const uint32_t *const *sets,
                         const size_t *lens, size_t k, uint64_t *count,
                         unsigned flags) {
  if (!count) return ctx_fail(ctx, SETOPS_ERR_INVALID, "count is NULL");
  return svs_impl(ctx, sets, lens, k, nullptr, 0, count, flags);
}

int setops_gpu_validate_sorted(setops_ctx *ctx, const uint32_t *a, size_t n,
                               int *is_sorted, unsigned flags) {
  if (!ctx || !is_sorted || (n && !a))
    return ctx_fail(ctx, SETOPS_ERR_INVALID, "NULL argument");
  if (n < 2) {
    *is_sorted = 1;
    return SETOPS_OK;
  }
  CK(cudaSetDevice(ctx->device));
  const uint32_t *da = a;
  if (flags & SETOPS_HOST) RK(ctx_stage_in(ctx, 0, a, n, &da));
  CK(cudaMemsetAsync(ctx->dflag, 0, sizeof(int), ctx->st));
  CK(launch_validate_sorted(da, n, ctx->dflag, ctx->sms, ctx->st));
  ctx->launches++;
  CK(cudaMemcpyAsync(&ctx->hres[1], ctx->dflag, sizeof(int),
                     cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  int bad = 0;
  std::memcpy(&bad, &ctx->hres[1], sizeof(int));
  *is_sorted = bad ? 0 : 1;
  return SETOPS_OK;
}

}  // extern "C"
