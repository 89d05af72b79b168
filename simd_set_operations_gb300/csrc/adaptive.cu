// adaptive.cu -- C ABI of the k-set small_adaptive path (include/setops_gpu.h):
// setops_gpu_adaptive / setops_gpu_adaptive_count.  Kernel: adaptive.cuh.
#include <algorithm>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/setops_gpu.h"
#include "adaptive.cuh"
#include "runtime.h"

using namespace setops;

#define CK(call)                                            \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return ctx_cuda(ctx, e_, #call); \
  } while (0)
#define RK(call)                    \
  do {                              \
    int r_ = (call);                \
    if (r_ != SETOPS_OK) return r_; \
  } while (0)

namespace {

constexpr int kNT = 256, kIT = 4;  // tiles of 1,024 probe-set elements

const KernelInfo &adaptive_info() {
  static const KernelInfo k{reinterpret_cast<const void *>(&adaptive_kernel<kNT, kIT>), kNT, 0,
                            AdaptiveCfg<kNT, kIT>::kTile, "adaptive_256_i4", false};
  return k;
}

int adaptive_impl(setops_ctx *ctx, const uint32_t *const *sets, const size_t *lens, size_t k,
                  uint32_t *out, size_t out_cap, uint64_t *len_host, unsigned flags) {
  if (!ctx) return SETOPS_ERR_INVALID;
  if (!sets || !lens || k < 2)
    return ctx_fail(ctx, SETOPS_ERR_INVALID, "small_adaptive needs k >= 2 sets");
  if (k > size_t(kKsetMax))
    return ctx_fail(ctx, SETOPS_ERR_TOO_LARGE,
                    "small_adaptive supports up to " + std::to_string(kKsetMax) + " sets");
  for (size_t i = 0; i < k; ++i)
    if (lens[i] && !sets[i])
      return ctx_fail(ctx, SETOPS_ERR_INVALID, "NULL set with non-zero length");
  const bool host = (flags & SETOPS_HOST) != 0;
  const bool mat = out != nullptr;
  // the probe set is the smallest; the others are searched smallest first
  std::vector<size_t> order(k);
  std::iota(order.begin(), order.end(), size_t(0));
  std::stable_sort(order.begin(), order.end(),
                   [&](size_t x, size_t y) { return lens[x] < lens[y]; });
  const uint64_t mn = lens[order[0]];
  if (mat && out_cap < mn) return ctx_fail(ctx, SETOPS_ERR_CAPACITY, "out_cap < smallest set");
  if (mn == 0) {
    *len_host = 0;
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
      if (lens[i]) CK(cudaMemcpyAsync(dst, sets[i], lens[i] * 4, cudaMemcpyHostToDevice, ctx->st));
      d[i] = dst;
      off += lens[i];
    }
  } else {
    for (size_t i = 0; i < k; ++i) d[i] = sets[i];
  }
  uint32_t *dout = out;
  if (host && mat) {
    RK(buf_reserve(ctx, ctx->out0, mn * 4));
    dout = static_cast<uint32_t *>(ctx->out0.p);
  }
  const KernelInfo &ki = adaptive_info();
  int occ = 1;
  RK(ctx_occupancy(ctx, ki, &occ));
  const uint64_t ntiles = (mn + ki.tile - 1) / ki.tile;
  const uint64_t grid = std::max<uint64_t>(1, std::min<uint64_t>(uint64_t(occ) * ctx->sms, ntiles));
  RK(ctx_status_words(ctx, ntiles));
  uint32_t epoch = 0;
  RK(ctx_next_epoch(ctx, &epoch));
  AdaptiveArgs a{};
  for (size_t i = 0; i < k; ++i) {
    a.sets[i] = d[order[i]];
    a.lens[i] = lens[order[i]];
  }
  a.k = int(k);
  a.out = mat ? dout : nullptr;
  a.out_cap = mat ? out_cap : 0;
  a.out_len = &ctx->dlen[0];
  a.status = static_cast<uint64_t *>(ctx->status.p);
  a.sync = ctx->sync;
  a.err = ctx->derr;
  a.epoch = epoch;
  void *args[] = {&a};
  RK(ctx_launch(ctx, ki, grid, args));
  ctx->launches++;
  uint64_t n = 0;
  RK(ctx_read_u64(ctx, &ctx->dlen[0], &n));
  if (host && mat && n > 0) {
    CK(cudaMemcpyAsync(out, dout, n * 4, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
  }
  *len_host = n;
  return SETOPS_OK;
}

}  // namespace

extern "C" {

int setops_gpu_adaptive(setops_ctx *ctx, const uint32_t *const *sets, const size_t *lens,
                        size_t k, uint32_t *out, size_t out_cap, size_t *out_len,
                        unsigned flags) {
  if (!out_len) return ctx_fail(ctx, SETOPS_ERR_INVALID, "out_len is NULL");
  uint64_t n = 0;
  uint32_t dummy = 0;
  const int rc = adaptive_impl(ctx, sets, lens, k, out ? out : &dummy, out_cap, &n, flags);
  if (rc == SETOPS_OK) *out_len = size_t(n);
  return rc;
}

int setops_gpu_adaptive_count(setops_ctx *ctx, const uint32_t *const *sets, const size_t *lens,
                              size_t k, uint64_t *count, unsigned flags) {
  if (!count) return ctx_fail(ctx, SETOPS_ERR_INVALID, "count is NULL");
  return adaptive_impl(ctx, sets, lens, k, nullptr, 0, count, flags);
}

}  // extern "C"
