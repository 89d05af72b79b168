// batch.cu -- C ABI of the batched intersection (many pairs, one launch),
// its policy and its autotuner.  Kernels: batch.cuh.
#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "batch.cuh"
#include "runtime.h"
#include "setops_gpu.h"

using namespace setops;

namespace {

#define CK(call)                                                     \
  do {                                                               \
    cudaError_t e_ = (call);                                         \
    if (e_ != cudaSuccess) return ctx_cuda(ctx, e_, #call);          \
  } while (0)
#define RK(call)                    \
  do {                              \
    int r_ = (call);                \
    if (r_ != SETOPS_OK) return r_; \
  } while (0)

template <int NT, int TA, int VW, int MINB, bool MAT>
KernelInfo mk_batch(const char *name) {
  using Cfg = TileCfg<NT, TA, VW, MAT>;
  return KernelInfo{reinterpret_cast<const void *>(&batch_kernel<NT, TA, VW, MINB, MAT>), NT,
                    Cfg::kSmemBytes, TA, name, false};
}
#define BATCH_ROW(NT, TA, VW, MINB)                                                 \
  {mk_batch<NT, TA, VW, MINB, false>("batch_" #NT "_a" #TA "_t" #VW "_b" #MINB),     \
   mk_batch<NT, TA, VW, MINB, true>("batch_" #NT "_a" #TA "_t" #VW "_b" #MINB)}
// NT threads; A tiles of TA elements; T of VW words; MINB CTAs/SM
const KernelInfo kBatchU32[][2] = {
    BATCH_ROW(256, 4096, 4096, 8),  // 0: 8 warps, 4096-element tiles
    BATCH_ROW(128, 2048, 2048, 8),  // 1: 4 warps, smaller tiles (many small pairs)
    BATCH_ROW(256, 2048, 2048, 8),  // 2: 8 warps, smaller tiles
};
constexpr int kNumBatch = int(sizeof(kBatchU32) / sizeof(kBatchU32[0]));

// Copies n host words of T into buffer b; returns the device pointer.
template <class T>
int stage(setops_ctx *ctx, DevBuf &b, const T *h, size_t n, const T **d) {
  RK(buf_reserve(ctx, b, std::max<size_t>(n, 1) * sizeof(T)));
  if (n) CK(cudaMemcpyAsync(b.p, h, n * sizeof(T), cudaMemcpyHostToDevice, ctx->st));
  *d = static_cast<const T *>(b.p);
  return SETOPS_OK;
}

struct BatchDev {
  const uint32_t *pool;
  const uint64_t *a_off, *a_len, *b_off, *b_len;
};

// One batched launch on device arrays.  unit_cap > 0: long pairs are split
// over CTAs (room for unit_cap units; more: no splitting).
int launch_batch(setops_ctx *ctx, const BatchDev &d, uint64_t npairs, uint32_t *out,
                 const uint64_t *out_off, uint64_t *out_lens, int variant, uint32_t ratio,
                 uint64_t unit_cap = 0) {
  const KernelInfo &k = kBatchU32[variant][out ? 1 : 0];
  int occ = 1;
  RK(ctx_occupancy(ctx, k, &occ));
  if (unit_cap) unit_cap = std::max<uint64_t>(unit_cap, npairs);
  const uint64_t work = std::max<uint64_t>(npairs, unit_cap);  // tickets, at most
  const uint64_t grid = std::max<uint64_t>(1, std::min<uint64_t>(uint64_t(occ) * ctx->sms, work));
  BatchArgs a{};
  a.pool = d.pool;
  a.a_off = d.a_off;
  a.a_len = d.a_len;
  a.b_off = d.b_off;
  a.b_len = d.b_len;
  a.npairs = npairs;
  a.out_off = out_off;
  a.out = out;
  a.out_lens = out_lens;
  a.search_ratio = ratio;
  a.sync = ctx->sync + 1;  // its own coordination slot
  a.err = ctx->derr;
  if (unit_cap) {
    RK(buf_reserve(ctx, ctx->units, prefix_bytes(npairs, unit_cap)));
    launch_prefix(d.a_len, d.b_len, npairs, ctx->units.p, nullptr, nullptr, unit_cap, &a, ctx->st);
    CK(cudaGetLastError());
    ctx->launches += 2;
  }
  void *args[] = {&a};
  return ctx_launch(ctx, k, grid, args);
}

// Shared body of the batch entry points.  out == NULL: count mode (per-pair
// counts to out_lens).
int batch_impl(setops_ctx *ctx, const uint32_t *pool, size_t pool_len, const uint64_t *a_off,
               const uint64_t *a_len, const uint64_t *b_off, const uint64_t *b_len,
               size_t npairs, uint32_t *out, size_t out_cap, const uint64_t *out_off,
               uint64_t *out_lens, unsigned flags) {
  if (!ctx) return SETOPS_ERR_INVALID;
  if (npairs == 0) return SETOPS_OK;
  if (!pool || !a_off || !a_len || !b_off || !b_len || !out_lens)
    return ctx_fail(ctx, SETOPS_ERR_INVALID, "NULL batch array");
  const bool host = (flags & SETOPS_HOST) != 0;
  const bool mat = out != nullptr;
  const int v = ctx->batch_variant;  // shape and search ratio: the batch policy
  CK(cudaSetDevice(ctx->device));
  BatchDev d{pool, a_off, a_len, b_off, b_len};
  const uint64_t *doff = out_off;
  uint64_t *dlens = out_lens;
  uint32_t *dout = out;
  uint64_t need = 0;  // output words the pairs need (materialise, computed offsets)
  if (host) {
    // the caller's lengths are on the host: offsets and capacity are known here
    RK(stage(ctx, ctx->in[0], pool, pool_len, &d.pool));
    RK(stage(ctx, ctx->in[1], a_off, npairs, &d.a_off));
    RK(stage(ctx, ctx->in[2], a_len, npairs, &d.a_len));
    RK(stage(ctx, ctx->in[3], b_off, npairs, &d.b_off));
    RK(stage(ctx, ctx->in[4], b_len, npairs, &d.b_len));
    for (size_t p = 0; p < npairs; ++p) {
      if (a_off[p] + a_len[p] > pool_len || b_off[p] + b_len[p] > pool_len)
        return ctx_fail(ctx, SETOPS_ERR_INVALID, "pair " + std::to_string(p) + " outside the pool");
    }
    if (mat) {
      std::vector<uint64_t> offs;
      const uint64_t *ho = out_off;
      if (!ho) {
        offs.resize(npairs);
        for (size_t p = 0; p < npairs; ++p) {
          offs[p] = need;
          need += std::min(a_len[p], b_len[p]);
        }
        ho = offs.data();
      } else {
        for (size_t p = 0; p < npairs; ++p)
          need = std::max<uint64_t>(need, out_off[p] + std::min(a_len[p], b_len[p]));
      }
      if (need > out_cap)
        return ctx_fail(ctx, SETOPS_ERR_CAPACITY, "out_cap " + std::to_string(out_cap) +
                                                      " < " + std::to_string(need) + " output words");
      RK(stage(ctx, ctx->in[5], ho, npairs, &doff));
      CK(cudaStreamSynchronize(ctx->st));  // `offs` is a local
      RK(buf_reserve(ctx, ctx->out0, std::max<uint64_t>(need, 1) * 4));
      dout = static_cast<uint32_t *>(ctx->out0.p);
    }
    RK(buf_reserve(ctx, ctx->out1, npairs * 8));
    dlens = static_cast<uint64_t *>(ctx->out1.p);
  } else if (mat && !out_off) {
    // device lengths: offsets by a device scan; its total is checked here
    RK(buf_reserve(ctx, ctx->in[5], npairs * 8));
    RK(buf_reserve(ctx, ctx->units, prefix_bytes(npairs, 0)));
    uint64_t *o = static_cast<uint64_t *>(ctx->in[5].p);
    launch_prefix(a_len, b_len, npairs, ctx->units.p, o, &ctx->dlen[1], 0, nullptr, ctx->st);
    CK(cudaGetLastError());
    ctx->launches += 2;
    RK(ctx_read_u64(ctx, &ctx->dlen[1], &need));
    if (need > out_cap)
      return ctx_fail(ctx, SETOPS_ERR_CAPACITY, "out_cap " + std::to_string(out_cap) +
                                                    " < " + std::to_string(need) + " output words");
    doff = o;
  }
  // room for the unit map: exact when the lengths are on the host; from the
  // output capacity on the device (materialise); else a guess (the map falls
  // back to one unit per pair when the units do not fit)
  uint64_t unit_cap = npairs > 0xFFFFFFFFull ? 0 : 2 * npairs + 4096;
  if (host) {
    uint64_t units = 0;
    for (size_t q = 0; q < npairs; ++q) {
      const uint64_t mn = std::min(a_len[q], b_len[q]);
      units += mn > kBatchUnit ? (mn + kBatchUnit - 1) / kBatchUnit : 1;
    }
    unit_cap = unit_cap ? units : 0;
  } else if (mat) {
    unit_cap = unit_room(npairs, need ? need : out_cap);
  }
  RK(launch_batch(ctx, d, npairs, mat ? dout : nullptr, doff, dlens, v, ctx->batch_search_ratio,
                  unit_cap));
  if (host) {
    if (mat && need) CK(cudaMemcpyAsync(out, dout, need * 4, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(out_lens, dlens, npairs * 8, cudaMemcpyDeviceToHost, ctx->st));
  }
  return ctx_check_device(ctx);  // waits; reports device-side errors
}

// ---- BSR pairs ----
constexpr int kBsrThreads = 256;
constexpr int kBsrCapWords = 4096;  // longer set staged in shared memory up to this many words

int launch_batch_bsr(setops_ctx *ctx, const BatchBsrArgs &a0, bool mat) {
  const void *fn = mat ? reinterpret_cast<const void *>(&batch_bsr_kernel<kBsrThreads, kBsrCapWords, true>)
                       : reinterpret_cast<const void *>(&batch_bsr_kernel<kBsrThreads, kBsrCapWords, false>);
  const KernelInfo k{fn, kBsrThreads, 0, 1, mat ? "batch_bsr_mat" : "batch_bsr_count", false};
  int occ = 1;
  RK(ctx_occupancy(ctx, k, &occ));
  const uint64_t grid = std::max<uint64_t>(1, std::min<uint64_t>(uint64_t(occ) * ctx->sms, a0.npairs));
  BatchBsrArgs a = a0;
  a.sync = ctx->sync + 1;
  a.err = ctx->derr;
  void *args[] = {&a};
  return ctx_launch(ctx, k, grid, args);
}

// Shared body of the BSR batch entry points.  out_bases == NULL: count mode
// (per-pair popcount sums to out_lens).
int batch_bsr_impl(setops_ctx *ctx, const uint32_t *bases, const uint32_t *states,
                   size_t pool_len, const uint64_t *a_off, const uint64_t *a_len,
                   const uint64_t *b_off, const uint64_t *b_len, size_t npairs,
                   uint32_t *out_bases, uint32_t *out_states, size_t out_cap,
                   const uint64_t *out_off, uint64_t *out_lens, unsigned flags) {
  if (!ctx) return SETOPS_ERR_INVALID;
  if (npairs == 0) return SETOPS_OK;
  if (!bases || !states || !a_off || !a_len || !b_off || !b_len || !out_lens)
    return ctx_fail(ctx, SETOPS_ERR_INVALID, "NULL batch array");
  const bool host = (flags & SETOPS_HOST) != 0;
  const bool mat = out_bases != nullptr;
  if (mat && !out_states) return ctx_fail(ctx, SETOPS_ERR_INVALID, "out_states is NULL");
  CK(cudaSetDevice(ctx->device));
  BatchBsrArgs a{};
  a.bases = bases;
  a.states = states;
  a.a_off = a_off;
  a.a_len = a_len;
  a.b_off = b_off;
  a.b_len = b_len;
  a.npairs = npairs;
  a.out_off = out_off;
  a.out_bases = out_bases;
  a.out_states = out_states;
  a.out_lens = out_lens;
  uint64_t need = 0;
  if (host) {
    RK(stage(ctx, ctx->in[0], bases, pool_len, &a.bases));
    RK(stage(ctx, ctx->stage1, states, pool_len, &a.states));
    RK(stage(ctx, ctx->in[1], a_off, npairs, &a.a_off));
    RK(stage(ctx, ctx->in[2], a_len, npairs, &a.a_len));
    RK(stage(ctx, ctx->in[3], b_off, npairs, &a.b_off));
    RK(stage(ctx, ctx->in[4], b_len, npairs, &a.b_len));
    for (size_t q = 0; q < npairs; ++q) {
      if (a_off[q] + a_len[q] > pool_len || b_off[q] + b_len[q] > pool_len)
        return ctx_fail(ctx, SETOPS_ERR_INVALID, "pair " + std::to_string(q) + " outside the pool");
    }
    std::vector<uint64_t> offs;
    if (mat) {
      const uint64_t *ho = out_off;
      if (!ho) {
        offs.resize(npairs);
        for (size_t q = 0; q < npairs; ++q) {
          offs[q] = need;
          need += std::min(a_len[q], b_len[q]);
        }
        ho = offs.data();
      } else {
        for (size_t q = 0; q < npairs; ++q)
          need = std::max<uint64_t>(need, out_off[q] + std::min(a_len[q], b_len[q]));
      }
      if (need > out_cap)
        return ctx_fail(ctx, SETOPS_ERR_CAPACITY, "out_cap " + std::to_string(out_cap) +
                                                      " < " + std::to_string(need) + " output words");
      RK(stage(ctx, ctx->in[5], ho, npairs, &a.out_off));
      RK(buf_reserve(ctx, ctx->out0, std::max<uint64_t>(need, 1) * 4));
      RK(buf_reserve(ctx, ctx->stage0, std::max<uint64_t>(need, 1) * 4));
      a.out_bases = static_cast<uint32_t *>(ctx->out0.p);
      a.out_states = static_cast<uint32_t *>(ctx->stage0.p);
    }
    RK(buf_reserve(ctx, ctx->out1, npairs * 8));
    a.out_lens = static_cast<uint64_t *>(ctx->out1.p);
    CK(cudaStreamSynchronize(ctx->st));  // `offs` is a local
  } else if (mat && !out_off) {
    RK(buf_reserve(ctx, ctx->in[5], npairs * 8));
    RK(buf_reserve(ctx, ctx->units, prefix_bytes(npairs, 0)));
    uint64_t *o = static_cast<uint64_t *>(ctx->in[5].p);
    launch_prefix(a_len, b_len, npairs, ctx->units.p, o, &ctx->dlen[1], 0, nullptr, ctx->st);
    CK(cudaGetLastError());
    ctx->launches += 2;
    RK(ctx_read_u64(ctx, &ctx->dlen[1], &need));
    if (need > out_cap)
      return ctx_fail(ctx, SETOPS_ERR_CAPACITY, "out_cap " + std::to_string(out_cap) +
                                                    " < " + std::to_string(need) + " output words");
    a.out_off = o;
  }
  RK(launch_batch_bsr(ctx, a, mat));
  if (host) {
    if (mat && need) {
      CK(cudaMemcpyAsync(out_bases, a.out_bases, need * 4, cudaMemcpyDeviceToHost, ctx->st));
      CK(cudaMemcpyAsync(out_states, a.out_states, need * 4, cudaMemcpyDeviceToHost, ctx->st));
    }
    CK(cudaMemcpyAsync(out_lens, a.out_lens, npairs * 8, cudaMemcpyDeviceToHost, ctx->st));
  }
  return ctx_check_device(ctx);  // waits; reports device-side errors
}

}  // namespace

// A batch captured once into a CUDA graph and replayed (see setops_gpu.h).
struct setops_batch_plan {
  setops_ctx *ctx = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  void *dmem = nullptr;  // the plan's own coordination words and offsets
  int kernels = 0;       // kernel launches per replay
};

// The batch kernel of a shape (for callers launching on their own stream).
const KernelInfo &batch_kernel_info(bool mat, int variant) {
  if (variant < 0 || variant >= kNumBatch) variant = 0;
  return kBatchU32[variant][mat ? 1 : 0];
}

extern "C" {

int setops_gpu_batch_intersect(setops_ctx *ctx, const uint32_t *pool, size_t pool_len,
                               const uint64_t *a_off, const uint64_t *a_len,
                               const uint64_t *b_off, const uint64_t *b_len, size_t npairs,
                               uint32_t *out, size_t out_cap, const uint64_t *out_off,
                               uint64_t *out_lens, unsigned flags) {
  if (!out && npairs) return ctx_fail(ctx, SETOPS_ERR_INVALID, "out is NULL");
  return batch_impl(ctx, pool, pool_len, a_off, a_len, b_off, b_len, npairs, out, out_cap,
                    out_off, out_lens, flags);
}

int setops_gpu_batch_count(setops_ctx *ctx, const uint32_t *pool, size_t pool_len,
                           const uint64_t *a_off, const uint64_t *a_len, const uint64_t *b_off,
                           const uint64_t *b_len, size_t npairs, uint64_t *counts,
                           unsigned flags) {
  return batch_impl(ctx, pool, pool_len, a_off, a_len, b_off, b_len, npairs, nullptr, 0,
                    nullptr, counts, flags);
}

int setops_gpu_batch_intersect_bsr(setops_ctx *ctx, const uint32_t *bases,
                                   const uint32_t *states, size_t pool_len,
                                   const uint64_t *a_off, const uint64_t *a_len,
                                   const uint64_t *b_off, const uint64_t *b_len, size_t npairs,
                                   uint32_t *out_bases, uint32_t *out_states, size_t out_cap,
                                   const uint64_t *out_off, uint64_t *out_lens, unsigned flags) {
  if ((!out_bases || !out_states) && npairs) return ctx_fail(ctx, SETOPS_ERR_INVALID, "output is NULL");
  return batch_bsr_impl(ctx, bases, states, pool_len, a_off, a_len, b_off, b_len, npairs,
                        out_bases, out_states, out_cap, out_off, out_lens, flags);
}

int setops_gpu_batch_count_bsr(setops_ctx *ctx, const uint32_t *bases, const uint32_t *states,
                               size_t pool_len, const uint64_t *a_off, const uint64_t *a_len,
                               const uint64_t *b_off, const uint64_t *b_len, size_t npairs,
                               uint64_t *counts, unsigned flags) {
  return batch_bsr_impl(ctx, bases, states, pool_len, a_off, a_len, b_off, b_len, npairs,
                        nullptr, nullptr, 0, nullptr, counts, flags);
}

int setops_gpu_batch_plan_create(setops_ctx *ctx, const uint32_t *pool, size_t pool_len,
                                 const uint64_t *a_off, const uint64_t *a_len,
                                 const uint64_t *b_off, const uint64_t *b_len, size_t npairs,
                                 uint32_t *out, size_t out_cap, const uint64_t *out_off,
                                 uint64_t *out_lens, setops_batch_plan **plan_out) {
  if (!ctx || !plan_out) return SETOPS_ERR_INVALID;
  *plan_out = nullptr;
  (void)pool_len;
  if (npairs == 0 || !pool || !a_off || !a_len || !b_off || !b_len || !out_lens)
    return ctx_fail(ctx, SETOPS_ERR_INVALID, "batch plan: NULL array or no pairs");
  CK(cudaSetDevice(ctx->device));
  const bool mat = out != nullptr;
  const bool scan = mat && !out_off;
  auto *plan = new setops_batch_plan;
  plan->ctx = ctx;
  const size_t sync_bytes = 256;  // LaunchSync, padded
  const size_t offs_bytes = scan ? ((npairs * 8 + 8 + 15) & ~size_t(15)) : 0;
  // the unit map: room from the output capacity (materialise; it bounds the
  // pairs' smaller lengths) or a guess (count; unsplit when it does not fit)
  const uint64_t unit_cap = npairs > 0xFFFFFFFFull ? 0
                            : mat                  ? unit_room(npairs, out_cap)
                                                   : 2 * npairs + 4096;
  const size_t bytes = sync_bytes + offs_bytes + prefix_bytes(npairs, unit_cap);
  cudaError_t e = cudaMalloc(&plan->dmem, bytes);
  if (e == cudaSuccess) e = cudaMemset(plan->dmem, 0, bytes);
  if (e != cudaSuccess) {
    cudaFree(plan->dmem);
    delete plan;
    return ctx_cuda(ctx, e, "batch plan scratch");
  }
  LaunchSync *sync = static_cast<LaunchSync *>(plan->dmem);
  uint64_t *offs = reinterpret_cast<uint64_t *>(static_cast<char *>(plan->dmem) + sync_bytes);
  const KernelInfo &k = kBatchU32[ctx->batch_variant][mat ? 1 : 0];
  int occ = 1;
  int rc = ctx_occupancy(ctx, k, &occ);
  if (rc == SETOPS_OK) {
    const uint64_t grid = std::max<uint64_t>(
        1, std::min<uint64_t>(uint64_t(occ) * ctx->sms, std::max<uint64_t>(unit_cap, npairs)));
    BatchArgs a{};
    a.pool = pool;
    a.a_off = a_off;
    a.a_len = a_len;
    a.b_off = b_off;
    a.b_len = b_len;
    a.npairs = npairs;
    a.out_off = scan ? offs : out_off;
    a.out = out;
    a.out_lens = out_lens;
    a.search_ratio = ctx->batch_search_ratio;
    a.out_cap = mat ? std::max<uint64_t>(out_cap, 1) : 0;  // checked per pair on the device
    a.sync = sync;
    a.err = ctx->derr;
    void *args[] = {&a};
    // capture: prefixes (offsets, unit map) + batch kernel, on the context's stream
    e = cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      if (scan || unit_cap)
        launch_prefix(a_len, b_len, npairs, static_cast<char *>(plan->dmem) + sync_bytes + offs_bytes,
                      scan ? offs : nullptr, offs + npairs, unit_cap, &a, ctx->st);
      cudaError_t le = cudaGetLastError();
      if (le == cudaSuccess)
        le = cudaLaunchKernel(k.fn, dim3(unsigned(grid)), dim3(k.nt), args, k.dyn_smem, ctx->st);
      e = cudaStreamEndCapture(ctx->st, &plan->graph);
      if (le != cudaSuccess) e = le;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&plan->exec, plan->graph, 0);
    if (e != cudaSuccess) rc = ctx_cuda(ctx, e, "batch plan capture");
  }
  if (rc != SETOPS_OK) {
    if (plan->exec) cudaGraphExecDestroy(plan->exec);
    if (plan->graph) cudaGraphDestroy(plan->graph);
    cudaFree(plan->dmem);
    delete plan;
    return rc;
  }
  plan->kernels = scan || unit_cap ? 3 : 1;
  *plan_out = plan;
  return SETOPS_OK;
}

int setops_gpu_batch_plan_launch(setops_batch_plan *plan) {
  if (!plan) return SETOPS_ERR_INVALID;
  setops_ctx *ctx = plan->ctx;
  CK(cudaSetDevice(ctx->device));
  CK(cudaGraphLaunch(plan->exec, ctx->st));
  ctx->launches += uint64_t(plan->kernels);
  return SETOPS_OK;
}

int setops_gpu_batch_plan_destroy(setops_batch_plan *plan) {
  if (!plan) return SETOPS_OK;
  setops_ctx *ctx = plan->ctx;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->st);  // no replay in flight
  if (plan->exec) cudaGraphExecDestroy(plan->exec);
  if (plan->graph) cudaGraphDestroy(plan->graph);
  cudaFree(plan->dmem);
  delete plan;
  return SETOPS_OK;
}

int setops_gpu_batch_set_policy(setops_ctx *ctx, int variant, uint32_t search_ratio) {
  if (!ctx || variant < 0 || variant >= kNumBatch) return SETOPS_ERR_INVALID;
  ctx->batch_variant = variant;
  ctx->batch_search_ratio = search_ratio;
  return SETOPS_OK;
}

int setops_gpu_batch_get_policy(const setops_ctx *ctx, int *variant, uint32_t *search_ratio) {
  if (!ctx || !variant || !search_ratio) return SETOPS_ERR_INVALID;
  *variant = ctx->batch_variant;
  *search_ratio = ctx->batch_search_ratio;
  return SETOPS_OK;
}

int setops_gpu_batch_num_variants(void) { return kNumBatch; }

int setops_gpu_batch_autotune(setops_ctx *ctx, const uint32_t *pool, size_t pool_len,
                              const uint64_t *a_off, const uint64_t *a_len,
                              const uint64_t *b_off, const uint64_t *b_len, size_t npairs,
                              int reps, unsigned flags) {
  if (!ctx || npairs == 0) return SETOPS_ERR_INVALID;
  if (!pool || !a_off || !a_len || !b_off || !b_len)
    return ctx_fail(ctx, SETOPS_ERR_INVALID, "NULL batch array");
  CK(cudaSetDevice(ctx->device));
  const bool host = (flags & SETOPS_HOST) != 0;
  BatchDev d{pool, a_off, a_len, b_off, b_len};
  uint64_t need = 0;
  std::vector<uint64_t> offs;
  if (host) {
    RK(stage(ctx, ctx->in[0], pool, pool_len, &d.pool));
    RK(stage(ctx, ctx->in[1], a_off, npairs, &d.a_off));
    RK(stage(ctx, ctx->in[2], a_len, npairs, &d.a_len));
    RK(stage(ctx, ctx->in[3], b_off, npairs, &d.b_off));
    RK(stage(ctx, ctx->in[4], b_len, npairs, &d.b_len));
    offs.resize(npairs);
    for (size_t p = 0; p < npairs; ++p) {
      offs[p] = need;
      need += std::min(a_len[p], b_len[p]);
    }
    const uint64_t *doff = nullptr;
    RK(stage(ctx, ctx->in[5], offs.data(), npairs, &doff));
    CK(cudaStreamSynchronize(ctx->st));
  } else {
    RK(buf_reserve(ctx, ctx->in[5], npairs * 8));
    RK(buf_reserve(ctx, ctx->units, prefix_bytes(npairs, 0)));
    launch_prefix(a_len, b_len, npairs, ctx->units.p, static_cast<uint64_t *>(ctx->in[5].p),
                  &ctx->dlen[1], 0, nullptr, ctx->st);
    CK(cudaGetLastError());
    RK(ctx_read_u64(ctx, &ctx->dlen[1], &need));
  }
  RK(buf_reserve(ctx, ctx->out0, std::max<uint64_t>(need, 1) * 4));
  RK(buf_reserve(ctx, ctx->out1, npairs * 8));
  const uint64_t *doff = static_cast<const uint64_t *>(ctx->in[5].p);
  uint32_t *dout = static_cast<uint32_t *>(ctx->out0.p);
  uint64_t *dlens = static_cast<uint64_t *>(ctx->out1.p);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const uint32_t ratios[] = {0, 16, 64, 256, 1024};
  float best = 1e30f;
  int best_v = ctx->batch_variant;
  uint32_t best_r = ctx->batch_search_ratio;
  int rc = SETOPS_OK;
  for (int v = 0; v < kNumBatch && rc == SETOPS_OK; ++v) {
    for (uint32_t r : ratios) {
      std::vector<float> ts;
      for (int i = 0; i < std::max(reps, 1) + 1 && rc == SETOPS_OK; ++i) {
        cudaEventRecord(e0, ctx->st);
        rc = launch_batch(ctx, d, npairs, dout, doff, dlens, v, r);
        cudaEventRecord(e1, ctx->st);
        if (rc == SETOPS_OK) rc = ctx_check_device(ctx);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (i > 0) ts.push_back(ms);  // the first run warms up
      }
      if (rc != SETOPS_OK) break;
      std::sort(ts.begin(), ts.end());
      const float med = ts[ts.size() / 2];
      if (med < best) {
        best = med;
        best_v = v;
        best_r = r;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != SETOPS_OK) return rc;
  ctx->batch_variant = best_v;
  ctx->batch_search_ratio = best_r;
  return SETOPS_OK;
}

}  // extern "C"
