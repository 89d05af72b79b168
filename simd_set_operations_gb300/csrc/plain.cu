// plain.cu -- the plain GPU paths a caller writes without batching or
// serving (include/setops_bench.h): one launch per pair, one BSR call per
// pair, one k-set call per query, looped in C++ so that the baselines of the
// batched and served paths are timed without foreign-language call overhead.
#include <chrono>

#include <cuda_runtime.h>
#include <vector>

#include "../../include/setops_bench.h"
#include "../../include/setops_gpu.h"

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

}  // namespace

extern "C" {

int setops_bench_pairs_one_by_one(setops_ctx *ctx, const uint32_t *pool, const uint64_t *a_off,
                                  const uint64_t *a_len, const uint64_t *b_off,
                                  const uint64_t *b_len, size_t npairs, uint32_t *out,
                                  const uint64_t *out_off, uint64_t *lens_dev,
                                  double *seconds) {
  if (!ctx || (npairs && (!pool || !a_off || !a_len || !b_off || !b_len || !out || !out_off ||
                          !lens_dev)))
    return SETOPS_ERR_INVALID;
  const double t0 = now_s();
  for (size_t p = 0; p < npairs; ++p) {
    const size_t na = size_t(a_len[p]), nb = size_t(b_len[p]);
    const int rc = setops_gpu_intersect_async(ctx, pool + a_off[p], na, pool + b_off[p], nb,
                                              out + out_off[p], na < nb ? na : nb,
                                              lens_dev + p, 0);
    if (rc != SETOPS_OK) return rc;
  }
  const int rc = setops_gpu_synchronize(ctx);
  if (seconds) *seconds = now_s() - t0;
  return rc;
}

int setops_bench_bsr_pairs_one_by_one(setops_ctx *ctx, const uint32_t *bases,
                                      const uint32_t *states, const uint64_t *a_off,
                                      const uint64_t *a_len, const uint64_t *b_off,
                                      const uint64_t *b_len, size_t npairs,
                                      uint32_t *out_bases, uint32_t *out_states,
                                      const uint64_t *out_off, uint64_t *lens,
                                      double *seconds) {
  if (!ctx || (npairs && (!bases || !states || !a_off || !a_len || !b_off || !b_len ||
                          !out_bases || !out_states || !out_off || !lens)))
    return SETOPS_ERR_INVALID;
  const double t0 = now_s();
  for (size_t p = 0; p < npairs; ++p) {
    const size_t na = size_t(a_len[p]), nb = size_t(b_len[p]);
    size_t n = 0;
    const int rc = setops_gpu_intersect_bsr(
        ctx, bases + a_off[p], states + a_off[p], na, bases + b_off[p], states + b_off[p], nb,
        out_bases + out_off[p], out_states + out_off[p], na < nb ? na : nb, &n, 0);
    if (rc != SETOPS_OK) return rc;
    lens[p] = n;
  }
  if (seconds) *seconds = now_s() - t0;
  return SETOPS_OK;
}

int setops_bench_record_event(void *event, void *stream) {
  if (!event) return SETOPS_ERR_INVALID;
  const cudaError_t e = cudaEventRecordWithFlags(static_cast<cudaEvent_t>(event),
                                                 static_cast<cudaStream_t>(stream),
                                                 cudaEventRecordExternal);
  return e == cudaSuccess ? SETOPS_OK : SETOPS_ERR_CUDA;
}

int setops_bench_queries_one_by_one(setops_ctx *ctx, const uint32_t *pool, const uint64_t *offs,
                                    const uint64_t *lens, const uint32_t *ids,
                                    const uint32_t *ks, size_t kstride, size_t nq,
                                    uint32_t *out, size_t out_cap, uint64_t *latency_ns,
                                    uint64_t *counts, double *seconds) {
  if (!ctx || (nq && (!pool || !offs || !lens || !ids || !ks || !out)) || kstride == 0)
    return SETOPS_ERR_INVALID;
  std::vector<const uint32_t *> sets(kstride);
  std::vector<size_t> slen(kstride);
  const double t0 = now_s();
  for (size_t q = 0; q < nq; ++q) {
    const size_t k = ks[q];
    if (k > kstride) return SETOPS_ERR_INVALID;
    for (size_t i = 0; i < k; ++i) {
      const uint32_t id = ids[q * kstride + i];
      sets[i] = pool + offs[id];
      slen[i] = size_t(lens[id]);
    }
    const double tq = now_s();
    size_t n = 0;
    const int rc = setops_gpu_svs(ctx, sets.data(), slen.data(), k, out, out_cap, &n, 0);
    if (rc != SETOPS_OK) return rc;
    if (latency_ns) latency_ns[q] = uint64_t((now_s() - tq) * 1e9);
    if (counts) counts[q] = n;
  }
  if (seconds) *seconds = now_s() - t0;
  return SETOPS_OK;
}

}  // extern "C"
