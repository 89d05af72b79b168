// autotune.cu -- the autotuner of the 2-set policy table (include/setops_gpu.h).
//
// The reference picks its intersection algorithm per instruction set at
// compile time (setops/src/intersect.rs:26-36).  Here the choice is a table
// of (algorithm, kernel variant) per size-ratio band and size class of the
// smaller input, and this file fills it by measurement on the GPU at hand:
// for every cell it generates a seeded pair of that shape (the reference
// generator's construction, benchmark/src/generators.rs:30-68, at the given
// density and 1 % selectivity), times every candidate kernel with CUDA
// events, checks that every candidate finds the same number of matches, and
// writes the fastest into the table.  Density is not a key of the table: the
// window kernels choose dense or sparse handling per tile from the values
// themselves; the autotuner's density only shapes its test pairs.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/setops_bench.h"
#include "../../include/setops_gpu.h"
#include "kernels.h"
#include "runtime.h"

using namespace setops;

#define CK(call)                                            \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return ctx_cuda(ctx, e_, #call); \
  } while (0)

namespace {

struct DevPair {
  uint32_t *a = nullptr, *b = nullptr, *out = nullptr;
  uint64_t *len = nullptr;
  ~DevPair() {
    cudaFree(a);
    cudaFree(b);
    cudaFree(out);
    cudaFree(len);
  }
};

// Representative smaller-input length of each size class (runtime.h's
// size_class: [0, 2^12), [2^12, 2^16), [2^16, 2^22), [2^22, ...)).
constexpr uint64_t kClassLen[kSizeClasses] = {uint64_t(1) << 10, uint64_t(1) << 14,
                                              uint64_t(1) << 19, uint64_t(1) << 23};

}  // namespace

extern "C" {

int setops_gpu_autotune(setops_ctx *ctx, int band_lo, int band_hi, size_t max_elems,
                        double density, int reps, int *tuned) {
  if (tuned) *tuned = 0;
  if (!ctx || band_lo < 0 || band_hi >= kRatioBands || band_lo > band_hi || !(density > 0) ||
      density > 1 || max_elems < 2)
    return SETOPS_ERR_INVALID;
  CK(cudaSetDevice(ctx->device));
  reps = std::max(reps, 1);

  std::vector<unsigned> cands;
  for (int v = 0; v < num_variants(ALGO_BITMAP, false); ++v)
    cands.push_back(SETOPS_ALGO_BITMAP | SETOPS_VARIANT(v));
  for (int v = 0; v < num_variants(ALGO_MERGE, false); ++v)
    cands.push_back(SETOPS_ALGO_MERGE | SETOPS_VARIANT(v));
  for (int v = 0; v < num_variants(ALGO_GALLOP, false); ++v)
    cands.push_back(SETOPS_ALGO_GALLOP | SETOPS_VARIANT(v));

  // the largest pair any cell uses
  uint64_t cap_small = 0, cap_large = 0;
  for (int c = 0; c < kSizeClasses; ++c)
    for (int band = band_lo; band <= band_hi; ++band) {
      const uint64_t mn = kClassLen[c];
      const uint64_t mx = uint64_t(double(mn) * double(uint64_t(1) << band) * 1.4);
      if (mx > max_elems) continue;
      cap_small = std::max(cap_small, mn);
      cap_large = std::max(cap_large, mx);
    }
  if (cap_small == 0) return SETOPS_OK;  // no cell fits max_elems

  DevPair d;
  CK(cudaMalloc(&d.a, cap_small * 4));
  CK(cudaMalloc(&d.b, cap_large * 4));
  CK(cudaMalloc(&d.out, cap_small * 4));
  CK(cudaMalloc(&d.len, sizeof(uint64_t)));
  std::vector<uint32_t> hs(cap_small), hl(cap_large);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  int rc = SETOPS_OK;
  int done = 0;
  for (int c = 0; c < kSizeClasses && rc == SETOPS_OK; ++c) {
    for (int band = band_lo; band <= band_hi && rc == SETOPS_OK; ++band) {
      const uint64_t mn = kClassLen[c];
      // a ratio inside the band: 1.4 * 2^band
      const uint64_t mx = uint64_t(double(mn) * double(uint64_t(1) << band) * 1.4);
      if (mx > max_elems) continue;
      if (setops_gen_twoset(0x5e7u + 131u * uint64_t(band) + 7u * uint64_t(c), density, 0.01,
                            mn, mx, hs.data(), hl.data()) != 0) {
        rc = ctx_fail(ctx, SETOPS_ERR_INVALID, "autotune: pair generation failed");
        break;
      }
      if (cudaMemcpyAsync(d.a, hs.data(), mn * 4, cudaMemcpyHostToDevice, ctx->st) != cudaSuccess ||
          cudaMemcpyAsync(d.b, hl.data(), mx * 4, cudaMemcpyHostToDevice, ctx->st) != cudaSuccess) {
        rc = ctx_cuda(ctx, cudaGetLastError(), "autotune: copy");
        break;
      }
      float best = 1e30f;
      unsigned best_flags = 0;
      uint64_t want = UINT64_MAX;
      for (unsigned f : cands) {
        // a search per element of a balanced pair is never the answer
        if (band == 0 && (f & SETOPS_ALGO_MASK) == SETOPS_ALGO_GALLOP) continue;
        auto launch = [&]() {
          return setops_gpu_intersect_async(ctx, d.a, mn, d.b, mx, d.out, mn, d.len, f);
        };
        rc = launch();  // warm-up and the match count
        if (rc != SETOPS_OK) break;
        uint64_t n = 0;
        rc = ctx_read_u64(ctx, d.len, &n);
        if (rc != SETOPS_OK) break;
        if (want == UINT64_MAX) want = n;
        if (n != want) {
          rc = ctx_fail(ctx, SETOPS_ERR_CUDA,
                        "autotune: candidates disagree on the match count (" +
                            std::to_string(n) + " vs " + std::to_string(want) + ")");
          break;
        }
        cudaEventRecord(e0, ctx->st);
        for (int r = 0; r < reps && rc == SETOPS_OK; ++r) rc = launch();
        cudaEventRecord(e1, ctx->st);
        if (rc != SETOPS_OK) break;
        rc = ctx_check_device(ctx);  // synchronises
        if (rc != SETOPS_OK) break;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
          best = ms;
          best_flags = f;
        }
      }
      if (rc != SETOPS_OK) break;
      if (best_flags) {
        ctx->policy[0][band][c] = best_flags;
        ++done;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (tuned) *tuned = done;
  return rc;
}

// The BSR table, the same way: a cell's pair is generated as arrays,
// encoded to BSR words on the device (setops/src/bsr.rs:140-163), and every
// BSR candidate (merge-family variants, among them the block-broadcast
// kernel, and search variants) is timed; all must agree on the result's word
// count.  Bands and classes are by word count, as the BSR choice is; a set's
// word count depends on its density, so the larger set is rescaled once when
// the first pair's word ratio falls outside the band.
int setops_gpu_autotune_bsr(setops_ctx *ctx, int band_lo, int band_hi, size_t max_elems,
                            double density, int reps, int *tuned) {
  if (tuned) *tuned = 0;
  if (!ctx || band_lo < 0 || band_hi >= kRatioBands || band_lo > band_hi || !(density > 0) ||
      density > 1 || max_elems < 2)
    return SETOPS_ERR_INVALID;
  CK(cudaSetDevice(ctx->device));
  reps = std::max(reps, 1);

  std::vector<unsigned> cands;
  for (int v = 0; v < num_variants(ALGO_MERGE, true); ++v)
    cands.push_back(SETOPS_ALGO_MERGE | SETOPS_VARIANT(v));
  for (int v = 0; v < num_variants(ALGO_GALLOP, true); ++v)
    cands.push_back(SETOPS_ALGO_GALLOP | SETOPS_VARIANT(v));

  // device room for the largest pair any cell may generate (a rescale at
  // most doubles the larger set, within max_elems)
  uint64_t cap_small = 0, cap_large = 0;
  for (int c = 0; c < kSizeClasses; ++c)
    for (int band = band_lo; band <= band_hi; ++band) {
      const uint64_t mn = kClassLen[c];
      const uint64_t mx = std::min<uint64_t>(
          max_elems, uint64_t(double(mn) * double(uint64_t(1) << band) * 1.4 * 2.0));
      if (uint64_t(double(mn) * double(uint64_t(1) << band) * 1.4) > max_elems) continue;
      cap_small = std::max(cap_small, mn);
      cap_large = std::max(cap_large, mx);
    }
  if (cap_small == 0) return SETOPS_OK;

  DevPair d;            // arrays
  DevPair w;            // BSR: a/b bases, out bases
  uint32_t *sa = nullptr, *sb = nullptr, *so = nullptr;  // states
  struct Free {
    uint32_t **p[3];
    ~Free() {
      for (auto q : p) cudaFree(*q);
    }
  } fr{{&sa, &sb, &so}};
  CK(cudaMalloc(&d.a, cap_small * 4));
  CK(cudaMalloc(&d.b, cap_large * 4));
  CK(cudaMalloc(&w.a, cap_small * 4));
  CK(cudaMalloc(&w.b, cap_large * 4));
  CK(cudaMalloc(&w.out, cap_small * 4));
  CK(cudaMalloc(&w.len, sizeof(uint64_t)));
  CK(cudaMalloc(&sa, cap_small * 4));
  CK(cudaMalloc(&sb, cap_large * 4));
  CK(cudaMalloc(&so, cap_small * 4));
  std::vector<uint32_t> hs(cap_small), hl(cap_large);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  int rc = SETOPS_OK;
  int done = 0;
  auto band_of = [](uint64_t mn, uint64_t mx) {
    int band = 0;
    for (uint64_t r = mx / mn; r > 1 && band < kRatioBands - 1; r >>= 1) ++band;
    return band;
  };
  for (int c = 0; c < kSizeClasses && rc == SETOPS_OK; ++c) {
    for (int band = band_lo; band <= band_hi && rc == SETOPS_OK; ++band) {
      const uint64_t mn = kClassLen[c];
      double scale = 1.0;
      size_t nwa = 0, nwb = 0;
      bool fits = true;
      for (int attempt = 0; attempt < 2 && rc == SETOPS_OK; ++attempt) {
        const uint64_t mx = uint64_t(double(mn) * double(uint64_t(1) << band) * 1.4 * scale);
        if (mx > max_elems || mx > cap_large || mx < 1) {
          fits = false;
          break;
        }
        if (setops_gen_twoset(0xb5e7u + 131u * uint64_t(band) + 7u * uint64_t(c), density, 0.01,
                              mn, mx, hs.data(), hl.data()) != 0) {
          rc = ctx_fail(ctx, SETOPS_ERR_INVALID, "autotune: pair generation failed");
          break;
        }
        if (cudaMemcpyAsync(d.a, hs.data(), mn * 4, cudaMemcpyHostToDevice, ctx->st) != cudaSuccess ||
            cudaMemcpyAsync(d.b, hl.data(), mx * 4, cudaMemcpyHostToDevice, ctx->st) != cudaSuccess) {
          rc = ctx_cuda(ctx, cudaGetLastError(), "autotune: copy");
          break;
        }
        rc = setops_gpu_bsr_from_sorted(ctx, d.a, mn, w.a, sa, &nwa, 0);
        if (rc == SETOPS_OK) rc = setops_gpu_bsr_from_sorted(ctx, d.b, mx, w.b, sb, &nwb, 0);
        if (rc != SETOPS_OK || nwa == 0 || nwb == 0) break;
        const uint64_t lo = std::min<uint64_t>(nwa, nwb), hi = std::max<uint64_t>(nwa, nwb);
        if (band_of(lo, hi) == band) break;
        // aim the word ratio at 1.4 * 2^band
        scale *= 1.4 * double(uint64_t(1) << band) / (double(hi) / double(lo));
        if (scale > 2.0) scale = 2.0;
      }
      if (rc != SETOPS_OK) break;
      if (!fits || nwa == 0 || nwb == 0) continue;
      const uint64_t lo = std::min<uint64_t>(nwa, nwb), hi = std::max<uint64_t>(nwa, nwb);
      const int cell_band = band_of(lo, hi), cell_class = size_class(lo);
      if (cell_band < band_lo || cell_band > band_hi) continue;
      float best = 1e30f;
      unsigned best_flags = 0;
      uint64_t want = UINT64_MAX;
      for (unsigned f : cands) {
        if (cell_band == 0 && (f & SETOPS_ALGO_MASK) == SETOPS_ALGO_GALLOP) continue;
        PairJob j;
        j.a = w.a;
        j.sa = sa;
        j.b = w.b;
        j.sb = sb;
        j.na = nwa;
        j.nb = nwb;
        j.bsr = true;
        j.out = w.out;
        j.out_s = so;
        j.out_cap = lo;
        j.len_dev = w.len;
        j.choice = ctx_choose(ctx, nwa, nwb, true, f);
        rc = ctx_launch_pair(ctx, j);  // warm-up and the result's word count
        if (rc != SETOPS_OK) break;
        uint64_t n = 0;
        rc = ctx_read_u64(ctx, w.len, &n);
        if (rc != SETOPS_OK) break;
        if (want == UINT64_MAX) want = n;
        if (n != want) {
          rc = ctx_fail(ctx, SETOPS_ERR_CUDA,
                        "autotune: BSR candidates disagree on the result (" + std::to_string(n) +
                            " vs " + std::to_string(want) + " words)");
          break;
        }
        cudaEventRecord(e0, ctx->st);
        for (int r = 0; r < reps && rc == SETOPS_OK; ++r) rc = ctx_launch_pair(ctx, j);
        cudaEventRecord(e1, ctx->st);
        if (rc != SETOPS_OK) break;
        rc = ctx_check_device(ctx);
        if (rc != SETOPS_OK) break;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
          best = ms;
          best_flags = f;
        }
      }
      if (rc != SETOPS_OK) break;
      if (best_flags) {
        ctx->policy[1][cell_band][cell_class] = best_flags;
        ++done;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (tuned) *tuned = done;
  return rc;
}

int setops_gpu_device_key(setops_ctx *ctx, char *buf, size_t cap) {
  if (!ctx || !buf || cap == 0) return SETOPS_ERR_INVALID;
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, ctx->device));
  int drv = 0;
  CK(cudaDriverGetVersion(&drv));
  const int n = std::snprintf(buf, cap, "%s|sm_%d%d|%d SMs|driver %d", prop.name, prop.major,
                              prop.minor, prop.multiProcessorCount, drv);
  return (n < 0 || size_t(n) >= cap) ? SETOPS_ERR_CAPACITY : SETOPS_OK;
}

}  // extern "C"
