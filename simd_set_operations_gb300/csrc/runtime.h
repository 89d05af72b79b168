// runtime.h -- host-side context shared by the runtime translation units.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "kernels.h"

namespace setops {

constexpr int kSyncSlots = 8;      // coordination words (one per stream lane)
constexpr int kLenWords = 64;      // device u64 result slots
constexpr int kRatioBands = 32;    // policy bands: floor(log2(max/min))
constexpr int kSizeClasses = 4;    // policy size classes of min(na, nb)
// Size class of a pair by its smaller input: [0, 2^12), [2^12, 2^16),
// [2^16, 2^22), [2^22, ...)
inline int size_class(uint64_t mn) {
  return mn < (uint64_t(1) << 12) ? 0 : mn < (uint64_t(1) << 16) ? 1 : mn < (uint64_t(1) << 22) ? 2 : 3;
}
constexpr uint64_t kMinTilesPerCta = 4;  // merge: tiles per CTA before more CTAs

struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
};

struct Choice {
  Algo algo = ALGO_MERGE;
  int variant = 0;
};

// One 2-set launch on device pointers.  na/nb are the lengths, or upper
// bounds when na_dev/nb_dev give the actual lengths on the device.
struct PairJob {
  const uint32_t *a = nullptr, *b = nullptr;
  const uint32_t *sa = nullptr, *sb = nullptr;
  uint64_t na = 0, nb = 0;
  const uint64_t *na_dev = nullptr, *nb_dev = nullptr;
  bool bsr = false;
  uint32_t *out = nullptr, *out_s = nullptr;  // NULL: count only
  uint64_t out_cap = 0;
  uint64_t *len_dev = nullptr;
  Choice choice;
  int skip_rule = 0;
  uint32_t ratio_thr = 0;
  int sync_slot = 0;
  uint64_t grid_cap = 0;  // 0: no cap
};

}  // namespace setops

struct setops_ctx {
  int device = 0;
  cudaStream_t own = nullptr;
  cudaStream_t st = nullptr;
  int sms = 0;
  std::string err;
  void *dsmall = nullptr;
  setops::LaunchSync *sync = nullptr;  // kSyncSlots entries
  int *derr = nullptr;
  int *dflag = nullptr;
  uint64_t *dlen = nullptr;   // kLenWords device result words
  uint64_t *hres = nullptr;   // 16 pinned host words
  setops::DevBuf status;
  setops::DevBuf in[6];
  setops::DevBuf out0, out1;
  setops::DevBuf stage0, stage1;
  setops::DevBuf inter[2];
  setops::DevBuf units;  // batch: the long-pair unit map
  setops::DevBuf plen;   // multi-pair host call: per-pair result lengths
  cudaStream_t aux = nullptr;           // multi-pair host call: the in-place pairs' stream
  cudaEvent_t ev_main = nullptr, ev_aux = nullptr;
  uint64_t *hlens = nullptr;            // pinned host copy of plen
  size_t hlens_cap = 0;                 // entries
  uint32_t epoch = 1;
  uint64_t launches = 0;
  std::map<const void *, int> occ;
  unsigned policy[2][setops::kRatioBands][setops::kSizeClasses] = {};
  int batch_variant = 0;             // batch kernel shape
  uint32_t batch_search_ratio = 16;  // batch pairs with max/min >= this: search path

  std::vector<setops::DevBuf *> all_bufs() {
    std::vector<setops::DevBuf *> v = {&status, &out0, &out1, &stage0,
                                       &stage1, &inter[0], &inter[1], &units,
                                       &plen};
    for (auto &b : in) v.push_back(&b);
    return v;
  }
};

// The batch kernel of a shape (batch.cu).
const setops::KernelInfo &batch_kernel_info(bool mat, int variant);

// Runtime helpers (runtime.cu).
int ctx_fail(setops_ctx *ctx, int status, const std::string &what);
int ctx_cuda(setops_ctx *ctx, cudaError_t e, const char *what);
int buf_reserve(setops_ctx *ctx, setops::DevBuf &b, size_t bytes);
int ctx_occupancy(setops_ctx *ctx, const setops::KernelInfo &k, int *blocks);
int ctx_next_epoch(setops_ctx *ctx, uint32_t *epoch);
int ctx_status_words(setops_ctx *ctx, uint64_t n);
int ctx_check_device(setops_ctx *ctx);
int ctx_read_u64(setops_ctx *ctx, const uint64_t *dev, uint64_t *out);
setops::Choice ctx_choose(const setops_ctx *ctx, uint64_t na, uint64_t nb,
                          bool bsr, unsigned flags);
uint32_t ctx_search_threshold(const setops_ctx *ctx, bool bsr);
int ctx_launch_pair(setops_ctx *ctx, const setops::PairJob &j);
int ctx_launch(setops_ctx *ctx, const setops::KernelInfo &k, uint64_t grid,
               void **args);
int ctx_stage_in(setops_ctx *ctx, int slot, const uint32_t *h, size_t n,
                 const uint32_t **d);
