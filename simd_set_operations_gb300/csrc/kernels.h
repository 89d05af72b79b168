// kernels.h -- host-side view of the compiled kernel variants.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace setops {

struct MergeArgs;
struct GallopArgs;

// One compiled kernel: entry point, block size, dynamic shared memory, the
// number of merged elements (merge), small-set elements (search) or A
// elements (bitmap) one tile covers, and whether it must be launched
// cooperatively (all CTAs resident: it holds grid-wide barriers).
struct KernelInfo {
  const void *fn;
  int nt;
  size_t dyn_smem;
  int tile;
  const char *name;
  bool coop = false;
};

enum Algo { ALGO_MERGE = 1, ALGO_GALLOP = 2, ALGO_BITMAP = 3 };

int num_variants(Algo algo, bool bsr);
// SETOPS_ALGO_BITMAP variant with coarse bitmaps for sparse tiles (the
// default for size ratios 2-31 and for SvS steps below the search ratio)
constexpr int kCoarseBitmap = 7;
// SETOPS_ALGO_BITMAP variant whose materialise kernel stages both inputs in
// shared memory by asynchronous copies (the default for size ratios below 2)
constexpr int kStagedWindow = 8;
// SETOPS_ALGO_GALLOP variant with eight lanes per element and no sample (the
// in-place search over host memory), and whether a u32 search variant puts
// one thread on each element (its rounds of single probes wait on the link
// when the larger set is host memory)
constexpr int kGallopNineWay = 3;
bool gallop_thread_per_element(int variant);
// BSR SETOPS_ALGO_MERGE variant that compares 32-word blocks of the two sets
// all against all, a warp per run of blocks (bcast.cuh)
constexpr int kBcastBsr = 3;
// The fused k-set kernel (kset.cuh): count or materialise.
const KernelInfo &kset_kernel(bool mat);
// 256 threads, 4096-element tiles of the smallest set, 3 CTAs per SM: of 16
// shapes timed on the k-set configuration (k = 3, 5, 8) the fastest in sum,
// 22.9 / 27.7 / 35.1 us against 24.3 / 31.3 / 40.3 for 128 threads with
// 2048-element tiles at 6 CTAs per SM
constexpr int kKsetThreads = 256;
// kind: 0 count, 1 materialise
const KernelInfo &variant(Algo algo, bool bsr, bool mat, int v);

// Utility kernels (launch on `st`).
cudaError_t launch_validate_sorted(const uint32_t *a, uint64_t n, int *flag,
                                   int sms, cudaStream_t st);
cudaError_t launch_bsr_encode(const uint32_t *in, uint64_t n, uint32_t *bases,
                              uint32_t *states, uint64_t *nwords,
                              uint64_t *status, LaunchSync *sync, int *err,
                              uint32_t epoch, int grid, cudaStream_t st);
cudaError_t launch_bsr_decode(const uint32_t *bases, const uint32_t *states,
                              uint64_t n, uint32_t *out, uint64_t out_cap,
                              uint64_t *out_len, uint64_t *status,
                              LaunchSync *sync, int *err, uint32_t epoch,
                              int grid, cudaStream_t st);
// A look-back wait that nothing ever satisfies (status[0..1] hold no word
// of tag `epoch`), ended by the wait limit; *waited gets its duration.
cudaError_t launch_wait_check(uint64_t *status, uint32_t epoch, int *err, uint64_t *waited,
                              cudaStream_t st);
constexpr int kBsrEncodeTile = 256 * 8;  // elements per encode tile
constexpr int kBsrDecodeTile = 256 * 4;  // words per decode tile
const void *bsr_encode_fn();
const void *bsr_decode_fn();
constexpr int kUtilThreads = 256;

}  // namespace setops
