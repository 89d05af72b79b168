// noalloc.cu -- setops_gpu_intersect_noalloc: the 2-set materialising
// intersection for callers that cannot allocate device memory.
//
// Who needs it.  The context API (setops_gpu_create and the calls on a
// context) allocates: the context's own buffers at creation, and scratch that
// grows on demand the first time a larger input arrives.  Some callers cannot
// allow that.  A host program that owns all device memory through its own
// pool may forbid allocations outside it.  A latency-bound path cannot take a
// cudaMalloc/cudaFree, which may synchronise the device and has no latency
// bound.  A process whose device memory is nearly all taken (a resident
// index filling the GPU) may see an allocation fail halfway through a query.
// This entry point takes the caller's input and output buffers and uses only
// memory the library already holds.
//
// The scratch it needs (the merge kernel's staging area for matches, its
// per-CTA words and its launch-coordination words) lives in one file-scope
// __device__ array of fixed size, which every GPU that loads the library
// holds until the process exits.  That fixes the limit: the smaller input
// may hold at most SETOPS_NOALLOC_MAX_SMALL elements.
//
// In host code the array's name is only a host-side stand-in for the symbol,
// not a device address; the device address comes from cudaGetSymbolAddress,
// once per device, with that device current.  The first call on a device
// does that set-up (together with the kernel's shared-memory attribute and
// occupancy query); that first call should come before any stream capture.
// The set-up is also when the CUDA runtime, which loads a library's device
// code on first use by default, loads the array and the kernel onto the
// device: the first call therefore does take device memory, once.  A caller
// whose GPU will later be full makes that first call (tiny inputs will do)
// while memory is still free, or runs with CUDA_MODULE_LOADING=EAGER so that
// everything is loaded when the process starts.  A set-up that failed is
// tried again on the next call.
//
// Every call on a device shares the array, and a call leaves its contents
// behind.  Each call therefore first zeroes what the kernel needs zeroed
// (the launch-coordination words, the error word, the result word and the
// per-CTA words it will use); the staging area is written before it is read.
// Two calls that overlapped on the GPU would race on the array; this entry
// point prevents that within a process by holding a per-device lock for the
// whole call and returning only after its work on the stream has finished.
#include <cstdint>
#include <mutex>

#include <cuda_runtime.h>

#include "kernels.h"
#include "merge.cuh"
#include "setops_gpu.h"

namespace {

constexpr size_t kMaxSmall = SETOPS_NOALLOC_MAX_SMALL;  // staging words
constexpr uint64_t kMaxCtas = 2048;                     // per-CTA words
constexpr size_t kCtlBytes = 256;  // LaunchSync @0, error word @64, result @128
constexpr size_t kErrOff = 64, kResOff = 128;
constexpr size_t kStageOff = kCtlBytes + 2 * kMaxCtas * sizeof(uint64_t);
constexpr size_t kScratchBytes = kStageOff + kMaxSmall * sizeof(uint32_t);
constexpr int kMaxDevices = 64;
// The merge kernel this entry point runs: array keys, materialising, the
// default shape.
constexpr int kVariant = 0;

struct DeviceSetup {
  std::mutex lock;      // one call at a time on this device; guards the set-up
  bool ready = false;   // set only by a set-up that succeeded
  unsigned char *base = nullptr;  // device address of the scratch array
  int sms = 0;
  int occ = 0;
};
DeviceSetup g_setup[kMaxDevices];

}  // namespace

// The scratch: modest (about 4 MiB), held by every GPU that loads the
// library until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

// Once per device, with that device current and s.lock held.  A set-up
// that fails leaves s.ready false, so the next call tries again.
cudaError_t setup_device(int dev, DeviceSetup &s) {
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s.sms, cudaDevAttrMultiProcessorCount, dev);
  const setops::KernelInfo &k = setops::variant(setops::ALGO_MERGE, false, true, kVariant);
  if (e == cudaSuccess && k.dyn_smem > 0)
    e = cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(k.dyn_smem));
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&s.occ, k.fn, k.nt, k.dyn_smem);
  if (e == cudaSuccess && s.occ < 1) e = cudaErrorInvalidConfiguration;
  if (e != cudaSuccess) return e;
  s.base = static_cast<unsigned char *>(p);
  s.ready = true;
  return cudaSuccess;
}

}  // namespace

extern "C" int setops_gpu_intersect_noalloc(const uint32_t *a, size_t na,
                                            const uint32_t *b, size_t nb,
                                            uint32_t *out, size_t out_cap,
                                            size_t *out_len, void *stream) {
  if (!out_len) return SETOPS_ERR_INVALID;
  *out_len = 0;
  const size_t mn = na < nb ? na : nb;
  if ((na && !a) || (nb && !b) || (mn && !out)) return SETOPS_ERR_INVALID;
  if (mn > kMaxSmall) return SETOPS_ERR_TOO_LARGE;
  if (out_cap < mn) return SETOPS_ERR_CAPACITY;
  if (mn == 0) return SETOPS_OK;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return SETOPS_ERR_CUDA;
  DeviceSetup &s = g_setup[dev];
  std::lock_guard<std::mutex> guard(s.lock);
  if (!s.ready && setup_device(dev, s) != cudaSuccess) return SETOPS_ERR_CUDA;

  const setops::KernelInfo &k = setops::variant(setops::ALGO_MERGE, false, true, kVariant);
  const uint64_t total = uint64_t(na) + uint64_t(nb);
  const uint64_t per = uint64_t(k.tile) * 4;  // at least four chunks per CTA
  uint64_t grid = uint64_t(s.occ) * uint64_t(s.sms);
  if (grid > (total + per - 1) / per) grid = (total + per - 1) / per;
  if (grid < 1) grid = 1;
  if (grid > kMaxCtas) grid = kMaxCtas;

  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char *base = s.base;
  uint64_t *status = reinterpret_cast<uint64_t *>(base + kCtlBytes);
  // zero what must start at zero: coordination, error and result words, and
  // the per-CTA count and co-rank words this launch uses
  if (cudaMemsetAsync(base, 0, kCtlBytes, st) != cudaSuccess ||
      cudaMemsetAsync(status, 0, size_t(2 * grid) * sizeof(uint64_t), st) != cudaSuccess)
    return SETOPS_ERR_CUDA;

  setops::MergeArgs m{};
  m.a = a;
  m.b = b;
  m.na = na;
  m.nb = nb;
  m.stage = reinterpret_cast<uint32_t *>(base + kStageOff);
  m.out = out;
  m.out_cap = out_cap;
  m.out_len = reinterpret_cast<uint64_t *>(base + kResOff);
  m.status = status;
  m.coranks = status + grid;
  m.sync = reinterpret_cast<setops::LaunchSync *>(base);
  m.err = reinterpret_cast<int *>(base + kErrOff);
  m.epoch = 1;  // the per-CTA words were zeroed: nothing stale carries epoch 1
  void *args[] = {&m};
  if (cudaLaunchKernel(k.fn, dim3(unsigned(grid)), dim3(unsigned(k.nt)), args, k.dyn_smem,
                       st) != cudaSuccess)
    return SETOPS_ERR_CUDA;

  struct {
    int err;
    int pad[15];
    uint64_t len;
  } res{};
  static_assert(kResOff - kErrOff == 64, "result word layout");
  if (cudaMemcpyAsync(&res, base + kErrOff, sizeof(res), cudaMemcpyDeviceToHost, st) !=
          cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return SETOPS_ERR_CUDA;
  if (res.err == setops::DEV_ERR_CAPACITY) return SETOPS_ERR_CAPACITY;
  if (res.err != 0) return SETOPS_ERR_TIMEOUT;
  *out_len = size_t(res.len);
  return SETOPS_OK;
}
