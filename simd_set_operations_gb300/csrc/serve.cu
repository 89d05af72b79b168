// serve.cu -- serving k-set queries against a resident posting-list index,
// with continuous batching (setops_srv_*), and an open-loop Poisson load
// runner for measuring it.
//
// A query names k lists of the index; its answer is their intersection,
// computed smallest-first like the reference's svs_generic
// (setops/src/intersect/svs.rs:50-73) with naive_merge semantics per step.
//
// One server thread owns two batch slots, each with its own CUDA stream and
// scratch.  Whenever a slot is free and queries are waiting, it admits
// waiting queries in arrival order while their scratch fits the slot's share
// of the memory budget, and runs the batch asynchronously on the slot's
// stream:
//   step s = 1 .. kmax-1: one batched launch (batch.cuh) intersecting, for
//     every query with k > s, its running result (step 1: its smallest list)
//     with its next list; results alternate between two device pools;
//   then a scan of the final lengths and a gather kernel that write every
//     query's answer, compacted, straight into mapped pinned host memory.
// A host callback at the end of the stream wakes the server thread, which
// hands the answers to the completed queue.  With two slots a batch is
// admitted and launched while the previous one is still on the GPU.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "batch.cuh"
#include "runtime.h"
#include "setops_bench.h"
#include "setops_gpu.h"

using namespace setops;

namespace {

constexpr int kMaxK = 16;
constexpr int kSlots = 2;
constexpr size_t kMaxBatch = 1 << 16;

uint64_t now_ns() {
  return uint64_t(std::chrono::duration_cast<std::chrono::nanoseconds>(
                      std::chrono::steady_clock::now().time_since_epoch())
                      .count());
}

// Final lengths -> compact result offsets; counts and offsets to host.
template <int NT>
__global__ void __launch_bounds__(NT) serve_scan_kernel(uint32_t n, const uint32_t *ks,
                                                        uint64_t *const *lens_by_step,
                                                        uint64_t *res_off, uint64_t *h_counts,
                                                        uint64_t *h_total) {
  constexpr int NW = NT / 32;
  __shared__ unsigned long long ws[NW];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  unsigned long long base = 0;
  for (uint32_t c0 = 0; c0 < n; c0 += NT) {
    const uint32_t q = c0 + uint32_t(t);
    unsigned long long v = 0;
    if (q < n) v = lens_by_step[ks[q] - 2][q];  // the last step is k - 1 (index k - 2)
    unsigned long long incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) ws[warp] = incl;
    __syncthreads();
    unsigned long long before = 0, tot = 0;
#pragma unroll
    for (int k = 0; k < NW; ++k) {
      before += (k < warp) ? ws[k] : 0ull;
      tot += ws[k];
    }
    if (q < n) {
      res_off[q] = base + before + incl - v;
      h_counts[q] = v;
    }
    base += tot;
    __syncthreads();
  }
  if (t == 0) *h_total = base;
}

// Copies each query's answer (in the pool its last step wrote) to the
// compact host buffer.  One warp per query.
__global__ void serve_gather_kernel(uint32_t n, const uint32_t *ks, const uint64_t *inter_off,
                                    const uint32_t *inter0, const uint32_t *inter1,
                                    uint64_t *const *lens_by_step, const uint64_t *res_off,
                                    uint32_t *h_res) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t w0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t q = w0; q < n; q += nw) {
    const uint32_t k = ks[q];
    const uint64_t c = lens_by_step[k - 2][q];
    // step s writes pool (s & 1): step k - 1 wrote pool ((k - 1) & 1)
    const uint32_t *src = (((k - 1) & 1) ? inter1 : inter0) + inter_off[q];
    uint32_t *dst = h_res + res_off[q];
    for (uint64_t i = lane; i < c; i += 32) dst[i] = src[i];
  }
}

struct Query {
  uint64_t tag;
  uint32_t k;
  uint32_t ids[kMaxK];
  uint64_t t_submit;
};

struct Done {
  uint64_t tag;
  std::vector<uint32_t> res;
  uint64_t latency_ns;
};

struct Slot {
  cudaStream_t st = nullptr;
  bool busy = false;
  bool finished = false;  // set by the stream callback
  uint64_t seq = 0;       // launch order
  std::vector<Query> qs;
  void *dmem = nullptr;   // device scratch
  size_t dcap = 0;
  void *hmem = nullptr;   // pinned host: arrays to upload
  size_t hcap = 0;
  void *hres = nullptr;   // mapped pinned host: counts, offsets, answers
  size_t hres_cap = 0;
  uint64_t *h_counts = nullptr;
  uint64_t *h_total = nullptr;
  uint32_t *h_res = nullptr;
  std::vector<uint64_t> res_off_host;
};

}  // namespace

struct setops_srv {
  setops_ctx *ctx = nullptr;
  int device = 0;
  const uint32_t *pool = nullptr;  // device index
  std::vector<uint64_t> offs, lens;  // host copies (for planning)
  void *owned = nullptr;           // index copied to the device by the server
  size_t budget = 0;
  std::thread th;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Query> pending;
  std::deque<Done> done;
  bool stop = false;
  int err = SETOPS_OK;
  std::string errmsg;
  Slot slots[kSlots];
  uint64_t seq = 0;
  uint64_t batches = 0, queries = 0, max_batch = 0;
  uint64_t launches = 0;  // server thread only
  // batch kernel (materialise) fixed at start: entry, block, shared memory,
  // resident grid
  const void *kfn = nullptr;
  int knt = 0;
  size_t ksmem = 0;
  uint64_t grid = 1;
};

namespace {

void CUDART_CB slot_done(void *arg) {
  auto *pr = static_cast<std::pair<setops_srv *, int> *>(arg);
  setops_srv *srv = pr->first;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->slots[pr->second].finished = true;
  }
  srv->cv.notify_all();
}

std::pair<setops_srv *, int> g_cb_args[64][kSlots];  // stable callback arguments

int grow_device(Slot &s, size_t bytes) {
  if (s.dcap >= bytes) return SETOPS_OK;
  if (s.dmem) cudaFree(s.dmem);
  s.dmem = nullptr;
  s.dcap = 0;
  size_t b = std::max<size_t>(bytes, size_t(1) << 20);
  if (cudaMalloc(&s.dmem, b) != cudaSuccess) return SETOPS_ERR_NOMEM;
  s.dcap = b;
  return SETOPS_OK;
}

int grow_host(void *&p, size_t &cap, size_t bytes, bool mapped) {
  if (cap >= bytes) return SETOPS_OK;
  if (p) cudaFreeHost(p);
  p = nullptr;
  cap = 0;
  size_t b = std::max<size_t>(bytes, size_t(1) << 20);
  if (cudaHostAlloc(&p, b, mapped ? cudaHostAllocMapped : cudaHostAllocDefault) != cudaSuccess)
    return SETOPS_ERR_NOMEM;
  cap = b;
  return SETOPS_OK;
}

inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

// Runs one batch asynchronously on slot `si`.
int launch(setops_srv *srv, int si) {
  Slot &s = srv->slots[si];
  const uint32_t n = uint32_t(s.qs.size());
  uint32_t kmax = 2;
  for (auto &q : s.qs) kmax = std::max(kmax, q.k);
  const uint32_t steps = kmax - 1;
  // plan: smallest list first; capacity of a query = its smallest list
  std::vector<uint64_t> cap(n), ioff(n);
  uint64_t total = 0;
  for (uint32_t i = 0; i < n; ++i) {
    Query &q = s.qs[i];
    std::stable_sort(q.ids, q.ids + q.k,
                     [&](uint32_t x, uint32_t y) { return srv->lens[x] < srv->lens[y]; });
    cap[i] = srv->lens[q.ids[0]];
    ioff[i] = total;
    total += cap[i];
  }
  // host arrays (pinned): ks, inter_off, a_off_1, a_len_1, then per step
  // b_off_s, b_len_s
  const size_t nb8 = size_t(n) * 8;
  const size_t off_ks = 0, off_ioff = align16(size_t(n) * 4), off_aoff = off_ioff + align16(nb8);
  const size_t off_alen = off_aoff + align16(nb8), off_steps = off_alen + align16(nb8);
  const size_t step_bytes = 2 * align16(nb8);
  const size_t up_bytes = off_steps + steps * step_bytes;
  if (grow_host(s.hmem, s.hcap, up_bytes, false)) return SETOPS_ERR_NOMEM;
  char *h = static_cast<char *>(s.hmem);
  uint32_t *h_ks = reinterpret_cast<uint32_t *>(h + off_ks);
  uint64_t *h_ioff = reinterpret_cast<uint64_t *>(h + off_ioff);
  uint64_t *h_aoff = reinterpret_cast<uint64_t *>(h + off_aoff);
  uint64_t *h_alen = reinterpret_cast<uint64_t *>(h + off_alen);
  for (uint32_t i = 0; i < n; ++i) {
    const Query &q = s.qs[i];
    h_ks[i] = q.k;
    h_ioff[i] = ioff[i];
    h_aoff[i] = srv->offs[q.ids[0]];
    h_alen[i] = srv->lens[q.ids[0]];
  }
  for (uint32_t st = 1; st <= steps; ++st) {
    uint64_t *boff = reinterpret_cast<uint64_t *>(h + off_steps + (st - 1) * step_bytes);
    uint64_t *blen = reinterpret_cast<uint64_t *>(h + off_steps + (st - 1) * step_bytes + align16(nb8));
    for (uint32_t i = 0; i < n; ++i) {
      const Query &q = s.qs[i];
      const bool live = st < q.k;  // finished queries pair with an empty list
      boff[i] = live ? srv->offs[q.ids[st]] : 0;
      blen[i] = live ? srv->lens[q.ids[st]] : 0;
    }
  }
  // device scratch: uploaded arrays, per-step lengths, their pointer table,
  // result offsets, two result pools
  const size_t off_lens = align16(up_bytes);
  const size_t off_tab = off_lens + steps * align16(nb8);
  const size_t off_roff = off_tab + align16(kMaxK * 8);
  const size_t off_i0 = off_roff + align16(nb8);
  const size_t off_i1 = off_i0 + align16(total * 4 + 16);
  // long queries: each step's pairs split into units over CTAs (the map is
  // rebuilt on the device per step; a step's smaller lengths are bounded by
  // the queries' smallest lists)
  uint64_t maxcap = 0;
  for (uint32_t i = 0; i < n; ++i) maxcap = std::max(maxcap, cap[i]);
  const uint64_t unit_cap = maxcap > kBatchUnit ? unit_room(n, total) : 0;
  const size_t off_units = off_i1 + align16(total * 4 + 16);
  const size_t dbytes = off_units + (unit_cap ? prefix_bytes(n, unit_cap) : 0);
  if (grow_device(s, dbytes)) return SETOPS_ERR_NOMEM;
  // mapped host results: counts, total, answers
  const size_t hr_bytes = align16(nb8) + 16 + align16(total * 4 + 16);
  if (grow_host(s.hres, s.hres_cap, hr_bytes, true)) return SETOPS_ERR_NOMEM;
  char *hr = static_cast<char *>(s.hres);
  s.h_counts = reinterpret_cast<uint64_t *>(hr);
  s.h_total = reinterpret_cast<uint64_t *>(hr + align16(nb8));
  s.h_res = reinterpret_cast<uint32_t *>(hr + align16(nb8) + 16);
  void *dres = nullptr;
  if (cudaHostGetDevicePointer(&dres, s.hres, 0) != cudaSuccess) return SETOPS_ERR_CUDA;
  char *dr = static_cast<char *>(dres);
  uint64_t *d_counts_h = reinterpret_cast<uint64_t *>(dr);
  uint64_t *d_total_h = reinterpret_cast<uint64_t *>(dr + align16(nb8));
  uint32_t *d_res_h = reinterpret_cast<uint32_t *>(dr + align16(nb8) + 16);

  char *d = static_cast<char *>(s.dmem);
  cudaStream_t st = s.st;
  if (cudaMemcpyAsync(d, h, up_bytes, cudaMemcpyHostToDevice, st) != cudaSuccess) return SETOPS_ERR_CUDA;
  uint64_t *lens_dev[kMaxK] = {};
  for (uint32_t k = 0; k < steps; ++k) lens_dev[k] = reinterpret_cast<uint64_t *>(d + off_lens + k * align16(nb8));
  if (cudaMemcpyAsync(d + off_tab, lens_dev, sizeof(lens_dev), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return SETOPS_ERR_CUDA;
  const uint32_t *d_ks = reinterpret_cast<const uint32_t *>(d + off_ks);
  const uint64_t *d_ioff = reinterpret_cast<const uint64_t *>(d + off_ioff);
  const uint64_t *d_aoff = reinterpret_cast<const uint64_t *>(d + off_aoff);
  const uint64_t *d_alen = reinterpret_cast<const uint64_t *>(d + off_alen);
  uint32_t *inter[2] = {reinterpret_cast<uint32_t *>(d + off_i0), reinterpret_cast<uint32_t *>(d + off_i1)};
  setops_ctx *ctx = srv->ctx;
  for (uint32_t k = 1; k <= steps; ++k) {
    BatchArgs a{};
    a.pool = (k == 1) ? srv->pool : inter[(k - 1) & 1];
    a.pool_b = srv->pool;
    a.a_off = (k == 1) ? d_aoff : d_ioff;
    a.a_len = (k == 1) ? d_alen : lens_dev[k - 2];
    a.b_off = reinterpret_cast<const uint64_t *>(d + off_steps + (k - 1) * step_bytes);
    a.b_len = reinterpret_cast<const uint64_t *>(d + off_steps + (k - 1) * step_bytes + align16(nb8));
    a.npairs = n;
    a.out_off = d_ioff;
    a.out = inter[k & 1];
    a.out_lens = lens_dev[k - 1];
    a.search_ratio = ctx->batch_search_ratio;
    a.sync = ctx->sync + 2 + si;  // one coordination slot per batch slot
    a.err = ctx->derr;
    if (unit_cap) {
      launch_prefix(a.a_len, a.b_len, n, d + off_units, nullptr, nullptr, unit_cap, &a, st);
      srv->launches += 2;
    }
    void *args[] = {&a};
    const uint64_t work = std::max<uint64_t>(n, unit_cap);
    if (cudaLaunchKernel(srv->kfn, dim3(unsigned(std::min<uint64_t>(srv->grid, work))),
                         dim3(srv->knt), args, srv->ksmem, st) != cudaSuccess)
      return SETOPS_ERR_CUDA;
    ++srv->launches;
  }
  uint64_t *const *d_tab = reinterpret_cast<uint64_t *const *>(d + off_tab);
  uint64_t *d_roff = reinterpret_cast<uint64_t *>(d + off_roff);
  serve_scan_kernel<1024><<<1, 1024, 0, st>>>(n, d_ks, d_tab, d_roff, d_counts_h, d_total_h);
  const uint32_t gb = std::min<uint32_t>((n + 7) / 8, 1024);
  serve_gather_kernel<<<gb, 256, 0, st>>>(n, d_ks, d_ioff, inter[0], inter[1], d_tab, d_roff, d_res_h);
  if (cudaGetLastError() != cudaSuccess) return SETOPS_ERR_CUDA;
  srv->launches += 2;
  // result offsets come back with the answers: the host recomputes them
  // from the counts (same order, same sums)
  g_cb_args[srv->device][si] = {srv, si};
  if (cudaLaunchHostFunc(st, slot_done, &g_cb_args[srv->device][si]) != cudaSuccess)
    return SETOPS_ERR_CUDA;
  return SETOPS_OK;
}

// Hands a finished slot's answers to the completed queue (lock held by the
// caller is released around the copy).
void harvest(setops_srv *srv, int si, std::unique_lock<std::mutex> &lk) {
  Slot &s = srv->slots[si];
  std::vector<Query> qs;
  qs.swap(s.qs);
  lk.unlock();
  const uint64_t t = now_ns();
  std::vector<Done> out(qs.size());
  uint64_t off = 0;
  for (size_t i = 0; i < qs.size(); ++i) {
    const uint64_t c = s.h_counts[i];
    out[i].tag = qs[i].tag;
    out[i].res.assign(s.h_res + off, s.h_res + off + c);
    out[i].latency_ns = t - qs[i].t_submit;
    off += c;
  }
  lk.lock();
  for (auto &d : out) srv->done.push_back(std::move(d));
  s.busy = false;
  s.finished = false;
}

void server_loop(setops_srv *srv) {
  cudaSetDevice(srv->device);
  std::unique_lock<std::mutex> lk(srv->mu);
  for (;;) {
    // completed slots first, oldest first
    for (;;) {
      int best = -1;
      for (int i = 0; i < kSlots; ++i)
        if (srv->slots[i].busy && srv->slots[i].finished &&
            (best < 0 || srv->slots[i].seq < srv->slots[best].seq))
          best = i;
      if (best < 0) break;
      harvest(srv, best, lk);
      srv->cv.notify_all();
    }
    int fs = -1;
    for (int i = 0; i < kSlots; ++i)
      if (!srv->slots[i].busy) fs = i;
    if (fs >= 0 && !srv->pending.empty() && srv->err == SETOPS_OK) {
      // admit queries in arrival order while their scratch fits the slot's
      // share of the budget (always at least one)
      Slot &s = srv->slots[fs];
      const size_t share = srv->budget / kSlots;
      size_t used = 0;
      while (!srv->pending.empty() && s.qs.size() < kMaxBatch) {
        const Query &q = srv->pending.front();
        uint64_t mn = ~0ull;
        for (uint32_t j = 0; j < q.k; ++j) mn = std::min(mn, srv->lens[q.ids[j]]);
        const size_t cost = 3 * mn * 4 + 64 * 8;  // two result pools + answer + arrays
        if (!s.qs.empty() && used + cost > share) break;
        used += cost;
        s.qs.push_back(q);
        srv->pending.pop_front();
      }
      s.busy = true;
      s.finished = false;
      s.seq = ++srv->seq;
      srv->batches += 1;
      srv->queries += s.qs.size();
      srv->max_batch = std::max<uint64_t>(srv->max_batch, s.qs.size());
      lk.unlock();
      const int rc = launch(srv, fs);
      lk.lock();
      if (rc != SETOPS_OK) {
        srv->err = rc;
        srv->errmsg = std::string("batch launch failed: ") + cudaGetErrorString(cudaGetLastError());
        s.busy = false;
        s.qs.clear();
      }
      continue;
    }
    bool any_busy = false;
    for (auto &s : srv->slots) any_busy |= s.busy;
    if (srv->stop && srv->pending.empty() && !any_busy) break;
    if (srv->err != SETOPS_OK && !any_busy) {
      srv->pending.clear();
      if (srv->stop) break;
    }
    srv->cv.wait(lk);
  }
}

}  // namespace

extern "C" {

int setops_srv_start(setops_ctx *ctx, const uint32_t *pool, size_t pool_len,
                     const uint64_t *offs, const uint64_t *lens, size_t nlists,
                     size_t scratch_budget, unsigned flags, setops_srv **out) {
  if (!ctx || !out || !pool || !offs || !lens || nlists == 0) return SETOPS_ERR_INVALID;
  if (ctx->device < 0 || ctx->device >= 64) return SETOPS_ERR_INVALID;
  auto *srv = new setops_srv();
  srv->ctx = ctx;
  srv->device = ctx->device;
  srv->budget = scratch_budget ? scratch_budget : (size_t(256) << 20);
  cudaSetDevice(ctx->device);
  srv->offs.resize(nlists);
  srv->lens.resize(nlists);
  const bool host = (flags & SETOPS_HOST) != 0;
  int rc = SETOPS_OK;
  if (host) {
    std::memcpy(srv->offs.data(), offs, nlists * 8);
    std::memcpy(srv->lens.data(), lens, nlists * 8);
    if (cudaMalloc(&srv->owned, std::max<size_t>(pool_len, 1) * 4) != cudaSuccess)
      rc = SETOPS_ERR_NOMEM;
    else if (cudaMemcpy(srv->owned, pool, pool_len * 4, cudaMemcpyHostToDevice) != cudaSuccess)
      rc = SETOPS_ERR_CUDA;
    srv->pool = static_cast<const uint32_t *>(srv->owned);
  } else {
    if (cudaMemcpy(srv->offs.data(), offs, nlists * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(srv->lens.data(), lens, nlists * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = SETOPS_ERR_CUDA;
    srv->pool = pool;
  }
  for (size_t i = 0; rc == SETOPS_OK && i < nlists; ++i)
    if (srv->offs[i] + srv->lens[i] > pool_len) rc = SETOPS_ERR_INVALID;
  for (int i = 0; rc == SETOPS_OK && i < kSlots; ++i)
    if (cudaStreamCreateWithFlags(&srv->slots[i].st, cudaStreamNonBlocking) != cudaSuccess)
      rc = SETOPS_ERR_CUDA;
  if (rc == SETOPS_OK) {
    // the batch kernel the policy names, sized once here (the server thread
    // touches no shared context state)
    const KernelInfo &k = batch_kernel_info(true, ctx->batch_variant);
    int occ = 1;
    rc = ctx_occupancy(ctx, k, &occ);
    srv->kfn = k.fn;
    srv->knt = k.nt;
    srv->ksmem = k.dyn_smem;
    srv->grid = uint64_t(std::max(occ, 1)) * uint64_t(ctx->sms);
  }
  if (rc != SETOPS_OK) {
    for (auto &s : srv->slots)
      if (s.st) cudaStreamDestroy(s.st);
    if (srv->owned) cudaFree(srv->owned);
    delete srv;
    return ctx_fail(ctx, rc, "setops_srv_start failed");
  }
  srv->th = std::thread(server_loop, srv);
  *out = srv;
  return SETOPS_OK;
}

int setops_srv_submit(setops_srv *srv, const uint32_t *list_ids, size_t k, uint64_t tag) {
  if (!srv || !list_ids || k < 2 || k > size_t(kMaxK)) return SETOPS_ERR_INVALID;
  Query q{};
  q.tag = tag;
  q.k = uint32_t(k);
  for (size_t j = 0; j < k; ++j) {
    if (list_ids[j] >= srv->lens.size()) return SETOPS_ERR_INVALID;
    q.ids[j] = list_ids[j];
  }
  q.t_submit = now_ns();
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    if (srv->stop) return SETOPS_ERR_BUSY;
    if (srv->err != SETOPS_OK) return srv->err;
    srv->pending.push_back(q);
  }
  srv->cv.notify_all();
  return SETOPS_OK;
}

int setops_srv_poll(setops_srv *srv, uint64_t *tag, uint32_t *out, size_t out_cap,
                    size_t *out_len, uint64_t *latency_ns) {
  if (!srv || !tag || !out_len) return SETOPS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(srv->mu);
  if (srv->done.empty()) return srv->err != SETOPS_OK ? srv->err : SETOPS_ERR_NOT_READY;
  Done &d = srv->done.front();
  *out_len = d.res.size();
  *tag = d.tag;
  if (latency_ns) *latency_ns = d.latency_ns;
  if (d.res.size() > out_cap) return SETOPS_ERR_CAPACITY;  // kept: retry with room
  if (!d.res.empty()) {
    if (!out) return SETOPS_ERR_INVALID;
    std::memcpy(out, d.res.data(), d.res.size() * 4);
  }
  srv->done.pop_front();
  return SETOPS_OK;
}

int setops_srv_stats(setops_srv *srv, uint64_t *batches, uint64_t *queries,
                     uint64_t *max_batch, uint64_t *launches) {
  if (!srv) return SETOPS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(srv->mu);
  if (batches) *batches = srv->batches;
  if (queries) *queries = srv->queries;
  if (max_batch) *max_batch = srv->max_batch;
  if (launches) *launches = srv->launches;
  return SETOPS_OK;
}

int setops_srv_stop(setops_srv *srv) {
  if (!srv) return SETOPS_ERR_INVALID;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stop = true;
  }
  srv->cv.notify_all();
  if (srv->th.joinable()) srv->th.join();
  const int rc = srv->err;
  cudaSetDevice(srv->device);
  for (auto &s : srv->slots) {
    if (s.st) {
      cudaStreamSynchronize(s.st);
      cudaStreamDestroy(s.st);
    }
    if (s.dmem) cudaFree(s.dmem);
    if (s.hmem) cudaFreeHost(s.hmem);
    if (s.hres) cudaFreeHost(s.hres);
  }
  if (srv->owned) cudaFree(srv->owned);
  delete srv;
  return rc;
}

int setops_srv_run_load(setops_srv *srv, const uint32_t *ids, const uint32_t *ks,
                        size_t kstride, size_t nq, double rate_qps, uint64_t seed,
                        uint64_t *latency_ns, uint64_t *counts, uint32_t *answers,
                        size_t answer_stride, double *elapsed_s) {
  if (!srv || !ids || !ks || !latency_ns || nq == 0 || rate_qps <= 0 || kstride < 2)
    return SETOPS_ERR_INVALID;
  std::mt19937_64 rng(seed);
  std::exponential_distribution<double> gap(rate_qps);
  std::vector<uint64_t> due(nq), sent(nq);
  double t = 0;
  for (size_t q = 0; q < nq; ++q) {
    t += gap(rng);
    due[q] = uint64_t(t * 1e9);
  }
  std::vector<uint32_t> buf(1 << 16);
  size_t next = 0, got = 0;
  const uint64_t t0 = now_ns();
  auto drain = [&]() -> int {
    for (;;) {
      uint64_t tag = 0, lat = 0;
      size_t len = 0;
      int rc = setops_srv_poll(srv, &tag, buf.data(), buf.size(), &len, &lat);
      if (rc == SETOPS_ERR_CAPACITY) {
        buf.resize(len);
        rc = setops_srv_poll(srv, &tag, buf.data(), buf.size(), &len, &lat);
      }
      if (rc == SETOPS_ERR_NOT_READY) return SETOPS_OK;
      if (rc != SETOPS_OK) return rc;
      // open loop: latency counts from the query's scheduled arrival
      latency_ns[tag] = lat + (sent[tag] - (t0 + due[tag]));
      if (counts) counts[tag] = len;
      if (answers) {
        if (len > answer_stride) return SETOPS_ERR_CAPACITY;
        std::memcpy(answers + tag * answer_stride, buf.data(), len * sizeof(uint32_t));
      }
      ++got;
    }
  };
  while (got < nq) {
    const uint64_t now = now_ns();
    while (next < nq && now >= t0 + due[next]) {
      sent[next] = now_ns();
      const int rc = setops_srv_submit(srv, ids + next * kstride, ks[next], next);
      if (rc != SETOPS_OK) return rc;
      ++next;
    }
    const int rc = drain();
    if (rc != SETOPS_OK) return rc;
    if (next >= nq && got < nq) std::this_thread::yield();
  }
  if (elapsed_s) *elapsed_s = double(now_ns() - t0) * 1e-9;
  return SETOPS_OK;
}

}  // extern "C"
