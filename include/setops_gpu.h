/*
 * setops_gpu.h -- C ABI of the GB300 (sm_103a) sorted-u32 set-intersection
 * library (libsetops_gpu.so).
 *
 * This is the drop-in boundary for the hot path of the Rust crate `setops`
 * (UNSW-database/simd_set_operations).  Each entry point names the reference
 * interface it replaces.  The existing native boundary of that crate,
 * setops/ffi/qfilter/qfilter.h:8-39, sets the conventions kept here: plain
 * pointers and lengths, caller-owned output buffers, the result length as the
 * return channel.
 *
 * Conventions
 *   - Sets are strictly increasing arrays of uint32_t (unsigned order).  As in
 *     the reference, results on unsorted or duplicated input are unspecified;
 *     setops_gpu_validate_sorted() checks an input.
 *   - Materialising calls need out_cap >= min(|A|, |B|) (the reference's
 *     Intersect2C / UnsafeWriter convention: setops/src/intersect.rs:54-67,
 *     setops/src/intersect/qfilter_c.rs:11); otherwise SETOPS_ERR_CAPACITY.
 *   - Every call returns a status (0 = OK, negative = error) instead of the
 *     reference's assert!/abort.  setops_gpu_last_error() gives the text.
 *   - flags: SETOPS_HOST means every set/output pointer of the call is host
 *     memory (the call copies in and out and returns when done; pinned memory
 *     gives full copy speed).  Without it the pointers are device pointers.
 *     Device-pointer calls still return their length/count to host memory and
 *     synchronise, except the *_async calls.
 *   - A context serialises its work on one CUDA stream; calls on one context
 *     must not overlap from several host threads.  Distinct contexts are
 *     independent.
 */
#ifndef SETOPS_GPU_H
#define SETOPS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
enum {
  SETOPS_OK = 0,
  SETOPS_ERR_INVALID = -1,   /* bad argument (NULL pointer, k < 2, ...)       */
  SETOPS_ERR_CAPACITY = -2,  /* output capacity below min(|A|, |B|)           */
  SETOPS_ERR_CUDA = -3,      /* CUDA runtime error                           */
  SETOPS_ERR_NOMEM = -4,     /* device or pinned allocation failed           */
  SETOPS_ERR_TIMEOUT = -5,   /* a device-side wait hit its iteration limit   */
  SETOPS_ERR_UNSORTED = -6,  /* reserved for validation failures             */
  SETOPS_ERR_BUSY = -7,      /* serving queue full / call in progress        */
  SETOPS_ERR_TOO_LARGE = -8, /* input larger than an entry point supports    */
  SETOPS_ERR_NOT_READY = -9  /* serving: no completed query to return        */
};

/* ---- flags -------------------------------------------------------------- */
#define SETOPS_HOST 0x1u             /* pointers are host memory            */
/* Algorithm override (default: the tuned choice for the size ratio). */
#define SETOPS_ALGO_SHIFT 8
#define SETOPS_ALGO_MASK (0xffu << SETOPS_ALGO_SHIFT)
#define SETOPS_ALGO_AUTO (0u << SETOPS_ALGO_SHIFT)
#define SETOPS_ALGO_MERGE (1u << SETOPS_ALGO_SHIFT)  /* merge-path kernel    */
#define SETOPS_ALGO_GALLOP (2u << SETOPS_ALGO_SHIFT) /* search kernel        */
#define SETOPS_ALGO_BITMAP (3u << SETOPS_ALGO_SHIFT) /* tiled bitmap kernel  */
/* Variant of the chosen kernel (tile shape / probe group); 0 = default.
 * setops_gpu_num_variants() gives the count per algorithm.  For BSR sets,
 * SETOPS_ALGO_MERGE variant 3 is the block-broadcast kernel (32-word blocks
 * compared all against all, the scheme of broadcast_*_bsr,
 * setops/src/intersect/broadcast.rs:163-357); it is the BSR default for
 * size ratios below 32. */
#define SETOPS_VARIANT_SHIFT 16
#define SETOPS_VARIANT_MASK (0xffu << SETOPS_VARIANT_SHIFT)
#define SETOPS_VARIANT(v) (((unsigned)(v) & 0xffu) << SETOPS_VARIANT_SHIFT)

typedef struct setops_ctx setops_ctx;

/* ---- context ------------------------------------------------------------ */
/* Creates a context on CUDA device `device` with its own stream, scratch
 * pool and tuning table.  (The reference has no context: its functions are
 * pure CPU functions, setops/src/intersect.rs:40-42.) */
int setops_gpu_create(setops_ctx **out, int device);
int setops_gpu_destroy(setops_ctx *ctx);
/* Use an external CUDA stream (cudaStream_t) for all later work; NULL
 * restores the context's own stream. */
int setops_gpu_set_stream(setops_ctx *ctx, void *cuda_stream);
void *setops_gpu_get_stream(setops_ctx *ctx);
/* Waits for all queued work; reports device-side errors of async calls. */
int setops_gpu_synchronize(setops_ctx *ctx);
const char *setops_gpu_last_error(const setops_ctx *ctx);
const char *setops_status_string(int status);
/* Number of kernel variants of an algorithm (SETOPS_ALGO_MERGE / _GALLOP /
 * _BITMAP) for the given element kind (0 = u32 arrays, 1 = BSR; the bitmap
 * kernel has no BSR variant, and a BSR call asking for it gets the merge). */
int setops_gpu_num_variants(unsigned algo, int bsr);
/* Number of kernels this context has launched (for launch accounting). */
uint64_t setops_gpu_launch_count(const setops_ctx *ctx);

/* Bounded device waits (no counterpart: the reference runs on the CPU and
 * never waits on a GPU).  Every spin-wait in this library's kernels (a bulk
 * copy's barrier, a predecessor's published count, a grid-wide flag) gives
 * up after a time limit, records the fact and returns, so that the call
 * fails with SETOPS_ERR_TIMEOUT instead of hanging the GPU; the context
 * stays usable.  setops_gpu_set_wait_limit_ns sets that limit in
 * nanoseconds (0 = the default, 2 s) for every context on ctx's device; call
 * it while no work of this library runs on that device.
 * setops_gpu_check_wait_limit runs one wait that nothing ever satisfies and
 * returns SETOPS_ERR_TIMEOUT when the limit ended it, with *waited_ns the
 * time the device waited. */
int setops_gpu_set_wait_limit_ns(setops_ctx *ctx, uint64_t ns);
int setops_gpu_check_wait_limit(setops_ctx *ctx, uint64_t *waited_ns);
/* Algorithm policy: the kernel used for pairs whose size ratio max/min lies
 * in [2^band, 2^(band+1)), band in [0, 32); algo_flags = SETOPS_ALGO_MERGE,
 * SETOPS_ALGO_GALLOP or SETOPS_ALGO_BITMAP (arrays only) | SETOPS_VARIANT(v).
 * The autotuner writes this table;
 * it plays the role of the reference's compile-time choice of algorithm per
 * ISA (setops/src/intersect.rs:26-36) and the benchmark's name registry
 * (benchmark/src/timer.rs:75-169). */
int setops_gpu_set_policy(setops_ctx *ctx, int bsr, int ratio_band,
                          unsigned algo_flags);
int setops_gpu_get_policy(const setops_ctx *ctx, int bsr, int ratio_band,
                          unsigned *algo_flags);
/* The policy table is kept per size class of the pair's smaller input as
 * well: [0, 2^12), [2^12, 2^16), [2^16, 2^22) and [2^22, ...) elements
 * (size_class 0-3).  setops_gpu_set_policy sets a band's four classes at
 * once and setops_gpu_get_policy reads its class 3; these set and read one
 * cell. */
#define SETOPS_SIZE_CLASSES 4
int setops_gpu_set_policy_class(setops_ctx *ctx, int bsr, int ratio_band, int size_class,
                                unsigned algo_flags);
int setops_gpu_get_policy_class(const setops_ctx *ctx, int bsr, int ratio_band,
                                int size_class, unsigned *algo_flags);
/* The autotuner of the array table (the reference's counterpart is its
 * compile-time choice of algorithm per instruction set,
 * setops/src/intersect.rs:26-36).  For every ratio band in [band_lo,
 * band_hi] and size class whose test pair fits max_elems elements (smaller
 * set 2^10, 2^14, 2^19 or 2^23 elements, larger 1.4 * 2^band times that),
 * generates a seeded pair at `density` with 1 % matches, times every
 * algorithm and kernel variant on it (reps back-to-back materialising
 * launches, CUDA events), requires every candidate to find the same number
 * of matches (else SETOPS_ERR_CUDA), and writes the fastest into the table.
 * *tuned (optional) gets the number of cells written.  Takes seconds; run it
 * once per GPU and keep the table (setops_gpu_get_policy_class). */
int setops_gpu_autotune(setops_ctx *ctx, int band_lo, int band_hi, size_t max_elems,
                        double density, int reps, int *tuned);
/* The same for the BSR table: each cell's pair is generated as arrays (at
 * most max_elems elements), encoded to BSR words on the device, and every
 * BSR candidate (merge-family variants, among them the block-broadcast
 * kernel, and search variants) is timed; all must give the same result
 * words.  Bands and size classes are by word count, as the BSR choice is. */
int setops_gpu_autotune_bsr(setops_ctx *ctx, int band_lo, int band_hi, size_t max_elems,
                            double density, int reps, int *tuned);
/* A text naming the GPU and driver (for keying a saved policy table). */
int setops_gpu_device_key(setops_ctx *ctx, char *buf, size_t cap);

/* ---- 2-set, u32 arrays --------------------------------------------------
 * Replace `Intersect2<[u32], V> = fn(&[u32], &[u32], &mut V)`
 * (setops/src/intersect.rs:40) with V = Counter (setops/src/visitor.rs:24)
 * and V = VecWriter / SliceWriter / UnsafeWriter (visitor.rs:51,100,759), and
 * `Intersect2C<[u32]>` (intersect.rs:41); results equal naive_merge
 * (setops/src/intersect/merge.rs:7-33). */
int setops_gpu_intersect_count(setops_ctx *ctx, const uint32_t *a, size_t na,
                               const uint32_t *b, size_t nb, uint64_t *count,
                               unsigned flags);
int setops_gpu_intersect(setops_ctx *ctx, const uint32_t *a, size_t na,
                         const uint32_t *b, size_t nb, uint32_t *out,
                         size_t out_cap, size_t *out_len, unsigned flags);
/* Device-only, no synchronisation: the result length (or count, when out is
 * NULL) is written to the device word *len_dev.  Errors surface at
 * setops_gpu_synchronize(). */
int setops_gpu_intersect_async(setops_ctx *ctx, const uint32_t *a, size_t na,
                               const uint32_t *b, size_t nb, uint32_t *out,
                               size_t out_cap, uint64_t *len_dev,
                               unsigned flags);
/* npairs independent pairs in host memory (flags must include SETOPS_HOST):
 * pair i is a[i] (na[i] elements) and b[i] (nb[i]); its result goes to
 * out[i] (out_cap[i] >= min(na[i], nb[i])) and its length to out_len[i] --
 * for every pair exactly what setops_gpu_intersect gives.  The reference has
 * one Intersect2C call per pair (setops/src/intersect.rs:41); one call for
 * many lets the search-band pairs with pinned inputs and outputs, read in
 * place, run while the other pairs' inputs are copied over the host link.
 * Synchronous; pairs with a pageable output are intersected one call each
 * after the rest. */
int setops_gpu_intersect_pairs(setops_ctx *ctx, size_t npairs,
                               const uint32_t *const *a, const size_t *na,
                               const uint32_t *const *b, const size_t *nb,
                               uint32_t *const *out, const size_t *out_cap,
                               size_t *out_len, unsigned flags);

/* ---- 2-set, BSR (base-and-state) -----------------------------------------
 * Replace `Intersect2Bsr = fn(BsrRef, BsrRef, &mut BsrVec)`
 * (setops/src/bsr.rs:16) and the BSR Counter (setops/src/visitor.rs:399-403);
 * results equal branchless_merge_bsr (setops/src/intersect/merge.rs:62-87).
 * A BSR set is SoA: bases[] strictly increasing, states[] non-zero.
 * _count gives the element count (sum of popcount of the AND-ed states);
 * the materialising call gives the (base, state) words with a non-zero AND,
 * out_cap >= min(na, nb) words. */
int setops_gpu_intersect_bsr_count(setops_ctx *ctx, const uint32_t *bases_a,
                                   const uint32_t *states_a, size_t na,
                                   const uint32_t *bases_b,
                                   const uint32_t *states_b, size_t nb,
                                   uint64_t *count, unsigned flags);
int setops_gpu_intersect_bsr(setops_ctx *ctx, const uint32_t *bases_a,
                             const uint32_t *states_a, size_t na,
                             const uint32_t *bases_b, const uint32_t *states_b,
                             size_t nb, uint32_t *out_bases,
                             uint32_t *out_states, size_t out_cap,
                             size_t *out_len, unsigned flags);
/* BsrVec::from_sorted (setops/src/bsr.rs:140-163) on the device: encodes a
 * sorted set of n elements into *nwords (base, state) words; bases/states
 * need room for n words. */
int setops_gpu_bsr_from_sorted(setops_ctx *ctx, const uint32_t *in, size_t n,
                               uint32_t *bases, uint32_t *states,
                               size_t *nwords, unsigned flags);
/* BsrVec::to_sorted_set (setops/src/bsr.rs:77-88) on the device; out needs
 * room for the popcount total (<= 32 * n). */
int setops_gpu_bsr_to_sorted(setops_ctx *ctx, const uint32_t *bases,
                             const uint32_t *states, size_t n, uint32_t *out,
                             size_t out_cap, size_t *out_len, unsigned flags);

/* ---- k-set SvS -----------------------------------------------------------
 * Replace svs_generic (setops/src/intersect/svs.rs:50-73) / run_svs
 * (svs.rs:103-116) and `IntersectK` (setops/src/intersect.rs:42).  Sets are
 * intersected smallest-first (the reference assumes the caller ordered them,
 * svs.rs:7; intersection is order-independent, so the result is the same);
 * intermediate results stay on the device.  out_cap >= min(lens). */
int setops_gpu_svs(setops_ctx *ctx, const uint32_t *const *sets,
                   const size_t *lens, size_t k, uint32_t *out,
                   size_t out_cap, size_t *out_len, unsigned flags);
int setops_gpu_svs_count(setops_ctx *ctx, const uint32_t *const *sets,
                         const size_t *lens, size_t k, uint64_t *count,
                         unsigned flags);
/* Device arrays only, no synchronisation: the result length goes to the
 * device word *len_dev (like setops_gpu_intersect_async); errors surface at
 * setops_gpu_synchronize().  out == NULL: the count goes to *len_dev.  The
 * set pointer and length arrays are host arrays (read during the call). */
int setops_gpu_svs_async(setops_ctx *ctx, const uint32_t *const *sets,
                         const size_t *lens, size_t k, uint32_t *out,
                         size_t out_cap, uint64_t *len_dev, unsigned flags);
/* k-set intersection by the small_adaptive scheme (the reference's
 * small_adaptive, setops/src/intersect/adaptive.rs:107-148, an IntersectK,
 * setops/src/intersect.rs:42): every element of the smallest set is looked
 * up in the other sets, smallest first, and dropped at the first one that
 * lacks it, so the larger sets are read only where the survivors lie.  Same
 * arguments and result as setops_gpu_svs (out_cap >= the smallest length;
 * SETOPS_HOST for host arrays); k <= 16. */
int setops_gpu_adaptive(setops_ctx *ctx, const uint32_t *const *sets, const size_t *lens,
                        size_t k, uint32_t *out, size_t out_cap, size_t *out_len,
                        unsigned flags);
int setops_gpu_adaptive_count(setops_ctx *ctx, const uint32_t *const *sets, const size_t *lens,
                              size_t k, uint64_t *count, unsigned flags);

/* ---- batched 2-set --------------------------------------------------------
 * Many independent pairs in one launch.  Replaces a loop of Intersect2 /
 * Intersect2C calls over a dataset's pairs (setops/src/intersect.rs:40-41;
 * the benchmark's per-pair loop, benchmark/src/timer/harness.rs:35-97).  All
 * sets live in one pool: pair p is pool[a_off[p], +a_len[p]) and
 * pool[b_off[p], +b_len[p]), each strictly increasing.  The intersection of
 * pair p (as naive_merge, setops/src/intersect/merge.rs:7-33) goes to
 * out[out_off[p], +min(a_len[p], b_len[p])) and its length to out_lens[p].
 * out_off == NULL: the offsets are the running sum of min(a_len, b_len)
 * (then out_cap must cover that sum; otherwise SETOPS_ERR_CAPACITY).  With
 * caller offsets on the device the regions are the caller's responsibility.
 * flags: SETOPS_HOST = every array is host memory.  The kernel shape and the
 * size ratio from which a pair takes the search path instead of the tile
 * path come from the batch policy (setops_gpu_batch_set_policy, or the
 * autotuner).  The calls return when the batch is done. */
int setops_gpu_batch_intersect(setops_ctx *ctx, const uint32_t *pool, size_t pool_len,
                               const uint64_t *a_off, const uint64_t *a_len,
                               const uint64_t *b_off, const uint64_t *b_len, size_t npairs,
                               uint32_t *out, size_t out_cap, const uint64_t *out_off,
                               uint64_t *out_lens, unsigned flags);
/* Counter visitor per pair (setops/src/visitor.rs:24-49): counts[p]. */
int setops_gpu_batch_count(setops_ctx *ctx, const uint32_t *pool, size_t pool_len,
                           const uint64_t *a_off, const uint64_t *a_len, const uint64_t *b_off,
                           const uint64_t *b_len, size_t npairs, uint64_t *counts,
                           unsigned flags);
/* Batch policy: kernel shape (0 .. setops_gpu_batch_num_variants()-1) and
 * search ratio (pairs with max/min >= ratio take the search path; 0 = never). */
int setops_gpu_batch_set_policy(setops_ctx *ctx, int variant, uint32_t search_ratio);
int setops_gpu_batch_get_policy(const setops_ctx *ctx, int *variant, uint32_t *search_ratio);
int setops_gpu_batch_num_variants(void);
/* The same batch for BSR sets (Intersect2Bsr per pair, setops/src/bsr.rs:16;
 * result = branchless_merge_bsr, setops/src/intersect/merge.rs:62-87): every
 * set is (bases[off, +len), states[off, +len)) of one pool, lengths and
 * offsets in words; pair p's result words go to out_bases/out_states at
 * out_off[p] (NULL: offsets from a device scan of min(a_len, b_len)), its
 * word count to out_lens[p].  Capacity per pair: min(a_len, b_len) words. */
int setops_gpu_batch_intersect_bsr(setops_ctx *ctx, const uint32_t *bases,
                                   const uint32_t *states, size_t pool_len,
                                   const uint64_t *a_off, const uint64_t *a_len,
                                   const uint64_t *b_off, const uint64_t *b_len, size_t npairs,
                                   uint32_t *out_bases, uint32_t *out_states, size_t out_cap,
                                   const uint64_t *out_off, uint64_t *out_lens, unsigned flags);
/* Counter visitor per BSR pair (popcount sums, setops/src/visitor.rs:399-403). */
int setops_gpu_batch_count_bsr(setops_ctx *ctx, const uint32_t *bases, const uint32_t *states,
                               size_t pool_len, const uint64_t *a_off, const uint64_t *a_len,
                               const uint64_t *b_off, const uint64_t *b_len, size_t npairs,
                               uint64_t *counts, unsigned flags);
/* Steady-state replay.  A batch on DEVICE arrays captured once into a CUDA
 * graph (the offset scan when out_off is NULL, then the batch kernel, with
 * the context's batch policy at creation) and replayed by plan_launch on the
 * context's stream: no host work or synchronisation per replay.  The caller
 * may rewrite the arrays' contents between replays (same pointers, same
 * npairs).  The output capacity is checked on the device; an overflowing
 * pair records SETOPS_ERR_CAPACITY (reported by the next synchronising call,
 * e.g. setops_gpu_synchronize) and gets length 0.  out == NULL captures the
 * count form.  The plan owns its coordination words and offsets, so other
 * calls on the context may run between replays (not concurrently).  No
 * counterpart in the reference; it replaces a loop of batch calls. */
typedef struct setops_batch_plan setops_batch_plan;
int setops_gpu_batch_plan_create(setops_ctx *ctx, const uint32_t *pool, size_t pool_len,
                                 const uint64_t *a_off, const uint64_t *a_len,
                                 const uint64_t *b_off, const uint64_t *b_len, size_t npairs,
                                 uint32_t *out, size_t out_cap, const uint64_t *out_off,
                                 uint64_t *out_lens, setops_batch_plan **plan);
int setops_gpu_batch_plan_launch(setops_batch_plan *plan);
int setops_gpu_batch_plan_destroy(setops_batch_plan *plan);
/* Autotuner: times every kernel shape with several search ratios on the
 * given sample batch (materialising, `reps` timed runs each) and keeps the
 * fastest as the batch policy.  Plays the role of the reference's per-ISA
 * choice of algorithm (setops/src/intersect.rs:26-36). */
int setops_gpu_batch_autotune(setops_ctx *ctx, const uint32_t *pool, size_t pool_len,
                              const uint64_t *a_off, const uint64_t *a_len,
                              const uint64_t *b_off, const uint64_t *b_len, size_t npairs,
                              int reps, unsigned flags);

/* ---- serving k-set queries against a resident index ----------------------
 * No single counterpart in the reference: it serves run_svs / svs_generic
 * (setops/src/intersect/svs.rs:50-73,103-116) over a posting-list index, the
 * way a search engine would call it, with continuous batching.  The index is
 * a pool of sorted lists: list i is pool[offs[i], +lens[i]) (flags
 * SETOPS_HOST: host arrays, copied to the device; else device arrays, which
 * must outlive the server).  A query names k in [2, 16] list ids; its answer
 * is their ascending intersection (svs_generic with naive_merge semantics).
 * A server thread admits waiting queries into batches while their scratch
 * fits `scratch_budget` bytes (0: 256 MiB) and keeps up to two batches on
 * the GPU at once; queries arriving while a batch runs join the next one.
 * submit is non-blocking and thread-safe; poll returns one finished query
 * (tag, answer, latency from submit to completion) or SETOPS_ERR_NOT_READY;
 * SETOPS_ERR_CAPACITY leaves the answer queued and sets *out_len to its
 * size.  The server uses the context's device and batch policy; do not run
 * other calls on the same context concurrently with a server. */
typedef struct setops_srv setops_srv;
int setops_srv_start(setops_ctx *ctx, const uint32_t *pool, size_t pool_len,
                     const uint64_t *offs, const uint64_t *lens, size_t nlists,
                     size_t scratch_budget, unsigned flags, setops_srv **out);
int setops_srv_submit(setops_srv *srv, const uint32_t *list_ids, size_t k, uint64_t tag);
int setops_srv_poll(setops_srv *srv, uint64_t *tag, uint32_t *out, size_t out_cap,
                    size_t *out_len, uint64_t *latency_ns);
int setops_srv_stats(setops_srv *srv, uint64_t *batches, uint64_t *queries,
                     uint64_t *max_batch, uint64_t *launches);
/* Waits for every submitted query, stops the thread, frees the server. */
int setops_srv_stop(setops_srv *srv);

/* ---- 2-set without allocation ----------------------------------------------
 * No counterpart in the reference: it exists for callers of this library that
 * cannot allocate device memory -- a host program that owns all device
 * memory through its own pool, a latency-bound path that cannot take the
 * device-wide synchronisation and unbounded latency of cudaMalloc/cudaFree,
 * or a process whose GPU memory is already full.  The context API allocates
 * (at setops_gpu_create, and scratch that grows with the input); this call
 * allocates nothing and needs no context.
 *
 * Same result as setops_gpu_intersect on device pointers: a[0..na) and
 * b[0..nb) are device arrays, out (device) receives the ascending
 * intersection, out_cap >= min(na, nb), and *out_len (host) its length.  The
 * work runs on `stream` (a cudaStream_t; NULL = the default stream) on the
 * current device, and the call returns when it has finished.
 *
 * Its scratch is one fixed array that every GPU loading the library holds
 * until the process exits, which limits the smaller input to
 * SETOPS_NOALLOC_MAX_SMALL elements; larger calls return
 * SETOPS_ERR_TOO_LARGE.  All calls on a device share that array: calls that
 * overlapped on the GPU would race, so the call holds a per-device lock and
 * returns only when its work is done.  The first call on a device sets up
 * the array's device address (and the kernel's attributes); make that first
 * call before any stream capture.  That first call is also when the CUDA
 * runtime loads the array and the kernel onto the device (device code is
 * loaded on first use unless CUDA_MODULE_LOADING=EAGER), so it takes device
 * memory once: make it, with tiny inputs if need be, while the GPU still has
 * memory free.  Later calls allocate nothing. */
#define SETOPS_NOALLOC_MAX_SMALL ((size_t)1 << 20)
int setops_gpu_intersect_noalloc(const uint32_t *a, size_t na,
                                 const uint32_t *b, size_t nb, uint32_t *out,
                                 size_t out_cap, size_t *out_len,
                                 void *stream);

/* ---- validation ----------------------------------------------------------
 * *is_sorted = 1 when a[0..n) is strictly increasing (no counterpart: the
 * reference debug_asserts this, setops/src/bsr.rs:71-72). */
int setops_gpu_validate_sorted(setops_ctx *ctx, const uint32_t *a, size_t n,
                               int *is_sorted, unsigned flags);

#ifdef __cplusplus
}
#endif
#endif /* SETOPS_GPU_H */
