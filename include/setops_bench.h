/*
 * setops_bench.h -- benchmark-side helpers exported by libsetops_gpu.so:
 * seeded synthetic set generators and the reference's on-disk datafile
 * format.  Host code only; no GPU needed.
 *
 * The generators restate benchmark/src/generators.rs of
 * UNSW-database/simd_set_operations with a seeded PRNG (xoshiro256**, seeded
 * by SplitMix64) in place of the reference's unseeded thread_rng
 * (generators.rs:87), so inputs are reproducible; the value distributions and
 * the shared/unshared construction are the reference's.
 */
#ifndef SETOPS_BENCH_H
#define SETOPS_BENCH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* gen_twoset (benchmark/src/generators.rs:30-68) for explicit lengths:
 * max_value = floor(large_len / density); floor(selectivity * small_len)
 * shared elements plus disjoint fills, drawn without replacement from
 * [0, max_value) (shuffled_set, generators.rs:83-110), then sorted.  Returns
 * 0, or -1 on bad arguments. */
int setops_gen_twoset(uint64_t seed, double density, double selectivity,
                      size_t small_len, size_t large_len, uint32_t *small_out,
                      uint32_t *large_out);

/* Set lengths of gen_kset (generators.rs:112-135, get_skew :220-224):
 * lens[i] = max_len / floor((i+1)^skewness), listed smallest first (the
 * reference emits sets_count-1 .. 0). */
int setops_gen_kset_lens(size_t max_len, double skewness, size_t set_count,
                         size_t *lens);
/* gen_kset: every set contains floor(selectivity * smallest_len) shared
 * elements and uniform fill (sorted_set_containing, generators.rs:139-215);
 * outs[i] needs room for lens[i] from setops_gen_kset_lens. */
int setops_gen_kset(uint64_t seed, double density, double selectivity,
                    size_t max_len, double skewness, size_t set_count,
                    uint32_t *const *outs);

/* Batched uneven pairs: pair p has |A| and |B| each log-uniform in
 * [min_len, max_len], density U[dmin, dmax] (max_value = max(|A|,|B|) /
 * density) and selectivity U[smin, smax] of the smaller set.
 * setops_gen_batch_sizes draws the lengths; setops_gen_batch_fill writes
 * the sets into pool at the given offsets (nthreads workers; the output does
 * not depend on nthreads). */
int setops_gen_batch_sizes(uint64_t seed, size_t npairs, size_t min_len,
                           size_t max_len, uint64_t *a_len, uint64_t *b_len);
int setops_gen_batch_fill(uint64_t seed, size_t npairs, const uint64_t *a_len,
                          const uint64_t *b_len, const uint64_t *a_off,
                          const uint64_t *b_off, double dmin, double dmax,
                          double smin, double smax, uint32_t *pool,
                          int nthreads);

/* Posting-list index: list r (1-based rank) has
 * clip(floor(max_len / r^s), 1, max_len) documents drawn without
 * replacement from [0, doc_space), sorted.  setops_gen_index_lens fills
 * lens; setops_gen_index_fill writes the lists at offs into pool. */
int setops_gen_index_lens(size_t nlists, size_t max_len, double s,
                          uint64_t *lens);
int setops_gen_index_fill(uint64_t seed, size_t nlists, const uint64_t *lens,
                          const uint64_t *offs, uint64_t doc_space,
                          uint32_t *pool, int nthreads);

/* k-set queries over a posting-list index: k uniform in [kmin, kmax]
 * (kmax <= 16), then k distinct list ids (0-based popularity ranks) drawn
 * Zipf(s) over rank.  ids is nq x kmax, row q holding ks[q] ids. */
int setops_gen_queries(uint64_t seed, size_t nq, size_t nlists, uint32_t kmin,
                       uint32_t kmax, double s, uint32_t *ids, uint32_t *ks);

/* BSR encoding of many sorted sets of one pool (BsrVec::from_sorted,
 * setops/src/bsr.rs:140-163): set i = pool[offs[i], +lens[i]) becomes
 * wlens[i] words at bases/states[woffs[i], ...), sets packed in order.
 * bases/states need room for sum(lens) words. */
int setops_gen_bsr_encode(const uint32_t *pool, size_t nsets, const uint64_t *offs,
                          const uint64_t *lens, uint32_t *bases, uint32_t *states,
                          uint64_t *woffs, uint64_t *wlens);

/* Open-loop load for a server: query q (ids row q of an nq x kstride array,
 * ks[q] ids) arrives at the q-th point of a Poisson process of rate
 * rate_qps; latency_ns[q] runs from that arrival to completion, counts[q]
 * (optional) is the answer's length, and answers (optional, nq x
 * answer_stride u32) receives the answer itself in row q
 * (SETOPS_ERR_CAPACITY when one is longer than answer_stride).  Returns when
 * every query is done.  Exported by libsetops_gpu.so. */
struct setops_srv;
int setops_srv_run_load(struct setops_srv *srv, const uint32_t *ids, const uint32_t *ks,
                        size_t kstride, size_t nq, double rate_qps, uint64_t seed,
                        uint64_t *latency_ns, uint64_t *counts, uint32_t *answers,
                        size_t answer_stride, double *elapsed_s);

/* Sorted, duplicate-free sample of n values from [0, max_value). */
int setops_gen_sorted_sample(uint64_t seed, size_t n, uint64_t max_value,
                             uint32_t *out);

/* ---- datafile format (benchmark/src/datafile.rs:5-166) -------------------
 * Header: magic E9 AA 05, flag byte (bit 0 = little endian), u32 set count
 * (>= 2); then set_count u32 lengths; then the sets as 32-bit integers.
 * setops_datafile_write returns 0 or a negative code:
 *   -1 bad argument, -2 I/O error, -3 bad set count.
 * setops_datafile_read_header fills *set_count and lens (room for
 * max_sets entries) and returns 0 or: -2 I/O, -3 bad set count, -4 bad
 * magic, -5 bad endianness, -6 lens too small.  setops_datafile_read_sets
 * then reads all sets into the caller's buffers. */
int setops_datafile_write(const char *path, const uint32_t *const *sets,
                          const uint64_t *lens, size_t set_count);
int setops_datafile_read_header(const char *path, uint64_t *set_count,
                                uint64_t *lens, size_t max_sets);
int setops_datafile_read_sets(const char *path, uint32_t *const *sets);

/* The plain GPU paths a caller without batching or serving writes, looped
 * in C so that their timing holds no foreign-language call overhead (they
 * are the baselines of the batched and served paths).  Exported by
 * libsetops_gpu.so; `ctx` is a setops_ctx.
 *
 * setops_bench_pairs_one_by_one: one setops_gpu_intersect_async launch per
 * pair p, on device data: A = pool + a_off[p] (a_len[p] elements), B likewise,
 * output at out + out_off[p] (capacity min(a_len[p], b_len[p])), length to
 * the device word lens_dev[p]; then one setops_gpu_synchronize.  The offset
 * and length arrays are host arrays.  *seconds: wall time of the loop and the
 * synchronisation. */
struct setops_ctx;
int setops_bench_pairs_one_by_one(struct setops_ctx *ctx, const uint32_t *pool,
                                  const uint64_t *a_off, const uint64_t *a_len,
                                  const uint64_t *b_off, const uint64_t *b_len, size_t npairs,
                                  uint32_t *out, const uint64_t *out_off, uint64_t *lens_dev,
                                  double *seconds);
/* The same for BSR pairs: one setops_gpu_intersect_bsr call (which returns
 * the result length, so each call waits for its pair) per pair, words at
 * bases/states + a_off[p] etc. on the device, the result of pair p at
 * out_bases/out_states + out_off[p]; lens (host) gets each length. */
int setops_bench_bsr_pairs_one_by_one(struct setops_ctx *ctx, const uint32_t *bases,
                                      const uint32_t *states, const uint64_t *a_off,
                                      const uint64_t *a_len, const uint64_t *b_off,
                                      const uint64_t *b_len, size_t npairs, uint32_t *out_bases,
                                      uint32_t *out_states, const uint64_t *out_off,
                                      uint64_t *lens, double *seconds);
/* One setops_gpu_svs call per query q, in order: lists ids[q * kstride +
 * 0 .. ks[q]) of a device pool (list i = pool + offs[i], lens[i] elements;
 * offs and lens are host arrays), the answer to the device buffer out
 * (capacity out_cap, reused by every query).  latency_ns[q] (optional) gets
 * the call's wall time and counts[q] (optional) its answer's length. */
/* cudaEventRecordWithFlags(event, stream, cudaEventRecordExternal): an event
 * record that, made while `stream` is being captured into a CUDA graph,
 * records `event` at that point of every replay (so a captured region can be
 * timed).  Outside a capture it is a plain record.  Exported by
 * libsetops_gpu.so; event and stream are a cudaEvent_t and a cudaStream_t. */
int setops_bench_record_event(void *event, void *stream);
int setops_bench_queries_one_by_one(struct setops_ctx *ctx, const uint32_t *pool,
                                    const uint64_t *offs, const uint64_t *lens,
                                    const uint32_t *ids, const uint32_t *ks, size_t kstride,
                                    size_t nq, uint32_t *out, size_t out_cap,
                                    uint64_t *latency_ns, uint64_t *counts, double *seconds);

#ifdef __cplusplus
}
#endif
#endif /* SETOPS_BENCH_H */
