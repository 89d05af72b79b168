/*
 * oracle.h -- CPU restatement of the reference's sorted-u32 intersection path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU path and
 * the CPU baseline that bench.py times beside it.  Only tests/, the smoke()
 * entry of __graft_entry__.py and bench.py's CPU-baseline / reference legs may
 * load it.  The product library (libsetops_gpu.so) never links or calls it.
 *
 * Every function restates one function of UNSW-database/simd_set_operations
 * (Rust crate `setops`); the file:line it follows is given beside each
 * declaration.  All sets are strictly increasing arrays of uint32_t, compared
 * in unsigned order (the reference's benchmark passes i32 data whose values are
 * all < 2^31, where the two orders agree).
 *
 * Parity pin: the restatement is checked against (1) the reference's own
 * known-answer tests (setops/tests/unit_tests.rs:7-59, restated as fixtures in
 * tests/golden/), and (2) outputs of the reference's own C++ kernels
 * (setops/ffi/qfilter/qfilter.cpp, compiled unchanged from the reference tree
 * into oracle/_ref/ on x86 hosts) on seeded inputs, committed as fixtures.
 *
 * Materialising functions take an output buffer `out` with capacity
 * >= min(na, nb) (the reference's UnsafeWriter / Intersect2C convention,
 * setops/src/intersect.rs:54-67); passing out == NULL counts only (the
 * reference's Counter visitor, setops/src/visitor.rs:24-49).
 */
#ifndef SETOPS_ORACLE_H
#define SETOPS_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- 2-set, scalar (the parity oracle) --------------------------------- */

/* naive_merge: setops/src/intersect/merge.rs:7-33 */
size_t orc_naive_merge(const uint32_t *a, size_t na, const uint32_t *b,
                       size_t nb, uint32_t *out);

/* branchless_merge: setops/src/intersect/merge.rs:39-60 */
size_t orc_branchless_merge(const uint32_t *a, size_t na, const uint32_t *b,
                            size_t nb, uint32_t *out);

/* binary_search: setops/src/intersect/galloping.rs:110-131.  Returns the
 * index of `target` in set[lo..=hi] if present, else the insertion point. */
size_t orc_binary_search(const uint32_t *set, uint32_t target, ptrdiff_t lo,
                         ptrdiff_t hi);

/* galloping: setops/src/intersect/galloping.rs:7-30 (small drives, no swap) */
size_t orc_galloping(const uint32_t *small, size_t ns, const uint32_t *large,
                     size_t nl, uint32_t *out);

/* binary_search_intersect: setops/src/intersect/galloping.rs:32-49 */
size_t orc_binary_search_intersect(const uint32_t *small, size_t ns,
                                   const uint32_t *large, size_t nl,
                                   uint32_t *out);

/* ---- BSR (base-and-state) ---------------------------------------------- */

/* BsrVec::from_sorted: setops/src/bsr.rs:140-163.  bases/states need room
 * for n words; returns the word count. */
size_t orc_bsr_from_sorted(const uint32_t *in, size_t n, uint32_t *bases,
                           uint32_t *states);

/* BsrVec::to_sorted_set: setops/src/bsr.rs:77-88.  Returns element count;
 * out == NULL counts only. */
size_t orc_bsr_to_sorted(const uint32_t *bases, const uint32_t *states,
                         size_t n, uint32_t *out);

/* branchless_merge_bsr: setops/src/intersect/merge.rs:62-87.  Emits
 * (base, sa & sb) for equal bases whose AND is non-zero.  Returns the word
 * count; out_bases == NULL counts words only.  *elem_count (if non-NULL)
 * receives the Counter value: sum of popcount(state) over emitted words
 * (setops/src/visitor.rs:399-403). */
size_t orc_branchless_merge_bsr(const uint32_t *ba, const uint32_t *sa,
                                size_t na, const uint32_t *bb,
                                const uint32_t *sb, size_t nb,
                                uint32_t *out_bases, uint32_t *out_states,
                                uint64_t *elem_count);

/* galloping_bsr: setops/src/intersect/galloping.rs:51-76 */
size_t orc_galloping_bsr(const uint32_t *ba, const uint32_t *sa, size_t na,
                         const uint32_t *bb, const uint32_t *sb, size_t nb,
                         uint32_t *out_bases, uint32_t *out_states,
                         uint64_t *elem_count);

/* broadcast_{sse,avx2,avx512}_bsr: setops/src/intersect/broadcast.rs:163-357,
 * blocks of w = 4, 8 or 16 bases (w <= 16); the same outputs as
 * orc_branchless_merge_bsr. */
size_t orc_broadcast_bsr(int w, const uint32_t *ba, const uint32_t *sa, size_t na,
                         const uint32_t *bb, const uint32_t *sb, size_t nb,
                         uint32_t *out_bases, uint32_t *out_states,
                         uint64_t *elem_count);

/* ---- k-set --------------------------------------------------------------- */

/* svs_generic with naive_merge as the 2-set function:
 * setops/src/intersect/svs.rs:50-73 (run_svs :103-116).  `left` and `right`
 * are ping-pong buffers, each of capacity >= min(lens[0], lens[1]).  The
 * sets are intersected in the order given (the reference assumes
 * smallest-first).  *result receives whichever buffer holds the answer;
 * returns its length.  k >= 2. */
/* small_adaptive: setops/src/intersect/adaptive.rs:107-148 (sets[0] the
 * probe set; k <= 64).  Returns the count; out (optional) gets the elements. */
size_t orc_small_adaptive(const uint32_t *const *sets, const size_t *lens, size_t k,
                          uint32_t *out);
size_t orc_svs_generic(const uint32_t *const *sets, const size_t *lens,
                       size_t k, uint32_t *left, uint32_t *right,
                       uint32_t **result);

/* ---- CPU baselines (portable restatements of the reference's SIMD) ------ */

/* shuffling_avx2: setops/src/intersect/shuffling.rs:69-112 (8-lane blocks,
 * all-pairs equality by 8 rotations, branchless_merge tail). */
size_t orc_shuffling_w8(const uint32_t *a, size_t na, const uint32_t *b,
                        size_t nb, uint32_t *out);

/* galloping_avx512 = simd_galloping_impl::<16>:
 * setops/src/intersect/simd_galloping.rs:40-104, gallop_wide :195-216,
 * binary_search_wide :218-244, reduce_search_bound :246-265,
 * block_compare :267-288. */
size_t orc_simd_galloping_w16(const uint32_t *a, size_t na, const uint32_t *b,
                              size_t nb, uint32_t *out);

/* bmiss: setops/src/intersect/bmiss.rs:90-163 (4x4 byte-check filter on
 * bytes 0-1, then word check; branchless_merge tail). */
size_t orc_bmiss_w4(const uint32_t *a, size_t na, const uint32_t *b,
                    size_t nb, uint32_t *out);

/* Algorithm ids for the multi-pair runner. */
enum {
  ORC_NAIVE_MERGE = 0,
  ORC_BRANCHLESS_MERGE = 1,
  ORC_GALLOPING = 2,
  ORC_SHUFFLING_W8 = 3,
  ORC_SIMD_GALLOPING_W16 = 4,
  ORC_BMISS_W4 = 5,
  ORC_NUM_ALGOS = 6
};

/* Runs algorithm `algo` over n independent pairs, spread over `nthreads`
 * worker threads (pairs are claimed in order from a shared counter; one
 * pair never spans threads, as in the reference, which has no intra-pair
 * parallelism).  outs[i] may be NULL (count only).  counts[i] receives each
 * pair's intersection size.  Returns 0, or -1 on a bad argument. */
int orc_run_pairs(int algo, size_t n, const uint32_t *const *as,
                  const size_t *nas, const uint32_t *const *bs,
                  const size_t *nbs, uint32_t *const *outs, uint64_t *counts,
                  int nthreads);

/* Same, for k-set groups through orc_svs_generic.  Group g has sets
 * sets[offs[g] .. offs[g+1]) with lengths lens[...]; out[g] (capacity
 * >= the smallest set of the group, may be NULL) receives the result. */
int orc_run_svs_groups(size_t ngroups, const uint32_t *const *sets,
                       const size_t *lens, const size_t *offs,
                       uint32_t *const *outs, uint64_t *counts, int nthreads);
/* The same with the 2-set function `algo` (an ORC_* id other than
 * ORC_GALLOPING) in every SvS step, as svs_generic takes it as a parameter
 * (setops/src/intersect/svs.rs:50): the timed CPU baseline of k-set work. */
int orc_run_svs_groups_algo(int algo, size_t ngroups, const uint32_t *const *sets,
                            const size_t *lens, const size_t *offs,
                            uint32_t *const *outs, uint64_t *counts, int nthreads);

/* BSR pairs over threads: branchless_merge_bsr (algo 0) or galloping_bsr
 * (algo 1) per pair; words[i] = result word count; ob/os optional. */
int orc_run_bsr_pairs(int algo, size_t n, const uint32_t *const *ba,
                      const uint32_t *const *sa, const size_t *na,
                      const uint32_t *const *bb, const uint32_t *const *sb,
                      const size_t *nb, uint32_t *const *ob, uint32_t *const *os,
                      uint64_t *words, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
