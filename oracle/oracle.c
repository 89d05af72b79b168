/*
 * oracle.c -- CPU restatement of the reference's sorted-u32 intersection path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h): the checker for the GPU path and
 * the timed CPU baseline.  Plain C99 + GCC vector extensions; no ISA-specific
 * intrinsics, so it builds and gives identical results on x86_64 and aarch64.
 *
 * Each function names the reference file:line it restates.  The reference
 * algorithms are generic over an output "visitor"; here that is an output
 * pointer (materialise, like VecWriter / UnsafeWriter) or NULL (count, like
 * Counter).
 */
#define _GNU_SOURCE
#include "oracle.h"

#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

/* Emit helper: write v at out[n] when materialising; always bump n. */
#define EMIT(out, n, v)                                                        \
  do {                                                                         \
    if (out) (out)[(n)] = (v);                                                 \
    (n)++;                                                                     \
  } while (0)

/* ------------------------------------------------------------------------ */
/* naive_merge (setops/src/intersect/merge.rs:7-33): two cursors, three-way
 * compare, emit on equality and advance both. */
size_t orc_naive_merge(const uint32_t *a, size_t na, const uint32_t *b,
                       size_t nb, uint32_t *out) {
  size_t i = 0, j = 0, n = 0;
  while (i < na && j < nb) {
    uint32_t x = a[i], y = b[j];
    if (x < y) {
      i++;
    } else if (x > y) {
      j++;
    } else {
      EMIT(out, n, x);
      i++;
      j++;
    }
  }
  return n;
}

/* branchless_merge (setops/src/intersect/merge.rs:39-60): equality branch,
 * otherwise advance each cursor by the result of its less-than. */
size_t orc_branchless_merge(const uint32_t *a, size_t na, const uint32_t *b,
                            size_t nb, uint32_t *out) {
  size_t i = 0, j = 0, n = 0;
  while (i < na && j < nb) {
    uint32_t x = a[i], y = b[j];
    if (x == y) {
      EMIT(out, n, x);
      i++;
      j++;
    } else {
      i += (x < y);
      j += (y < x);
    }
  }
  return n;
}

/* binary_search (setops/src/intersect/galloping.rs:110-131): classic
 * inclusive-bounds search; returns the match index or the final `lo`. */
size_t orc_binary_search(const uint32_t *set, uint32_t target, ptrdiff_t lo,
                         ptrdiff_t hi) {
  while (lo <= hi) {
    ptrdiff_t mid = lo + (hi - lo) / 2;
    uint32_t v = set[mid];
    if (v < target)
      lo = mid + 1;
    else if (v > target)
      hi = mid - 1;
    else
      return (size_t)mid;
  }
  return (size_t)lo;
}

/* galloping (setops/src/intersect/galloping.rs:7-30): for each element of
 * `small`, double an offset while large[offset] <= target, binary-search
 * [offset/2, min(len-1, offset)], then drop the searched prefix of large. */
size_t orc_galloping(const uint32_t *small, size_t ns, const uint32_t *large,
                     size_t nl, uint32_t *out) {
  size_t n = 0;
  for (size_t k = 0; k < ns; k++) {
    uint32_t target = small[k];
    size_t offset = 1;
    while (offset < nl && large[offset] <= target) offset *= 2;
    ptrdiff_t lo = (ptrdiff_t)(offset / 2);
    ptrdiff_t hi = (ptrdiff_t)nl - 1;
    if ((ptrdiff_t)offset < hi) hi = (ptrdiff_t)offset;
    size_t base = orc_binary_search(large, target, lo, hi);
    if (base < nl && large[base] == target) EMIT(out, n, target);
    large += base;
    nl -= base;
  }
  return n;
}

/* binary_search_intersect (setops/src/intersect/galloping.rs:32-49). */
size_t orc_binary_search_intersect(const uint32_t *small, size_t ns,
                                   const uint32_t *large, size_t nl,
                                   uint32_t *out) {
  size_t n = 0;
  for (size_t k = 0; k < ns; k++) {
    uint32_t target = small[k];
    size_t base = orc_binary_search(large, target, 0, (ptrdiff_t)nl - 1);
    if (base < nl && large[base] == target) EMIT(out, n, target);
    large += base;
    nl -= base;
  }
  return n;
}

/* ------------------------------------------------------------------------ */
/* BsrVec::from_sorted (setops/src/bsr.rs:140-163): base = x >> 5, state bit
 * = 1 << (x & 31); consecutive elements with the same base share a word. */
size_t orc_bsr_from_sorted(const uint32_t *in, size_t n, uint32_t *bases,
                           uint32_t *states) {
  size_t w = 0;
  for (size_t k = 0; k < n; k++) {
    uint32_t base = in[k] >> 5, bit = 1u << (in[k] & 31u);
    if (w > 0 && bases[w - 1] == base) {
      states[w - 1] |= bit;
    } else {
      bases[w] = base;
      states[w] = bit;
      w++;
    }
  }
  return w;
}

/* BsrVec::to_sorted_set (setops/src/bsr.rs:77-88): each set bit of a state,
 * lowest first, gives (base << 5) | bit_index. */
size_t orc_bsr_to_sorted(const uint32_t *bases, const uint32_t *states,
                         size_t n, uint32_t *out) {
  size_t m = 0;
  for (size_t k = 0; k < n; k++) {
    uint32_t hi = bases[k] << 5, s = states[k];
    while (s) {
      EMIT(out, m, hi | (uint32_t)__builtin_ctz(s));
      s &= s - 1;
    }
  }
  return m;
}

/* branchless_merge_bsr (setops/src/intersect/merge.rs:62-87). */
size_t orc_branchless_merge_bsr(const uint32_t *ba, const uint32_t *sa,
                                size_t na, const uint32_t *bb,
                                const uint32_t *sb, size_t nb,
                                uint32_t *out_bases, uint32_t *out_states,
                                uint64_t *elem_count) {
  size_t i = 0, j = 0, w = 0;
  uint64_t c = 0;
  while (i < na && j < nb) {
    uint32_t x = ba[i], y = bb[j];
    if (x == y) {
      uint32_t s = sa[i] & sb[j];
      if (s != 0) {
        if (out_bases) {
          out_bases[w] = x;
          out_states[w] = s;
        }
        w++;
        c += (uint64_t)__builtin_popcount(s);
      }
      i++;
      j++;
    } else {
      i += (x < y);
      j += (y < x);
    }
  }
  if (elem_count) *elem_count = c;
  return w;
}

/* broadcast_*_bsr (setops/src/intersect/broadcast.rs:163-357): blocks of w
 * bases of A and of B compared all against all (w broadcasts of B's bases);
 * a lane of A's block whose base equals one of B's takes the OR of the ANDed
 * states (at most one term is non-zero: bases are distinct); lanes with an
 * equal base and a non-zero state are visited in lane order; then A's block
 * advances when its last base is at most B's last, B's when B's last is at
 * most A's.  The remainders (fewer than w words of either set) go through
 * branchless_merge_bsr, as in the reference. */
size_t orc_broadcast_bsr(int w, const uint32_t *ba, const uint32_t *sa, size_t na,
                         const uint32_t *bb, const uint32_t *sb, size_t nb,
                         uint32_t *out_bases, uint32_t *out_states,
                         uint64_t *elem_count) {
  if (w < 1) w = 1;
  if (w > 16) w = 16;
  const size_t W = (size_t)w;
  const size_t st_a = (na / W) * W, st_b = (nb / W) * W;
  size_t ia = 0, ib = 0, n = 0;
  uint64_t c = 0;
  while (ia < st_a && ib < st_b) {
    for (size_t l = 0; l < W; ++l) {
      const uint32_t base = ba[ia + l];
      uint32_t state = 0;
      int eq = 0;
      for (size_t m = 0; m < W; ++m) {
        const int e = base == bb[ib + m];
        eq |= e;
        state |= e ? (sa[ia + l] & sb[ib + m]) : 0u;
      }
      if (eq && state != 0) {
        if (out_bases) {
          out_bases[n] = base;
          out_states[n] = state;
        }
        ++n;
        c += (uint64_t)__builtin_popcount(state);
      }
    }
    const uint32_t a_max = ba[ia + W - 1], b_max = bb[ib + W - 1];
    ia += W * (a_max <= b_max);
    ib += W * (b_max <= a_max);
  }
  uint64_t c2 = 0;
  const size_t n2 = orc_branchless_merge_bsr(ba + ia, sa + ia, na - ia, bb + ib, sb + ib, nb - ib,
                                             out_bases ? out_bases + n : NULL,
                                             out_states ? out_states + n : NULL, &c2);
  if (elem_count) *elem_count = c + c2;
  return n + n2;
}

/* galloping_bsr (setops/src/intersect/galloping.rs:51-76): galloping on the
 * bases of `large`, AND of states on a base match. */
size_t orc_galloping_bsr(const uint32_t *ba, const uint32_t *sa, size_t na,
                         const uint32_t *bb, const uint32_t *sb, size_t nb,
                         uint32_t *out_bases, uint32_t *out_states,
                         uint64_t *elem_count) {
  size_t w = 0;
  uint64_t c = 0;
  for (size_t k = 0; k < na; k++) {
    uint32_t target = ba[k];
    size_t offset = 1;
    while (offset < nb && bb[offset] <= target) offset *= 2;
    ptrdiff_t lo = (ptrdiff_t)(offset / 2);
    ptrdiff_t hi = (ptrdiff_t)nb - 1;
    if ((ptrdiff_t)offset < hi) hi = (ptrdiff_t)offset;
    size_t idx = orc_binary_search(bb, target, lo, hi);
    if (idx < nb && bb[idx] == target) {
      uint32_t s = sa[k] & sb[idx];
      if (s != 0) {
        if (out_bases) {
          out_bases[w] = target;
          out_states[w] = s;
        }
        w++;
        c += (uint64_t)__builtin_popcount(s);
      }
    }
    bb += idx;
    sb += idx;
    nb -= idx;
  }
  if (elem_count) *elem_count = c;
  return w;
}

/* ------------------------------------------------------------------------ */
/* svs_generic (setops/src/intersect/svs.rs:50-73) with naive_merge: the
 * first two sets go to `left`; every further set swaps the two buffers and
 * intersects the previous result (now in `right`) with it into `left`. */
typedef size_t (*pair_fn)(const uint32_t *, size_t, const uint32_t *, size_t,
                          uint32_t *);

/* svs_generic with the 2-set function `f` (the reference passes f as a
 * parameter, svs.rs:50). */
static size_t svs_with(pair_fn f, const uint32_t *const *sets, const size_t *lens,
                       size_t k, uint32_t *left, uint32_t *right,
                       uint32_t **result) {
  if (k < 2) {
    if (result) *result = left;
    return 0;
  }
  size_t n = f(sets[0], lens[0], sets[1], lens[1], left);
  for (size_t s = 2; s < k; s++) {
    uint32_t *t = left;
    left = right;
    right = t;
    n = f(right, n, sets[s], lens[s], left);
  }
  if (result) *result = left;
  return n;
}

size_t orc_svs_generic(const uint32_t *const *sets, const size_t *lens,
                       size_t k, uint32_t *left, uint32_t *right,
                       uint32_t **result) {
  return svs_with(orc_naive_merge, sets, lens, k, left, right, result);
}

/* small_adaptive (setops/src/intersect/adaptive.rs:107-148, Demaine,
 * Lopez-Ortiz and Munro 2001): every element of sets[0] is looked up in each
 * later set in turn, galloping from that set's last position (offset doubles
 * while set[base + offset] <= element, then a binary search of [base,
 * min(len - 1, base + offset)]); the first set that lacks it moves on to the
 * next element; an element found in every set is emitted.  k <= 64. */
size_t orc_small_adaptive(const uint32_t *const *sets, const size_t *lens, size_t k,
                          uint32_t *out) {
  if (k < 2 || k > 64) return 0;
  size_t pos[64] = {0};
  size_t n = 0;
  for (size_t e = 0; e < lens[0]; e++) {
    const uint32_t element = sets[0][e];
    int found_all = 1;
    for (size_t i = 1; i < k; i++) {
      const uint32_t *set = sets[i];
      const size_t len = lens[i];
      const size_t base = pos[i];
      size_t offset = 1;
      while (base + offset < len && set[base + offset] <= element) offset *= 2;
      const ptrdiff_t lo = (ptrdiff_t)base;
      ptrdiff_t hi = (ptrdiff_t)len - 1;
      if ((ptrdiff_t)(base + offset) < hi) hi = (ptrdiff_t)(base + offset);
      const size_t nb = orc_binary_search(set, element, lo, hi);
      pos[i] = nb;
      if (nb >= len || set[nb] != element) {
        found_all = 0;
        break;
      }
    }
    if (found_all) EMIT(out, n, element);
  }
  return n;
}

/* ------------------------------------------------------------------------ */
/* Portable SIMD restatements (GCC vector extensions).                      */

typedef uint32_t v8u __attribute__((vector_size(32)));
typedef int32_t v8i __attribute__((vector_size(32)));
typedef uint32_t v4u __attribute__((vector_size(16)));
typedef int32_t v4i __attribute__((vector_size(16)));
typedef uint32_t v16u __attribute__((vector_size(64)));
typedef int32_t v16i __attribute__((vector_size(64)));

static inline v8u load8(const uint32_t *p) {
  v8u v;
  memcpy(&v, p, sizeof v);
  return v;
}
static inline v16u load16(const uint32_t *p) {
  v16u v;
  memcpy(&v, p, sizeof v);
  return v;
}

/* Lane mask of an 8-lane comparison result (-1 / 0 per lane). */
static inline unsigned mask8(v8i m) {
  unsigned r = 0;
  for (int l = 0; l < 8; l++) r |= (unsigned)(m[l] & 1) << l;
  return r;
}

/* Tail of every SIMD baseline: branchless_merge appended at out[n]. */
static inline size_t merge_tail(const uint32_t *a, size_t na,
                                const uint32_t *b, size_t nb, uint32_t *out,
                                size_t n) {
  return n + orc_branchless_merge(a, na, b, nb, out ? out + n : NULL);
}

/* shuffling_avx2 (setops/src/intersect/shuffling.rs:69-112): compare an
 * 8-block of a against all 8 rotations of an 8-block of b, OR the masks,
 * emit the flagged lanes of a in lane order, then advance whichever block
 * has the smaller last element (both on a tie). */
size_t orc_shuffling_w8(const uint32_t *a, size_t na, const uint32_t *b,
                        size_t nb, uint32_t *out) {
  const size_t W = 8;
  size_t sta = (na / W) * W, stb = (nb / W) * W;
  size_t i = 0, j = 0, n = 0;
  const v8i r1 = {1, 2, 3, 4, 5, 6, 7, 0};
  while (i < sta && j < stb) {
    v8u va = load8(a + i), vb = load8(b + j);
    v8i m = (v8i)(va == vb);
    v8u rb = vb;
    for (int r = 1; r < 8; r++) {
      rb = __builtin_shuffle(rb, (v8u)r1);
      m |= (v8i)(va == rb);
    }
    unsigned bits = mask8(m);
    if (out) {
      while (bits) {
        out[n++] = va[__builtin_ctz(bits)];
        bits &= bits - 1;
      }
    } else {
      n += (size_t)__builtin_popcount(bits);
    }
    uint32_t amax = a[i + W - 1], bmax = b[j + W - 1];
    i += W * (amax <= bmax);
    j += W * (bmax <= amax);
  }
  return merge_tail(a + i, na - i, b + j, nb - j, out, n);
}

/* gallop_wide (setops/src/intersect/simd_galloping.rs:195-216) and
 * binary_search_wide (:218-244): find the first `bound`-block whose last
 * element is >= target. */
static size_t gallop_wide(uint32_t target, const uint32_t *large, size_t nl,
                          size_t bound) {
  size_t upper;
  if (large[bound - 1] >= target) {
    upper = 0;
  } else {
    size_t off = 1;
    while ((off + 1) * bound - 1 < nl && large[(off + 1) * bound - 1] < target)
      off *= 2;
    upper = off;
  }
  size_t lo = upper / 2;
  size_t hi = nl / bound - 1;
  if (upper < hi) hi = upper;
  while (lo < hi) {
    size_t mid = lo + (hi - lo) / 2;
    if (large[(mid + 1) * bound - 1] < target)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

/* simd_galloping_impl::<16> (setops/src/intersect/simd_galloping.rs:49-104)
 * with reduce_search_bound (:246-265) and block_compare (:267-288). */
size_t orc_simd_galloping_w16(const uint32_t *small, size_t ns,
                              const uint32_t *large, size_t nl, uint32_t *out) {
  const size_t LANES = 16, NUM_LANES_IN_BOUND = 32;
  const size_t bound = LANES * NUM_LANES_IN_BOUND;
  size_t n = 0;
  if (ns > nl) {
    const uint32_t *t = small;
    small = large;
    large = t;
    size_t tn = ns;
    ns = nl;
    nl = tn;
  }
  while (ns > 0 && nl >= bound) {
    uint32_t target = small[0];
    size_t tb = gallop_wide(target, large, nl, bound);
    if (large[(tb + 1) * bound - 1] < target) {
      large += (tb + 1) * bound;
      nl -= (tb + 1) * bound;
      if (ns >= bound) {
        const uint32_t *t = small;
        small = large;
        large = t;
        size_t tn = ns;
        ns = nl;
        nl = tn;
        continue;
      }
      break;
    }
    large += tb * bound;
    nl -= tb * bound;
    /* reduce_search_bound: pick the quarter of the block (in vector units). */
    size_t inner;
    if (large[bound / 2 - 1] >= target)
      inner = (large[bound / 4 - 1] < target) ? NUM_LANES_IN_BOUND / 4 : 0;
    else if (large[bound * 3 / 4 - 1] < target)
      inner = NUM_LANES_IN_BOUND * 3 / 4;
    else
      inner = NUM_LANES_IN_BOUND / 2;
    /* block_compare: 8 vectors of 16 lanes against the splatted target. */
    const uint32_t *p = large + LANES * inner;
    v16u t = (v16u){0} + target;
    v16i acc = (v16i){0};
    for (int v = 0; v < 8; v++) acc |= (v16i)(t == load16(p + LANES * v));
    int any = 0;
    for (int l = 0; l < 16; l++) any |= acc[l];
    if (any) EMIT(out, n, target);
    small++;
    ns--;
  }
  return merge_tail(small, ns, large, nl, out, n);
}

/* bmiss (setops/src/intersect/bmiss.rs:90-163): a 4x4 block pair first
 * passes a byte filter (byte 0 and byte 1 of every (a_p, b_q) pair must both
 * agree for some pair), then a word check emits each a_p found in the b
 * block.  The reference does the byte filter with byte shuffles
 * (BYTE_CHECK_GROUP_A/B, setops/src/instructions.rs:100-125); here the same
 * predicate is evaluated on the low 16 bits of each pair. */
size_t orc_bmiss_w4(const uint32_t *a, size_t na, const uint32_t *b,
                    size_t nb, uint32_t *out) {
  const size_t W = 4;
  size_t sta = (na / W) * W, stb = (nb / W) * W;
  size_t i = 0, j = 0, n = 0;
  const v4u lo16 = {0xffffu, 0xffffu, 0xffffu, 0xffffu};
  while (i < sta && j < stb) {
    v4u va, vb;
    memcpy(&va, a + i, 16);
    memcpy(&vb, b + j, 16);
    v4u la = va & lo16, lb = vb & lo16;
    v4i bc = (v4i){0};
    for (int q = 0; q < 4; q++) bc |= (v4i)(la == (v4u){0} + lb[q]);
    if (bc[0] | bc[1] | bc[2] | bc[3]) {
      for (int p = 0; p < 4; p++) {
        v4i wc = (v4i)(vb == (v4u){0} + va[p]);
        if (wc[0] | wc[1] | wc[2] | wc[3]) EMIT(out, n, va[p]);
      }
    }
    uint32_t amax = a[i + W - 1], bmax = b[j + W - 1];
    i += W * (amax <= bmax);
    j += W * (bmax <= amax);
  }
  return merge_tail(a + i, na - i, b + j, nb - j, out, n);
}

/* ------------------------------------------------------------------------ */
/* Multi-pair runner: pairs spread over threads (the reference itself is
 * single-threaded; this is the all-cores CPU baseline harness). */

static pair_fn algo_fn(int algo) {
  switch (algo) {
    case ORC_NAIVE_MERGE: return orc_naive_merge;
    case ORC_BRANCHLESS_MERGE: return orc_branchless_merge;
    case ORC_GALLOPING: return orc_galloping;
    case ORC_SHUFFLING_W8: return orc_shuffling_w8;
    case ORC_SIMD_GALLOPING_W16: return orc_simd_galloping_w16;
    case ORC_BMISS_W4: return orc_bmiss_w4;
    default: return NULL;
  }
}

typedef struct {
  pair_fn fn;
  size_t n;
  const uint32_t *const *as;
  const size_t *nas;
  const uint32_t *const *bs;
  const size_t *nbs;
  uint32_t *const *outs;
  uint64_t *counts;
  /* k-set groups */
  const uint32_t *const *sets;
  const size_t *lens;
  const size_t *offs;
  atomic_size_t next;
} job_t;

static void *pair_worker(void *arg) {
  job_t *J = (job_t *)arg;
  for (;;) {
    size_t i = atomic_fetch_add(&J->next, 1);
    if (i >= J->n) break;
    /* galloping-style baselines expect the smaller set first */
    const uint32_t *a = J->as[i], *b = J->bs[i];
    size_t na = J->nas[i], nb = J->nbs[i];
    if (J->fn == orc_galloping && na > nb) {
      const uint32_t *t = a;
      a = b;
      b = t;
      size_t tn = na;
      na = nb;
      nb = tn;
    }
    J->counts[i] = J->fn(a, na, b, nb, J->outs ? J->outs[i] : NULL);
  }
  return NULL;
}

static void *svs_worker(void *arg) {
  job_t *J = (job_t *)arg;
  for (;;) {
    size_t g = atomic_fetch_add(&J->next, 1);
    if (g >= J->n) break;
    size_t o = J->offs[g], k = J->offs[g + 1] - o;
    size_t cap = 0;
    for (size_t s = 0; s < k; s++)
      if (J->lens[o + s] > cap) cap = J->lens[o + s];
    uint32_t *buf = (uint32_t *)malloc(2 * (cap + 1) * sizeof(uint32_t));
    if (!buf) {
      J->counts[g] = (uint64_t)-1;
      continue;
    }
    uint32_t *res = NULL;
    size_t c = svs_with(J->fn ? J->fn : orc_naive_merge, J->sets + o, J->lens + o, k, buf,
                        buf + cap + 1, &res);
    if (J->outs && J->outs[g]) memcpy(J->outs[g], res, c * sizeof(uint32_t));
    J->counts[g] = c;
    free(buf);
  }
  return NULL;
}

static int run_threads(job_t *J, void *(*worker)(void *), int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 512) nthreads = 512;
  atomic_store(&J->next, 0);
  if (nthreads == 1) {
    worker(J);
    return 0;
  }
  pthread_t th[512];
  int started = 0;
  for (int t = 0; t < nthreads; t++) {
    if (pthread_create(&th[t], NULL, worker, J) != 0) break;
    started++;
  }
  if (started == 0) worker(J);
  for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
  return 0;
}

int orc_run_pairs(int algo, size_t n, const uint32_t *const *as,
                  const size_t *nas, const uint32_t *const *bs,
                  const size_t *nbs, uint32_t *const *outs, uint64_t *counts,
                  int nthreads) {
  pair_fn fn = algo_fn(algo);
  if (!fn || (n && (!as || !nas || !bs || !nbs || !counts))) return -1;
  job_t J;
  memset(&J, 0, sizeof J);
  J.fn = fn;
  J.n = n;
  J.as = as;
  J.nas = nas;
  J.bs = bs;
  J.nbs = nbs;
  J.outs = outs;
  J.counts = counts;
  return run_threads(&J, pair_worker, nthreads);
}

int orc_run_svs_groups(size_t ngroups, const uint32_t *const *sets,
                       const size_t *lens, const size_t *offs,
                       uint32_t *const *outs, uint64_t *counts, int nthreads) {
  return orc_run_svs_groups_algo(ORC_NAIVE_MERGE, ngroups, sets, lens, offs, outs, counts,
                                 nthreads);
}

int orc_run_svs_groups_algo(int algo, size_t ngroups, const uint32_t *const *sets,
                            const size_t *lens, const size_t *offs,
                            uint32_t *const *outs, uint64_t *counts, int nthreads) {
  pair_fn fn = algo_fn(algo);
  if (!fn || fn == orc_galloping) return -1; /* galloping needs the smaller set first */
  if (ngroups && (!sets || !lens || !offs || !counts)) return -1;
  job_t J;
  memset(&J, 0, sizeof J);
  J.fn = fn;
  J.n = ngroups;
  J.sets = sets;
  J.lens = lens;
  J.offs = offs;
  J.outs = outs;
  J.counts = counts;
  return run_threads(&J, svs_worker, nthreads);
}

/* BSR pairs spread over threads: pair i = (ba[i], sa[i], na[i]) x (bb[i],
 * sb[i], nb[i]) through branchless_merge_bsr (algo 0) or galloping_bsr
 * (algo 1, the first set taken as the smaller); words[i] gets the result's
 * word count, results to ob[i]/os[i] when given. */
typedef size_t (*bsr_fn)(const uint32_t *, const uint32_t *, size_t, const uint32_t *,
                         const uint32_t *, size_t, uint32_t *, uint32_t *, uint64_t *);

typedef struct {
  bsr_fn fn;
  size_t n;
  const uint32_t *const *ba, *const *sa, *const *bb, *const *sb;
  const size_t *na, *nb;
  uint32_t *const *ob, *const *os;
  uint64_t *words;
  atomic_size_t next;
} bsr_job_t;

static void *bsr_worker(void *arg) {
  bsr_job_t *J = (bsr_job_t *)arg;
  for (;;) {
    size_t i = atomic_fetch_add(&J->next, 1);
    if (i >= J->n) break;
    J->words[i] = J->fn(J->ba[i], J->sa[i], J->na[i], J->bb[i], J->sb[i], J->nb[i],
                        J->ob ? J->ob[i] : NULL, J->os ? J->os[i] : NULL, NULL);
  }
  return NULL;
}

int orc_run_bsr_pairs(int algo, size_t n, const uint32_t *const *ba,
                      const uint32_t *const *sa, const size_t *na,
                      const uint32_t *const *bb, const uint32_t *const *sb,
                      const size_t *nb, uint32_t *const *ob, uint32_t *const *os,
                      uint64_t *words, int nthreads) {
  if ((algo != 0 && algo != 1) || (n && (!ba || !sa || !na || !bb || !sb || !nb || !words)))
    return -1;
  if ((ob == NULL) != (os == NULL)) return -1;
  bsr_job_t J;
  memset(&J, 0, sizeof J);
  J.fn = algo == 0 ? orc_branchless_merge_bsr : orc_galloping_bsr;
  J.n = n;
  J.ba = ba;
  J.sa = sa;
  J.na = na;
  J.bb = bb;
  J.sb = sb;
  J.nb = nb;
  J.ob = ob;
  J.os = os;
  J.words = words;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 512) nthreads = 512;
  atomic_store(&J.next, 0);
  if (nthreads == 1) {
    bsr_worker(&J);
    return 0;
  }
  pthread_t th[512];
  int started = 0;
  for (int t = 0; t < nthreads; t++) {
    if (pthread_create(&th[t], NULL, bsr_worker, &J) != 0) break;
    started++;
  }
  if (started == 0) bsr_worker(&J);
  for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
  return 0;
}
