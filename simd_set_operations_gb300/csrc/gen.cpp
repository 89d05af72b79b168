// gen.cpp -- seeded synthetic input generators and the datafile format
// (include/setops_bench.h).  Restates benchmark/src/generators.rs and
// benchmark/src/datafile.rs of the reference with a seeded PRNG.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/setops_bench.h"

namespace {

// ---- PRNG: xoshiro256** seeded by SplitMix64 ------------------------------
inline uint64_t splitmix64(uint64_t &x) {
  uint64_t z = (x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    uint64_t x = seed;
    for (auto &w : s) w = splitmix64(x);
  }
  static inline uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }
  inline uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  // uniform in [0, m), m <= 2^32 (multiply-shift; bias < m / 2^32)
  inline uint32_t below(uint64_t m) {
    return uint32_t(((next() >> 32) * m) >> 32);
  }
  inline double unit() { return double(next() >> 11) * (1.0 / 9007199254740992.0); }
};

uint64_t derive(uint64_t seed, uint64_t idx) {
  uint64_t x = seed ^ (idx * 0xd1b54a32d192ed03ull + 0x8cb92ba72f3d8dd7ull);
  return splitmix64(x);
}

// LSD radix sort of u32, 3 passes of 11 bits.
void radix_sort(std::vector<uint32_t> &v) {
  const size_t n = v.size();
  if (n < 256) {
    std::sort(v.begin(), v.end());
    return;
  }
  std::vector<uint32_t> tmp(n);
  uint32_t *src = v.data(), *dst = tmp.data();
  for (int pass = 0; pass < 3; ++pass) {
    const int shift = pass * 11;
    size_t cnt[2048] = {0};
    for (size_t i = 0; i < n; ++i) cnt[(src[i] >> shift) & 2047]++;
    size_t sum = 0;
    for (auto &c : cnt) {
      size_t t = c;
      c = sum;
      sum += t;
    }
    for (size_t i = 0; i < n; ++i) dst[cnt[(src[i] >> shift) & 2047]++] = src[i];
    std::swap(src, dst);
  }
  if (src != v.data()) std::memcpy(v.data(), src, n * 4);
}

void sort_unique(std::vector<uint32_t> &v) {
  radix_sort(v);
  v.erase(std::unique(v.begin(), v.end()), v.end());
}

void shuffle(std::vector<uint32_t> &v, Rng &r) {
  for (size_t i = v.size(); i > 1; --i) {
    const size_t j = size_t(r.next() % i);
    std::swap(v[i - 1], v[j]);
  }
}

// shuffled_set (generators.rs:83-110): result_len distinct values from
// [0, max_value) in random order.
std::vector<uint32_t> shuffled_set(size_t result_len, uint64_t max_value,
                                   Rng &r) {
  std::vector<uint32_t> items;
  if (result_len * 2 < max_value) {
    while (items.size() < result_len) {
      const size_t need = result_len - items.size();
      items.reserve(items.size() + 2 * need);
      for (size_t i = 0; i < 2 * need; ++i) items.push_back(r.below(max_value));
      sort_unique(items);
    }
    shuffle(items, r);
    items.resize(result_len);
  } else {
    items.resize(max_value);
    for (uint64_t i = 0; i < max_value; ++i) items[i] = uint32_t(i);
    shuffle(items, r);
    items.resize(std::min<uint64_t>(result_len, max_value));
  }
  return items;
}

// Two sets of the given lengths sharing floor(sel * small) elements.
void twoset(Rng &r, double density, double selectivity, size_t small_len,
            size_t large_len, uint32_t *small_out, uint32_t *large_out) {
  const uint64_t max_value =
      std::max<uint64_t>(1, uint64_t(double(large_len) / density));
  size_t shared = size_t(selectivity * double(small_len));
  size_t gen = small_len + large_len - shared;
  if (gen > max_value) {  // generators.rs:46-50
    shared = small_len + large_len - size_t(max_value);
    gen = size_t(max_value);
  }
  std::vector<uint32_t> values = shuffled_set(gen, max_value, r);
  std::vector<uint32_t> s(values.begin(), values.begin() + small_len);
  std::vector<uint32_t> l(values.begin(), values.begin() + shared);
  l.insert(l.end(), values.begin() + small_len, values.begin() + gen);
  radix_sort(s);
  radix_sort(l);
  std::memcpy(small_out, s.data(), small_len * 4);
  std::memcpy(large_out, l.data(), large_len * 4);
}

template <class F>
void parallel_for(size_t n, int nthreads, F &&f) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads == 1 || n < 2) {
    for (size_t i = 0; i < n; ++i) f(i);
    return;
  }
  std::atomic<size_t> next{0};
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t)
    th.emplace_back([&] {
      for (;;) {
        const size_t i = next.fetch_add(1);
        if (i >= n) break;
        f(i);
      }
    });
  for (auto &x : th) x.join();
}

}  // namespace

extern "C" {

int setops_gen_twoset(uint64_t seed, double density, double selectivity,
                      size_t small_len, size_t large_len, uint32_t *small_out,
                      uint32_t *large_out) {
  if (density <= 0 || selectivity < 0 || selectivity > 1 ||
      small_len > large_len || (small_len && !small_out) ||
      (large_len && !large_out))
    return -1;
  if (double(large_len) / density >= 4294967296.0) return -1;
  Rng r(seed);
  twoset(r, density, selectivity, small_len, large_len, small_out, large_out);
  return 0;
}

int setops_gen_kset_lens(size_t max_len, double skewness, size_t set_count,
                         size_t *lens) {
  if (!lens || set_count < 2) return -1;
  for (size_t k = 0; k < set_count; ++k) {
    const size_t idx = set_count - 1 - k;  // smallest first
    const size_t skew = size_t(std::pow(double(idx + 1), skewness));
    lens[k] = max_len / std::max<size_t>(skew, 1);
  }
  return 0;
}

int setops_gen_kset(uint64_t seed, double density, double selectivity,
                    size_t max_len, double skewness, size_t set_count,
                    uint32_t *const *outs) {
  if (!outs || set_count < 2 || density <= 0) return -1;
  std::vector<size_t> lens(set_count);
  setops_gen_kset_lens(max_len, skewness, set_count, lens.data());
  const uint64_t max_value = uint64_t(double(max_len) / density);
  if (max_value >= (uint64_t(1) << 32)) return -1;
  Rng r(seed);
  const size_t shared_count = size_t(selectivity * double(lens[0]));
  std::vector<uint32_t> shared = shuffled_set(shared_count, max_value, r);
  std::vector<uint64_t> bitmap((max_value + 63) / 64, 0);
  for (uint32_t v : shared) bitmap[v >> 6] |= uint64_t(1) << (v & 63);
  for (size_t k = 0; k < set_count; ++k) {
    // sorted_set_containing (generators.rs:139-191): uniform fill disjoint
    // from the shared core, then the core, sorted.
    const size_t want = lens[k] - std::min(lens[k], shared.size());
    std::vector<uint32_t> fill;
    if (lens[k] * 2 < max_value) {
      while (fill.size() < want) {
        const size_t need = want - fill.size();
        for (size_t i = 0; i < 2 * need; ++i) {
          const uint32_t v = r.below(max_value);
          if (!((bitmap[v >> 6] >> (v & 63)) & 1)) fill.push_back(v);
        }
        sort_unique(fill);
      }
    } else {
      for (uint64_t v = 0; v < max_value; ++v)
        if (!((bitmap[v >> 6] >> (v & 63)) & 1)) fill.push_back(uint32_t(v));
    }
    shuffle(fill, r);
    fill.resize(want);
    fill.insert(fill.end(), shared.begin(), shared.end());
    radix_sort(fill);
    std::memcpy(outs[k], fill.data(), fill.size() * 4);
  }
  return 0;
}

int setops_gen_batch_sizes(uint64_t seed, size_t npairs, size_t min_len,
                           size_t max_len, uint64_t *a_len, uint64_t *b_len) {
  if ((npairs && (!a_len || !b_len)) || min_len < 1 || max_len < min_len)
    return -1;
  Rng r(seed);
  const double l0 = std::log2(double(min_len)), l1 = std::log2(double(max_len));
  for (size_t p = 0; p < npairs; ++p) {
    a_len[p] = uint64_t(std::floor(std::exp2(l0 + (l1 - l0) * r.unit())));
    b_len[p] = uint64_t(std::floor(std::exp2(l0 + (l1 - l0) * r.unit())));
  }
  return 0;
}

int setops_gen_batch_fill(uint64_t seed, size_t npairs, const uint64_t *a_len,
                          const uint64_t *b_len, const uint64_t *a_off,
                          const uint64_t *b_off, double dmin, double dmax,
                          double smin, double smax, uint32_t *pool,
                          int nthreads) {
  if (npairs && (!a_len || !b_len || !a_off || !b_off || !pool)) return -1;
  if (dmin <= 0 || dmax < dmin || smin < 0 || smax > 1 || smax < smin) return -1;
  parallel_for(npairs, nthreads, [&](size_t p) {
    Rng r(derive(seed, p));
    const double d = dmin + (dmax - dmin) * r.unit();
    const double s = smin + (smax - smin) * r.unit();
    const bool a_small = a_len[p] <= b_len[p];
    const size_t sl = a_small ? a_len[p] : b_len[p];
    const size_t ll = a_small ? b_len[p] : a_len[p];
    uint32_t *so = pool + (a_small ? a_off[p] : b_off[p]);
    uint32_t *lo = pool + (a_small ? b_off[p] : a_off[p]);
    twoset(r, d, s, sl, ll, so, lo);
  });
  return 0;
}

int setops_gen_index_lens(size_t nlists, size_t max_len, double s,
                          uint64_t *lens) {
  if (nlists && !lens) return -1;
  for (size_t i = 0; i < nlists; ++i) {
    double v = std::floor(double(max_len) / std::pow(double(i + 1), s));
    if (v < 1) v = 1;
    if (v > double(max_len)) v = double(max_len);
    lens[i] = uint64_t(v);
  }
  return 0;
}

int setops_gen_sorted_sample(uint64_t seed, size_t n, uint64_t max_value,
                             uint32_t *out) {
  if ((n && !out) || n > max_value || max_value > (uint64_t(1) << 32)) return -1;
  Rng r(seed);
  std::vector<uint32_t> v = shuffled_set(n, max_value, r);
  radix_sort(v);
  std::memcpy(out, v.data(), n * 4);
  return 0;
}

int setops_gen_bsr_encode(const uint32_t *pool, size_t nsets, const uint64_t *offs,
                          const uint64_t *lens, uint32_t *bases, uint32_t *states,
                          uint64_t *woffs, uint64_t *wlens) {
  // BsrVec::from_sorted (setops/src/bsr.rs:140-163): one word per distinct
  // x >> 5, its state the OR of 1 << (x & 31); sets packed back to back
  if ((nsets && (!pool || !offs || !lens || !bases || !states || !woffs || !wlens))) return -1;
  uint64_t w = 0;
  for (size_t i = 0; i < nsets; ++i) {
    const uint32_t *x = pool + offs[i];
    const uint64_t n = lens[i];
    woffs[i] = w;
    uint64_t k = 0;
    for (uint64_t j = 0; j < n; ++j) {
      const uint32_t b = x[j] >> 5, bit = 1u << (x[j] & 31);
      if (k > 0 && bases[w + k - 1] == b) {
        states[w + k - 1] |= bit;
      } else {
        bases[w + k] = b;
        states[w + k] = bit;
        ++k;
      }
    }
    wlens[i] = k;
    w += k;
  }
  return 0;
}

int setops_gen_queries(uint64_t seed, size_t nq, size_t nlists, uint32_t kmin,
                       uint32_t kmax, double s, uint32_t *ids, uint32_t *ks) {
  if ((nq && (!ids || !ks)) || kmin < 1 || kmax < kmin || kmax > 16 || nlists < kmax) return -1;
  // inverse CDF of Zipf(s) over popularity ranks 1..nlists
  std::vector<double> cdf(nlists);
  double acc = 0;
  for (size_t r = 0; r < nlists; ++r) {
    acc += 1.0 / std::pow(double(r + 1), s);
    cdf[r] = acc;
  }
  Rng rng(seed);
  for (size_t q = 0; q < nq; ++q) {
    const uint32_t k = kmin + rng.below(uint64_t(kmax - kmin + 1));
    ks[q] = k;
    uint32_t *row = ids + q * kmax;
    for (uint32_t j = 0; j < kmax; ++j) row[j] = 0;
    for (uint32_t j = 0; j < k; ++j) {
      uint32_t id = 0;
      for (int attempt = 0; attempt < 64; ++attempt) {  // distinct lists per query
        const double u = rng.unit() * acc;
        id = uint32_t(std::lower_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
        if (id >= nlists) id = uint32_t(nlists - 1);
        bool dup = false;
        for (uint32_t i = 0; i < j; ++i) dup |= row[i] == id;
        if (!dup) break;
        id = uint32_t(-1);
      }
      if (id == uint32_t(-1)) {  // heavy skew: take the first unused rank
        for (uint32_t c = 0; c < nlists; ++c) {
          bool used = false;
          for (uint32_t i = 0; i < j; ++i) used |= row[i] == c;
          if (!used) {
            id = c;
            break;
          }
        }
      }
      row[j] = id;
    }
  }
  return 0;
}

int setops_gen_index_fill(uint64_t seed, size_t nlists, const uint64_t *lens,
                          const uint64_t *offs, uint64_t doc_space,
                          uint32_t *pool, int nthreads) {
  if (nlists && (!lens || !offs || !pool)) return -1;
  if (doc_space > (uint64_t(1) << 32)) return -1;
  for (size_t i = 0; i < nlists; ++i)
    if (lens[i] > doc_space) return -1;
  parallel_for(nlists, nthreads, [&](size_t i) {
    Rng r(derive(seed, i));
    std::vector<uint32_t> v = shuffled_set(lens[i], doc_space, r);
    radix_sort(v);
    std::memcpy(pool + offs[i], v.data(), v.size() * 4);
  });
  return 0;
}

// ---- datafile (benchmark/src/datafile.rs) ---------------------------------
static const unsigned char kMagic[3] = {0xe9, 0xaa, 0x05};

static bool host_little_endian() {
  const uint32_t x = 1;
  unsigned char c;
  std::memcpy(&c, &x, 1);
  return c == 1;
}

int setops_datafile_write(const char *path, const uint32_t *const *sets,
                          const uint64_t *lens, size_t set_count) {
  if (!path || (set_count && (!sets || !lens))) return -1;
  if (set_count < 2 || set_count > 0xffffffffull) return -3;
  for (size_t i = 0; i < set_count; ++i)
    if (lens[i] > 0xffffffffull || (lens[i] && !sets[i])) return -1;
  FILE *f = std::fopen(path, "wb");
  if (!f) return -2;
  unsigned char hdr[8] = {kMagic[0], kMagic[1], kMagic[2],
                          (unsigned char)(host_little_endian() ? 1 : 0)};
  const uint32_t cnt = uint32_t(set_count);
  std::memcpy(hdr + 4, &cnt, 4);
  bool ok = std::fwrite(hdr, 1, 8, f) == 8;
  for (size_t i = 0; ok && i < set_count; ++i) {
    const uint32_t l = uint32_t(lens[i]);
    ok = std::fwrite(&l, 4, 1, f) == 1;
  }
  for (size_t i = 0; ok && i < set_count; ++i)
    if (lens[i]) ok = std::fwrite(sets[i], 4, lens[i], f) == lens[i];
  ok = (std::fclose(f) == 0) && ok;
  return ok ? 0 : -2;
}

static int read_header(FILE *f, uint64_t *set_count, std::vector<uint32_t> &lens) {
  unsigned char hdr[8];
  if (std::fread(hdr, 1, 8, f) != 8) return -2;
  if (std::memcmp(hdr, kMagic, 3) != 0) return -4;
  if (((hdr[3] & 1) != 0) != host_little_endian()) return -5;
  uint32_t cnt;
  std::memcpy(&cnt, hdr + 4, 4);
  if (cnt < 2) return -3;
  lens.resize(cnt);
  if (std::fread(lens.data(), 4, cnt, f) != cnt) return -2;
  *set_count = cnt;
  return 0;
}

int setops_datafile_read_header(const char *path, uint64_t *set_count,
                                uint64_t *lens, size_t max_sets) {
  if (!path || !set_count) return -1;
  FILE *f = std::fopen(path, "rb");
  if (!f) return -2;
  std::vector<uint32_t> l;
  int rc = read_header(f, set_count, l);
  std::fclose(f);
  if (rc) return rc;
  if (lens) {
    if (max_sets < l.size()) return -6;
    for (size_t i = 0; i < l.size(); ++i) lens[i] = l[i];
  }
  return 0;
}

int setops_datafile_read_sets(const char *path, uint32_t *const *sets) {
  if (!path || !sets) return -1;
  FILE *f = std::fopen(path, "rb");
  if (!f) return -2;
  uint64_t cnt = 0;
  std::vector<uint32_t> l;
  int rc = read_header(f, &cnt, l);
  for (size_t i = 0; rc == 0 && i < l.size(); ++i)
    if (l[i] && std::fread(sets[i], 4, l[i], f) != l[i]) rc = -2;
  std::fclose(f);
  return rc;
}

}  // extern "C"
