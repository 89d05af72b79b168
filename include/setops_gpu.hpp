/* setops_gpu.hpp -- C++ face of setops_gpu.h, shaped like the reference's
 * generic-visitor API (setops/src/intersect.rs:40-90, setops/src/visitor.rs):
 *
 *   Rust (reference)                          C++ (this header)
 *   intersect(a, b, &mut Counter)             intersect(ctx, a, b, Counter&)
 *   intersect(a, b, &mut VecWriter)           intersect(ctx, a, b, VecWriter&)
 *   Intersect2C: fn(&[T], &[T], &mut [T])     intersect_c(ctx, a, b, out)  (SliceWriter)
 *   run_2set(a, b, f) -> Vec                  run_2set(ctx, a, b)
 *   Intersect2Bsr on BsrVec                   intersect_bsr(ctx, a, b, BsrVec&)
 *   svs_generic / run_kset                    run_kset(ctx, sets)
 *
 * Header-only over the C ABI (link libsetops_gpu.so); host vectors in and
 * out (SETOPS_HOST).  Errors throw setops_gpu::Error with the library's
 * message -- the reference aborts on misuse (assert!, panic = "abort").
 * A Context is not thread-safe: one caller at a time, as with the C ABI. */
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "setops_gpu.h"

namespace setops_gpu {

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string &what) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

class Context {
 public:
  explicit Context(int device = 0) { check(setops_gpu_create(&ctx_, device)); }
  ~Context() {
    if (ctx_) setops_gpu_destroy(ctx_);
  }
  Context(const Context &) = delete;
  Context &operator=(const Context &) = delete;
  setops_ctx *get() const { return ctx_; }
  // Throws for a non-zero status, with the context's last error text.
  void check(int rc) const {
    if (rc == SETOPS_OK) return;
    std::string msg = setops_status_string(rc);
    if (ctx_) msg += std::string(": ") + setops_gpu_last_error(ctx_);
    throw Error(rc, msg);
  }

 private:
  setops_ctx *ctx_ = nullptr;
};

// Counter (setops/src/visitor.rs:24-49): counts matches.
struct Counter {
  uint64_t count = 0;
  void clear() { count = 0; }
};

// VecWriter (setops/src/visitor.rs:51-97): collects matches in order.
struct VecWriter {
  std::vector<uint32_t> items;
  void clear() { items.clear(); }
};

// BsrVec (setops/src/bsr.rs:20-30): structure-of-arrays base / state words.
struct BsrVec {
  std::vector<uint32_t> bases, states;
  std::size_t len() const { return bases.size(); }
};

// Intersect2<[u32], Counter>: adds |a ∩ b| to the counter.
inline void intersect(const Context &ctx, const std::vector<uint32_t> &a,
                      const std::vector<uint32_t> &b, Counter &v) {
  uint64_t n = 0;
  ctx.check(setops_gpu_intersect_count(ctx.get(), a.data(), a.size(), b.data(), b.size(), &n,
                                       SETOPS_HOST));
  v.count += n;
}

// Intersect2<[u32], VecWriter>: appends a ∩ b, ascending.
inline void intersect(const Context &ctx, const std::vector<uint32_t> &a,
                      const std::vector<uint32_t> &b, VecWriter &v) {
  const std::size_t cap = a.size() < b.size() ? a.size() : b.size();
  const std::size_t old = v.items.size();
  v.items.resize(old + cap);
  std::size_t n = 0;
  ctx.check(setops_gpu_intersect(ctx.get(), a.data(), a.size(), b.data(), b.size(),
                                 v.items.data() + old, cap, &n, SETOPS_HOST));
  v.items.resize(old + n);
}

// Intersect2C (setops/src/intersect.rs:41): into a caller-owned slice of
// capacity >= min(|a|, |b|) (the assert of qfilter_c.rs:11); returns the count.
inline std::size_t intersect_c(const Context &ctx, const std::vector<uint32_t> &a,
                               const std::vector<uint32_t> &b, uint32_t *out,
                               std::size_t out_cap) {
  std::size_t n = 0;
  ctx.check(setops_gpu_intersect(ctx.get(), a.data(), a.size(), b.data(), b.size(), out, out_cap,
                                 &n, SETOPS_HOST));
  return n;
}

// run_2set (setops/src/intersect.rs:44-53): a ∩ b as a new vector.
inline std::vector<uint32_t> run_2set(const Context &ctx, const std::vector<uint32_t> &a,
                                      const std::vector<uint32_t> &b) {
  VecWriter w;
  intersect(ctx, a, b, w);
  return std::move(w.items);
}

// Intersect2Bsr (setops/src/bsr.rs:16): out = a ∩ b in BSR form.
inline void intersect_bsr(const Context &ctx, const BsrVec &a, const BsrVec &b, BsrVec &out) {
  const std::size_t cap = a.len() < b.len() ? a.len() : b.len();
  out.bases.resize(cap);
  out.states.resize(cap);
  std::size_t n = 0;
  ctx.check(setops_gpu_intersect_bsr(ctx.get(), a.bases.data(), a.states.data(), a.len(),
                                     b.bases.data(), b.states.data(), b.len(), out.bases.data(),
                                     out.states.data(), cap, &n, SETOPS_HOST));
  out.bases.resize(n);
  out.states.resize(n);
}

// BsrVec::from_sorted / to_sorted_set (setops/src/bsr.rs:140-163, 77-88), on the GPU.
inline BsrVec bsr_from_sorted(const Context &ctx, const std::vector<uint32_t> &x) {
  BsrVec v;
  v.bases.resize(x.size());
  v.states.resize(x.size());
  std::size_t n = 0;
  ctx.check(setops_gpu_bsr_from_sorted(ctx.get(), x.data(), x.size(), v.bases.data(),
                                       v.states.data(), &n, SETOPS_HOST));
  v.bases.resize(n);
  v.states.resize(n);
  return v;
}

// svs_generic / run_kset (setops/src/intersect/svs.rs:50-73, intersect.rs:76-90):
// the intersection of k sets, smallest first, intermediates on the GPU.
inline std::vector<uint32_t> run_kset(const Context &ctx,
                                      const std::vector<std::vector<uint32_t>> &sets) {
  std::vector<const uint32_t *> ptrs;
  std::vector<std::size_t> lens;
  std::size_t cap = sets.empty() ? 0 : sets[0].size();
  for (const auto &s : sets) {
    ptrs.push_back(s.data());
    lens.push_back(s.size());
    if (s.size() < cap) cap = s.size();
  }
  std::vector<uint32_t> out(cap);
  std::size_t n = 0;
  ctx.check(setops_gpu_svs(ctx.get(), ptrs.data(), lens.data(), sets.size(), out.data(), cap, &n,
                           SETOPS_HOST));
  out.resize(n);
  return out;
}

}  // namespace setops_gpu
