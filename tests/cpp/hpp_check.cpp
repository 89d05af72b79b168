// Self-checking use of include/setops_gpu.hpp (run by tests/test_cpp_header.py
// on a GPU): closed-form sets whose intersections are known.
#include <cstdio>
#include <vector>

#include "setops_gpu.hpp"

static std::vector<uint32_t> multiples(uint32_t step, uint32_t n) {
  std::vector<uint32_t> v(n);
  for (uint32_t i = 0; i < n; ++i) v[i] = step * i;
  return v;
}

int main() {
  setops_gpu::Context ctx(0);
  const auto a = multiples(3, 1u << 20), b = multiples(2, 1u << 21);
  // a ∩ b = multiples of 6 below min(3 * 2^20, 2 * 2^21) = 3 * 2^20
  const uint32_t lim = 3u << 20;
  const auto want = multiples(6, (lim + 5) / 6);
  setops_gpu::Counter c;
  setops_gpu::intersect(ctx, a, b, c);
  setops_gpu::VecWriter w;
  setops_gpu::intersect(ctx, a, b, w);
  if (c.count != want.size() || w.items != want) return std::printf("2-set mismatch\n"), 1;
  std::vector<uint32_t> slice(a.size());
  if (setops_gpu::intersect_c(ctx, a, b, slice.data(), slice.size()) != want.size())
    return std::printf("slice mismatch\n"), 1;
  if (setops_gpu::run_2set(ctx, b, a) != want) return std::printf("run_2set mismatch\n"), 1;
  // BSR: same sets in base/state form
  setops_gpu::BsrVec ba = setops_gpu::bsr_from_sorted(ctx, a), bb = setops_gpu::bsr_from_sorted(ctx, b), bo;
  setops_gpu::intersect_bsr(ctx, ba, bb, bo);
  uint64_t pc = 0;
  for (uint32_t s : bo.states) pc += uint64_t(__builtin_popcount(s));
  if (pc != want.size()) return std::printf("bsr mismatch\n"), 1;
  // k sets: multiples of 2, 3 and 5 -> multiples of 30
  const auto k = setops_gpu::run_kset(ctx, {multiples(5, 1u << 18), multiples(3, 1u << 19), b});
  if (k != multiples(30, ((5u << 18) + 29) / 30)) return std::printf("kset mismatch\n"), 1;
  // errors throw with the library's message
  try {
    std::vector<uint32_t> small(1);
    setops_gpu::intersect_c(ctx, a, b, small.data(), 0);
    return std::printf("no capacity error\n"), 1;
  } catch (const setops_gpu::Error &e) {
    if (e.code() != SETOPS_ERR_CAPACITY) return std::printf("wrong error %d\n", e.code()), 1;
  }
  std::printf("ok\n");
  return 0;
}
