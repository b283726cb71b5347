// glp_tract.h -- the runs of agreeing common sites behind the kNN
// tract-length metric (insti -T: the number of common sites minus
// Haplotype::MaxTractLen, src/haplotype.cpp:62-90, over the common sites of
// KNN::CutDownHaps, src/kNN.cpp:216-257), one 64-site word at a time.
//
// Plain C++ or CUDA: knn_tract_dist_kernel (glp_knn.cuh) runs these on the
// device; the host build lets the same code be checked on the CPU.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define GLP_TRACT_FN __host__ __device__ __forceinline__
#else
#define GLP_TRACT_FN inline
#endif

namespace glp {

GLP_TRACT_FN uint32_t tract_popc(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return (uint32_t)__popcll(x);
#else
  return (uint32_t)__builtin_popcountll(x);
#endif
}

// Lowest and highest set bit of x != 0.
GLP_TRACT_FN int tract_lsb(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __ffsll((long long)x) - 1;
#else
  return __builtin_ctzll(x);
#endif
}

GLP_TRACT_FN int tract_msb(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return 63 - __clzll((long long)x);
#else
  return 63 - __builtin_clzll(x);
#endif
}

GLP_TRACT_FN uint32_t tract_max(uint32_t a, uint32_t b) { return a > b ? a : b; }

// Runs of agreeing common sites in a stretch of words: len common sites, pre
// of them before the first disagreement, suf after the last, best the longest
// run; pre == len when the stretch has no disagreement.
struct Tract {
  uint32_t len, pre, suf, best;
};

// One word: x the disagreements at common sites, m the common sites.
GLP_TRACT_FN Tract tract_word(uint64_t x, uint64_t m) {
  Tract t;
  t.len = tract_popc(m);
  if (x == 0) {
    t.pre = t.suf = t.best = t.len;
    return t;
  }
  const int lo = tract_lsb(x), hi = tract_msb(x);
  if (m == ~0ull) {  // every site common: the longest run of agreements in log steps
    const uint64_t r1 = ~x, r2 = r1 & (r1 >> 1), r4 = r2 & (r2 >> 2), r8 = r4 & (r4 >> 4),
                   r16 = r8 & (r8 >> 8), r32 = r16 & (r16 >> 16);
    // cur: the starts of runs of at least n agreements; n grows greedily
    uint64_t cur = ~0ull;
    uint32_t n = 0;
    const uint64_t rs[6] = {r32, r16, r8, r4, r2, r1};
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int i = 0; i < 6; ++i) {
      const uint64_t cand = cur & (rs[i] >> n);
      if (cand) {
        n += 32u >> i;
        cur = cand;
      }
    }
    t.pre = (uint32_t)lo;
    t.suf = (uint32_t)(63 - hi);
    t.best = n;
    return t;
  }
  t.pre = tract_popc(m & ((1ull << lo) - 1ull));
  t.suf = hi == 63 ? 0u : tract_popc(m >> (hi + 1));
  uint32_t best = tract_max(t.pre, t.suf);
  int prev = lo;
  for (uint64_t y = x & (x - 1ull); y; y &= y - 1ull) {  // runs between disagreements
    const int q = tract_lsb(y);                          // prev < q <= 63
    const uint64_t between = ((1ull << q) - 1ull) & ~((2ull << prev) - 1ull);
    best = tract_max(best, tract_popc(m & between));
    prev = q;
  }
  t.best = best;
  return t;
}

// The stretch l followed by the stretch r.
GLP_TRACT_FN Tract tract_join(const Tract l, const Tract r) {
  Tract t;
  t.len = l.len + r.len;
  t.pre = l.pre == l.len ? l.len + r.pre : l.pre;
  t.suf = r.suf == r.len ? r.len + l.suf : r.suf;
  t.best = tract_max(tract_max(l.best, r.best), l.suf + r.pre);
  return t;
}

}  // namespace glp
