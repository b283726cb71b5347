/*
 * glp_rng.h -- counter-based random streams shared by the CUDA kernels and the
 * CPU oracle, so that a generation can be replayed bit-for-bit on either side
 * without materialising a trace.
 *
 * Generator: Philox4x32-10 as published in J. K. Salmon, M. A. Moraes,
 * R. O. Dror, D. E. Shaw, "Parallel Random Numbers: As Easy as 1, 2, 3",
 * SC'11 (round function, multipliers and Weyl key increments from that paper).
 *
 * The reference draws from stateful generators instead: GSL's MT19937 on the
 * CPU path (impute.cpp:470, insti.cpp:1506, MHSampler.hpp:92) and curand
 * XORWOW on the GPU path (hmmLike.cu:188, 196, 225), seeded from time(NULL)
 * (impute.hpp:103-106), so its streams are not reproducible.  Here every draw
 * is a pure function of (seed, generation, sample, index, stream tag).
 *
 * Streams (counter = {index, sample, generation, tag}, key = seed):
 *   GLP_TAG_MH    index = cycle : x0 & 3 -> replaced parent slot
 *                                 (x1, x2) -> 53-bit double uniform for accept
 *   GLP_TAG_WORK  index = site/4: x[site % 4] -> 24-bit float uniform
 *   GLP_TAG_PROP  index = cycle : proposal draws of the device sampler
 *   GLP_TAG_INIT  index = slot  : initial quadruple draws of the device sampler
 *
 * This header is plain C99 / C++ / CUDA: no intrinsics, identical results on
 * x86-64, aarch64 and the device.
 */
#ifndef GLP_RNG_H
#define GLP_RNG_H

#include <stdint.h>

#if defined(__CUDACC__)
#define GLP_HD __host__ __device__ __forceinline__
#else
#define GLP_HD static inline
#endif

#define GLP_TAG_MH 0u
#define GLP_TAG_WORK 1u
#define GLP_TAG_PROP 2u
#define GLP_TAG_INIT 3u

typedef struct glp_u32x4 {
  uint32_t v[4];
} glp_u32x4;

GLP_HD uint32_t glp_mulhi32(uint32_t a, uint32_t b) {
  return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
}

/* Philox4x32 with 10 rounds (Salmon et al. 2011, section 4.2). */
GLP_HD glp_u32x4 glp_philox4x32_10(glp_u32x4 ctr, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  uint32_t c0 = ctr.v[0], c1 = ctr.v[1], c2 = ctr.v[2], c3 = ctr.v[3];
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = M0 * c0, hi0 = glp_mulhi32(M0, c0);
    const uint32_t lo1 = M1 * c2, hi1 = glp_mulhi32(M1, c2);
    const uint32_t n0 = hi1 ^ c1 ^ k0;
    const uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += W0;
    k1 += W1;
  }
  glp_u32x4 out;
  out.v[0] = c0;
  out.v[1] = c1;
  out.v[2] = c2;
  out.v[3] = c3;
  return out;
}

GLP_HD glp_u32x4 glp_draw(uint64_t seed, uint32_t generation, uint32_t sample,
                          uint32_t index, uint32_t tag) {
  glp_u32x4 c;
  c.v[0] = index;
  c.v[1] = sample;
  c.v[2] = generation;
  c.v[3] = tag;
  return glp_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

/* float uniform in [0, 1) with 24 random bits: exact in binary32. */
GLP_HD float glp_u24(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

/* double uniform in [0, 1) with 53 random bits. */
GLP_HD double glp_u53(uint32_t a, uint32_t b) {
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) *
         (1.0 / 9007199254740992.0);
}

/* MH cycle draws: replaced slot (0..3) and the accept uniform. */
GLP_HD void glp_mh_draw(uint64_t seed, uint32_t generation, uint32_t sample,
                        uint32_t cycle, uint32_t *slot, double *u) {
  glp_u32x4 x = glp_draw(seed, generation, sample, cycle, GLP_TAG_MH);
  *slot = x.v[0] & 3u;
  *u = glp_u53(x.v[1], x.v[2]);
}

/* 64-bit draw from two words, reduced modulo n (n <= 2^32; the bias is at
 * most n / 2^64). */
GLP_HD uint32_t glp_below(uint32_t hi, uint32_t lo, uint32_t n) {
  return (uint32_t)((((uint64_t)hi << 32) | (uint64_t)lo) % (uint64_t)n);
}

/* Surrogate draw for sample s, uniform over haplotypes [lo, hi) except the
 * sample's own pair 2s, 2s+1 (UnifSampler::SampleHap, sampler.cpp:29-39,
 * drawn by rejection there; here by skipping the pair).  Returns hi when the
 * range holds no other haplotype. */
GLP_HD uint32_t glp_uniform_hap(glp_u32x4 x, uint32_t s, uint32_t lo, uint32_t hi) {
  const uint32_t a = 2u * s;
  const int own = (a >= lo && a + 1u < hi);
  const uint32_t n = hi - lo - (own ? 2u : 0u);
  if (hi <= lo || n == 0u)
    return hi;
  uint32_t h = lo + glp_below(x.v[0], x.v[1], n);
  if (own && h >= a)
    h += 2u;
  return h;
}

/* Surrogate draw from a neighbour list of length klen (KNN::SampleHap,
 * kNN.cpp:74-90): the position is uniform over the list. */
GLP_HD uint32_t glp_table_pos(glp_u32x4 x, uint32_t klen) {
  return glp_below(x.v[2], x.v[3], klen);
}

/* One surrogate of sample s: slot `index` of the initial quadruple
 * (tag GLP_TAG_INIT) or the proposal of cycle `index` (GLP_TAG_PROP), from
 * the neighbour table nbr [N][klen] when given, else uniform over [lo, hi). */
GLP_HD uint32_t glp_surrogate(uint64_t seed, uint32_t generation, uint32_t s,
                              uint32_t index, uint32_t tag, uint32_t lo, uint32_t hi,
                              const uint32_t *nbr, uint32_t klen) {
  const glp_u32x4 x = glp_draw(seed, generation, s, index, tag);
  if (nbr)
    return nbr[(size_t)s * klen + glp_table_pos(x, klen)];
  return glp_uniform_hap(x, s, lo, hi);
}

/* The proposal of a chain's first cycle under kick-start (insti.cpp:1505-1511
 * with --kickstart; Sampler::SampleHap(I, true), sampler.cpp:12-27): a
 * reference-panel haplotype, index >= ref_lo.  The reference redraws from its
 * sampler until the index is one; here the draw is uniform over the
 * neighbour list's panel entries (in list order) when a list is given and
 * holds any, else uniform over [ref_lo, hi) (where the reference would loop
 * forever on a list without panel entries). */
GLP_HD uint32_t glp_surrogate_ref(uint64_t seed, uint32_t generation, uint32_t s,
                                  uint32_t index, uint32_t tag, uint32_t ref_lo, uint32_t hi,
                                  const uint32_t *nbr, uint32_t klen) {
  const glp_u32x4 x = glp_draw(seed, generation, s, index, tag);
  if (nbr) {
    const uint32_t *row = nbr + (size_t)s * klen;
    uint32_t c = 0;
    for (uint32_t k = 0; k < klen; ++k)
      c += row[k] >= ref_lo ? 1u : 0u;
    if (c) {
      uint32_t j = glp_below(x.v[2], x.v[3], c);
      for (uint32_t k = 0; k < klen; ++k)
        if (row[k] >= ref_lo) {
          if (j == 0)
            return row[k];
          --j;
        }
    }
  }
  return glp_uniform_hap(x, s, ref_lo, hi);
}

/* hmm_work uniform for one site. */
GLP_HD float glp_work_uniform(uint64_t seed, uint32_t generation,
                              uint32_t sample, uint32_t site) {
  glp_u32x4 x = glp_draw(seed, generation, sample, site >> 2, GLP_TAG_WORK);
  return glp_u24(x.v[site & 3u]);
}

#endif /* GLP_RNG_H */
