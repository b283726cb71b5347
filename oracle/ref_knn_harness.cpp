/*
 * ref_knn_harness.cpp -- C entry points into the reference's own kNN
 * surrogate restriction (kNN.hpp / kNN.cpp, haplotype.hpp / haplotype.cpp and
 * the Sampler base of sampler.cpp, compiled unmodified from the reference tree
 * by oracle/Makefile).  TEST INFRASTRUCTURE ONLY: the resulting
 * oracle/_ref/libglp_ref_knn.so pins the C restatement of the kNN build in
 * glp_oracle.c; it never runs on the product path.
 *
 *   glpr_knn        -> KNN::KNN (kNN.cpp:7-72: allele frequencies of the
 *                      given haplotypes, CutDownHaps, ClusterHaps) and
 *                      KNN::Neighbors (kNN.cpp:92-97) for every sample
 *   glpr_max_tract  -> Haplotype::MaxTractLen (haplotype.cpp:62-90)
 *   glpr_hamming    -> Haplotype::HammingDist (haplotype.cpp:22-33)
 *
 * KNN writes progress lines to std::cout; they are discarded here.
 */
#include <cstdint>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <vector>

#include "kNN.hpp"

namespace {

// Sends std::cout to a string buffer for the lifetime of the object.
struct QuietCout {
  std::ostringstream sink;
  std::streambuf *old;
  QuietCout() : old(std::cout.rdbuf(sink.rdbuf())) {}
  ~QuietCout() { std::cout.rdbuf(old); }
};

Haplotype from_bits(const uint8_t *bits, uint32_t n) {
  Haplotype h(n);
  for (uint32_t i = 0; i < n; ++i)
    h.Set(i, bits[i] != 0);
  return h;
}

}  // namespace

extern "C" {

// Neighbour lists of all H/2 samples: out[s][0 .. 2 ceil(k/2)) =
// KNN::Neighbors(2 s).  metric 0 = Hamming, 1 = tract length.  Returns 0, or
// -1 when the reference throws (its bound checks) or the list length differs.
int glpr_knn(const uint64_t *haps, uint32_t H, uint32_t wn, uint32_t S, uint32_t k,
             double lb, double ub, int use_maf, int metric, uint32_t *out) {
  gsl_rng *rng = gsl_rng_alloc(gsl_rng_default);
  int rc = 0;
  try {
    QuietCout quiet;
    std::vector<uint64_t> v(haps, haps + (size_t)H * wn);
    KNN knn(k, v, wn, S, lb, ub, use_maf != 0, rng,
            metric ? kNNDistT::tracLen : kNNDistT::hamming);
    const size_t len = 2 * ((k + 1) / 2);
    for (uint32_t s = 0; s < H / 2 && rc == 0; ++s) {
      const std::vector<unsigned> nb = knn.Neighbors(2 * s);
      if (nb.size() != len)
        rc = -1;
      else
        for (size_t i = 0; i < len; ++i)
          out[s * len + i] = nb[i];
    }
  } catch (const std::exception &) {
    rc = -1;
  }
  gsl_rng_free(rng);
  return rc;
}

// Longest run of agreeing sites of two n-site haplotypes given one allele
// (0/1) a byte.
uint32_t glpr_max_tract(const uint8_t *a, const uint8_t *b, uint32_t n) {
  return from_bits(a, n).MaxTractLen(from_bits(b, n));
}

uint32_t glpr_hamming(const uint8_t *a, const uint8_t *b, uint32_t n) {
  return from_bits(a, n).HammingDist(from_bits(b, n));
}

}  // extern "C"
