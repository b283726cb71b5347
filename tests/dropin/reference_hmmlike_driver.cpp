// The reference's own host driver on the drop-in: src/hmmLike.cpp (class
// HMMLike), src/glPack.cpp, src/glVQ.cpp and src/sampler.cpp compiled
// unchanged from the reference tree, with its unchanged src/hmmLike.h
// declaring the device API, linked against include/hmmlike_cuda_shim.cpp and
// libglphase_gpu.so in place of src/hmmLike.cu.  GSL and the Boost-based
// olivier/utils.hpp are replaced by the stand-ins of oracle/ref_shim (GSL's
// draws become a counter).
//
// The run is the planted-parent case of src/testing/cuda_tests.cpp:205-322,
// driven the way Insti::estimate drives it (insti.cpp:1634-1645): GLPack
// with 4-bit VQ codes over 2 samples x 1,024 sites, a UnifSampler over 12
// haplotypes, HMMLike's constructor (CheckDevice, SetDevice and the model
// copies) and one RunHMMOnSamples.  Haplotypes 5 and 6 carry the alternative
// allele over words 0 and 5, haplotypes 7 and 8 over words 1 and 7; sample 0
// is hom-alt over words 0 and 5, sample 1 over words 1 and 7, so each
// sample's father pair and mother pair must each end with one of its planted
// haplotypes.
//
// Exit status: 0 when the run passed on a device; 3 when no device is
// visible and HMMLike's constructor saw CheckDevice's std::runtime_error
// (what the reference's caller sees on a machine without a GPU); 1
// otherwise.
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "hmmLike.hpp"

int main() {
  const unsigned numSamps = 2, numHaps = 12, numSites = 1024, numWords = numSites / 64;
  const unsigned numCycles = 100;

  // GLs [sample][site][homRef, het, homAlt]: hom-alt where planted, a mild
  // mixture elsewhere
  std::vector<float> gls((size_t)numSamps * numSites * 3);
  for (unsigned s = 0; s < numSamps; ++s)
    for (unsigned m = 0; m < numSites; ++m) {
      const unsigned w = m / 64;
      const bool planted = s == 0 ? (w == 0 || w == 5) : (w == 1 || w == 7);
      float *g = &gls[((size_t)s * numSites + m) * 3];
      g[0] = planted ? 0.f : 0.2f + 0.1f * (m % 5);
      g[1] = planted ? 0.f : 0.3f;
      g[2] = 1.f - g[0] - g[1];
    }

  // the model constants of the reference test (cuda_tests.cpp:249-281)
  float mu = 0;
  for (unsigned i = 1; i < numHaps; ++i)
    mu += 1.0f / i;
  mu = 1 / mu;
  const float rho = 0.5f * mu * (numSites - 1) / (numSites * 1000.0f);
  mu = mu / (numHaps + mu);
  float mutMat[4][4];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j)
      mutMat[i][j] = (i == j) ? (1 - mu) * (1 - mu) : (i + j == 3) ? mu * mu : mu * (1 - mu);
  std::vector<float> tran(numSites * 3, 0.f);
  for (unsigned m = numSites - 1; m; --m) {
    const float d = rho * 1000.0f, r = d / (d + 4);
    tran[m * 3] = (1 - r) * (1 - r);
    tran[m * 3 + 1] = r * (1 - r);
    tran[m * 3 + 2] = r * r;
  }

  std::vector<uint64_t> panel((size_t)numWords * numHaps, 0);
  const uint64_t all = ~(uint64_t)0;
  panel[5 * numWords] = panel[6 * numWords] = all;
  panel[5 * numWords + 5] = panel[6 * numWords + 5] = all;
  panel[7 * numWords + 1] = panel[8 * numWords + 1] = all;
  panel[7 * numWords + 7] = panel[8 * numWords + 7] = all;

  gsl_rng *rng = gsl_rng_alloc(gsl_rng_default);
  GLPackHelper::Init init(gls, *rng);
  init.numSamps = numSamps;
  init.sampleStride = numSamps;
  init.useVQ = true;
  init.numBitsPerGL = BITSPERCODE;
  GLPack glPack(init);
  std::shared_ptr<Sampler> sampler = std::make_shared<UnifSampler>(rng, numSamps, numHaps);

  int rc = 0;
  try {
    HMMLike hmm(panel, numHaps, glPack, numCycles, tran, &mutMat, sampler, *rng, 0);
    unsigned first = 0, last = 0;
    const std::vector<unsigned> idx = hmm.RunHMMOnSamples(first, last);  // [N][4]
    std::printf("samples %u..%u, quadruples [N][4]:", first, last);
    for (unsigned v : idx)
      std::printf(" %u", v);
    std::printf("\n");
    if (first != 0 || last != numSamps - 1 || idx.size() != 4 * numSamps)
      rc = 1;
    for (unsigned s = 0; s < numSamps && rc == 0; ++s) {
      const unsigned lo = s ? 7 : 5, hi = s ? 8 : 6;
      auto in = [&](unsigned h) { return h >= lo && h <= hi; };
      const unsigned *q = &idx[4 * s];
      const bool father = in(q[0]) || in(q[1]), mother = in(q[2]) || in(q[3]);
      std::printf("sample %u: father pair %s, mother pair %s\n", s,
                  father ? "planted" : "MISSING", mother ? "planted" : "MISSING");
      if (!father || !mother)
        rc = 1;
    }
  } catch (const std::runtime_error &e) {
    std::printf("runtime_error: %s\n", e.what());
    rc = std::string(e.what()).find("no sm_103 device") != std::string::npos ? 3 : 1;
  }
  gsl_rng_free(rng);
  return rc;
}
