// The reference's device API (namespace HMMLikeCUDA, src/hmmLike.h:23-38)
// driven from C++ the way src/hmmLike.cpp drives it, linked against the
// out-of-line shim (include/hmmlike_cuda_shim.cpp) and libglphase_gpu.so.
// The declarations below are those a translation unit compiled against the
// reference's hmmLike.h sees (every function extern).
//
// Checks, printing one line per check and exiting non-zero on the first
// failure:
//  * calls before SetDevice and mis-sized arguments raise std::runtime_error
//    (the reference's convention for size errors, hmmLike.cu:333-336,
//    409-414) and leave the context usable;
//  * the planted-parent run of src/testing/cuda_tests.cpp:205-322 through
//    RunHMMOnDevice with 4-bit VQ GLs: 12 haplotypes x 1,024 sites,
//    haplotypes 5 and 6 carry the alternative allele over words 0 and 5,
//    haplotypes 7 and 8 over words 1 and 7, sample 0 is confidently hom-alt
//    over words 0 and 5 and sample 1 over words 1 and 7; each sample's final
//    father pair and mother pair must each hold one of its planted
//    haplotypes;
//  * a second SetDevice replaces the context and Cleanup releases it.
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace HMMLikeCUDA {
extern void CheckDevice();
extern void SetDevice(int devID);
extern void CopyTranToDevice(const std::vector<float> &tran);
extern void CopyMutationMatToDevice(const float (*mutMat)[4][4]);
extern void CopyPackedGLsToDevice(const std::vector<uint32_t> &packedGLs);
extern void CopyCodeBookToDevice(const std::vector<std::pair<float, float> > &codeBook);
extern void RunHMMOnDevice(const std::vector<uint64_t> &hapPanel,
                           const std::vector<unsigned> &extraPropHaps, unsigned numSites,
                           unsigned numSamples, unsigned numCycles,
                           std::vector<unsigned> &hapIdxs, unsigned long seed);
extern void Cleanup();
}  // namespace HMMLikeCUDA

namespace {

int failures = 0;

void check(bool ok, const char *what) {
  std::printf("%s %s\n", ok ? "ok  " : "FAIL", what);
  if (!ok)
    ++failures;
}

template <class F>
bool throws(F f, const char *needle) {
  try {
    f();
  } catch (const std::runtime_error &e) {
    return std::string(e.what()).find(needle) != std::string::npos;
  }
  return false;
}

// Nearest entry of the (homRef, het) codebook, by squared distance.
unsigned nearest(const std::vector<std::pair<float, float> > &cb, float r, float h) {
  unsigned best = 0;
  float bd = 1e30f;
  for (unsigned k = 0; k < cb.size(); ++k) {
    const float a = cb[k].first - r, b = cb[k].second - h, d = a * a + b * b;
    if (d < bd) {
      bd = d;
      best = k;
    }
  }
  return best;
}

}  // namespace

int main() {
  const unsigned numSamps = 2, numHaps = 12, numSites = 1024, numWords = numSites / 64;
  const unsigned numCycles = 100;

  check(throws([] { HMMLikeCUDA::CopyTranToDevice(std::vector<float>(30)); },
               "SetDevice was not called"),
        "a copy before SetDevice raises");
  HMMLikeCUDA::CheckDevice();
  HMMLikeCUDA::SetDevice(0);

  // model of the reference test's second part (cuda_tests.cpp:249-281)
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
  check(throws([] { HMMLikeCUDA::CopyTranToDevice(std::vector<float>(10)); }, "multiple of 3"),
        "a transition vector that is not [S][3] raises");
  HMMLikeCUDA::CopyTranToDevice(tran);
  HMMLikeCUDA::CopyMutationMatToDevice(&mutMat);

  // 16-entry (homRef, het) codebook and the samples' 4-bit codes, eight per
  // word, most significant nibble first (glPack.cpp:104-109)
  std::vector<std::pair<float, float> > cb;
  for (unsigned a = 0; a < 4; ++a)
    for (unsigned b = 0; b < 4; ++b)
      cb.push_back(std::make_pair(a / 3.0f, (a + b <= 3) ? b / 3.0f : 0.0f));
  std::vector<uint32_t> packed((size_t)numSites / 8 * numSamps, 0);
  for (unsigned s = 0; s < numSamps; ++s)
    for (unsigned m = 0; m < numSites; ++m) {
      const unsigned w = m / 64;
      const bool planted = s == 0 ? (w == 0 || w == 5) : (w == 1 || w == 7);
      // a mild mixture elsewhere, hom-alt (homRef 0, het 0) where planted
      const float r = planted ? 0.f : 0.2f + 0.1f * (m % 5), h = planted ? 0.f : 0.3f;
      const uint32_t code = nearest(cb, r, h);
      packed[(size_t)(m / 8) * numSamps + s] |= code << (28 - 4 * (m % 8));
    }
  HMMLikeCUDA::CopyCodeBookToDevice(cb);
  HMMLikeCUDA::CopyPackedGLsToDevice(packed);

  std::vector<uint64_t> panel((size_t)numWords * numHaps, 0);
  const uint64_t all = ~(uint64_t)0;
  panel[5 * numWords] = panel[6 * numWords] = all;
  panel[5 * numWords + 5] = panel[6 * numWords + 5] = all;
  panel[7 * numWords + 1] = panel[8 * numWords + 1] = all;
  panel[7 * numWords + 7] = panel[8 * numWords + 7] = all;

  // initial quadruples and proposals, uniform over the other samples'
  // haplotypes (UnifSampler::SampleHap, sampler.cpp:29-39), transposed
  // [4][N] / [C][N] as RunHMMOnSamples lays them out (hmmLike.cpp:90-102)
  uint64_t lcg = 112;
  auto draw = [&](unsigned s) {
    for (;;) {
      lcg = lcg * 6364136223846793005ull + 1442695040888963407ull;
      const unsigned h = (unsigned)(lcg >> 33) % numHaps;
      if (h / 2 != s)
        return h;
    }
  };
  std::vector<unsigned> idx(4 * numSamps), props((size_t)numCycles * numSamps);
  for (unsigned s = 0; s < numSamps; ++s) {
    for (unsigned k = 0; k < 4; ++k)
      idx[s + k * numSamps] = draw(s);
    for (unsigned c = 0; c < numCycles; ++c)
      props[c * numSamps + s] = draw(s);
  }
  std::vector<unsigned> short_idx(3);
  check(throws([&] {
          HMMLikeCUDA::RunHMMOnDevice(panel, props, numSites, numSamps, numCycles, short_idx,
                                      5ul);
        }, "size mismatch"),
        "mis-sized quadruples raise");
  HMMLikeCUDA::RunHMMOnDevice(panel, props, numSites, numSamps, numCycles, idx, 5ul);
  std::printf("quadruples [4][N]:");
  for (unsigned v : idx)
    std::printf(" %u", v);
  std::printf("\n");
  for (unsigned s = 0; s < numSamps; ++s) {
    const unsigned lo = s ? 7 : 5, hi = s ? 8 : 6;
    auto in = [&](unsigned h) { return h >= lo && h <= hi; };
    const unsigned f0 = idx[s], f1 = idx[s + numSamps], m0 = idx[s + 2 * numSamps],
                   m1 = idx[s + 3 * numSamps];
    check(in(f0) || in(f1), s ? "sample 1's father pair holds 7 or 8"
                              : "sample 0's father pair holds 5 or 6");
    check(in(m0) || in(m1), s ? "sample 1's mother pair holds 7 or 8"
                              : "sample 0's mother pair holds 5 or 6");
  }
  HMMLikeCUDA::SetDevice(0);  // replaces the context
  check(throws([] { HMMLikeCUDA::CopyPackedGLsToDevice(std::vector<uint32_t>()); }, ""),
        "an empty GL vector raises on the new context");
  HMMLikeCUDA::Cleanup();
  check(throws([] { HMMLikeCUDA::CopyTranToDevice(std::vector<float>(30)); },
               "SetDevice was not called"),
        "Cleanup releases the context");
  std::printf("%d failure(s)\n", failures);
  return failures ? 1 : 0;
}
