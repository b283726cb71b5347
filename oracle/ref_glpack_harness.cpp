/*
 * ref_glpack_harness.cpp -- C entry point into the reference's own GL packing
 * (glPack.hpp / glPack.cpp and glVQ.hpp / glVQ.cpp, compiled unmodified from
 * the reference tree by oracle/Makefile).  TEST INFRASTRUCTURE ONLY: the
 * resulting oracle/_ref/libglp_ref_glpack.so pins the host restatement
 * glphase_gb300/glpack.py; it never runs on the product path.
 *
 *   glpr_glpack -> GLPack::GLPack (glPack.cpp:5-30, which trains the VQ
 *                  codebook, glVQ.cpp:21-146), GLPack::GetPackedGLs
 *                  (glPack.cpp:32-84) over all samples at once, and
 *                  GLPack::GetCodeBook.
 *
 * GSL is replaced by oracle/ref_shim's stand-in, whose draws are a counter,
 * so the reference's codebook here is a deterministic function of the GLs.
 */
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "glPack.hpp"

extern "C" {

// gl: [N][S][3] genotype likelihoods.  use_vq != 0: codebook of 2^bits
// entries (bits 2, 4 or 8), else the 8-bit (homRef, het) nibble form.
// packed_out: ceil(S / (32 / bits)) * N words (the reference's order: site
// block major, sample minor); codebook_out: 2^bits (homRef, het) pairs, or
// null.  Returns 0, or -1 when the reference throws or the sizes differ.
int glpr_glpack(const float *gl, uint32_t N, uint32_t S, int use_vq, uint32_t bits,
                uint32_t *packed_out, float *codebook_out) {
  gsl_rng *rng = gsl_rng_alloc(gsl_rng_default);
  int rc = 0;
  try {
    const std::vector<float> gls(gl, gl + (size_t)N * S * 3);
    GLPackHelper::Init init(gls, *rng);
    init.numSamps = N;
    init.sampleStride = N;
    init.useVQ = use_vq != 0;
    init.numBitsPerGL = use_vq ? bits : 8;
    GLPack pack(init);
    const std::vector<uint32_t> words = pack.GetPackedGLs();
    const uint32_t per = 32 / init.numBitsPerGL;
    if (words.size() != (size_t)((S + per - 1) / per) * N) {
      rc = -1;
    } else {
      std::memcpy(packed_out, words.data(), words.size() * sizeof(uint32_t));
      if (codebook_out) {
        const std::vector<std::pair<float, float>> cb = pack.GetCodeBook();
        for (size_t k = 0; k < cb.size(); ++k) {
          codebook_out[2 * k] = cb[k].first;
          codebook_out[2 * k + 1] = cb[k].second;
        }
      }
    }
  } catch (const std::exception &) {
    rc = -1;
  }
  gsl_rng_free(rng);
  return rc;
}

}  // extern "C"
