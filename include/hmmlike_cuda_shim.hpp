// hmmlike_cuda_shim.hpp -- the reference's device API, namespace HMMLikeCUDA
// with the exact signatures of src/hmmLike.h:23-38, implemented inline over
// the C ABI of glphase_gpu.h.  A C++ caller written against the reference
// (src/hmmLike.cpp, Insti::cudaSolve) includes this header instead of
// hmmLike.h and links libglphase_gpu.so; nothing else changes.
//
// Two ways to use it:
//  * include it in place of hmmLike.h: the functions are inline;
//  * keep the reference's own hmmLike.h (it declares the functions extern)
//    and compile ONE translation unit that defines HMMLIKE_CUDA_SHIM_OUT_OF_LINE
//    before including this header: it then defines the functions with external
//    linkage, so src/hmmLike.cpp compiles unchanged and links against them in
//    place of hmmLike.cu.
//
// Status codes become std::runtime_error, the reference's own convention for
// size errors (src/hmmLike.cu:333-336, 409-414); unlike the reference, CUDA
// errors no longer call exit().  One context per process, as the reference's
// file-static device state.
#ifndef HMMLIKE_CUDA_SHIM_HPP
#define HMMLIKE_CUDA_SHIM_HPP

#include <stdint.h>

#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "glphase_gpu.h"

static_assert(sizeof(unsigned) == sizeof(uint32_t), "unsigned must be 32 bits");

#ifdef HMMLIKE_CUDA_SHIM_OUT_OF_LINE
#define HMMLIKE_CUDA_SHIM_FN
#else
#define HMMLIKE_CUDA_SHIM_FN inline
#endif

namespace HMMLikeCUDA {

namespace detail {
inline glp_ctx *&context() {
  static glp_ctx *ctx = 0;
  return ctx;
}
inline void check(int rc, const char *what) {
  if (rc != GLP_OK)
    throw std::runtime_error(std::string("[HMMLikeCUDA] ") + what + ": " +
                             glp_last_error(context()));
}
inline glp_ctx *need() {
  if (!context())
    throw std::runtime_error("[HMMLikeCUDA] SetDevice was not called");
  return context();
}
}  // namespace detail

// src/hmmLike.cu:266-320
HMMLIKE_CUDA_SHIM_FN void CheckDevice() {
  int n = 0, ma = 0, mi = 0, sms = 0;
  if (glp_check_device(0, &n, &ma, &mi, &sms) != GLP_OK)
    throw std::runtime_error("[HMMLikeCUDA] no sm_103 device found");
}

// src/hmmLike.cu:244-264
HMMLIKE_CUDA_SHIM_FN void SetDevice(int devID) {
  if (detail::context()) {
    glp_destroy(detail::context());
    detail::context() = 0;
  }
  detail::check(glp_create(devID, &detail::context()), "SetDevice");
}

// src/hmmLike.cu:322-337
HMMLIKE_CUDA_SHIM_FN void CopyTranToDevice(const std::vector<float> &tran) {
  if (tran.size() % 3)
    throw std::runtime_error("[HMMLikeCUDA] tran size is not a multiple of 3");
  detail::check(glp_set_tran(detail::need(), tran.data(), (uint32_t)(tran.size() / 3)),
                "CopyTranToDevice");
}

// src/hmmLike.cu:339-355
HMMLIKE_CUDA_SHIM_FN void CopyMutationMatToDevice(const float (*mutMat)[4][4]) {
  detail::check(glp_set_mutation_mat(detail::need(), &(*mutMat)[0][0]),
                "CopyMutationMatToDevice");
}

// src/hmmLike.cu:357-366
HMMLIKE_CUDA_SHIM_FN void CopyPackedGLsToDevice(const std::vector<uint32_t> &packedGLs) {
  detail::check(glp_set_packed_gls(detail::need(), packedGLs.data(), packedGLs.size()),
                "CopyPackedGLsToDevice");
}

// src/hmmLike.cu:368-383
HMMLIKE_CUDA_SHIM_FN void CopyCodeBookToDevice(const std::vector<std::pair<float, float> > &codeBook) {
  std::vector<float> flat;
  flat.reserve(codeBook.size() * 2);
  for (size_t i = 0; i < codeBook.size(); ++i) {
    flat.push_back(codeBook[i].first);
    flat.push_back(codeBook[i].second);
  }
  detail::check(glp_set_codebook(detail::need(), flat.data(), (uint32_t)codeBook.size()),
                "CopyCodeBookToDevice");
}

// src/hmmLike.cu:399-572
HMMLIKE_CUDA_SHIM_FN void RunHMMOnDevice(const std::vector<uint64_t> &hapPanel,
                           const std::vector<unsigned> &extraPropHaps, unsigned numSites,
                           unsigned numSamples, unsigned numCycles,
                           std::vector<unsigned> &hapIdxs, unsigned long seed) {
  if (hapIdxs.size() != (size_t)numSamples * 4 ||
      extraPropHaps.size() != (size_t)numSamples * numCycles)
    throw std::runtime_error("[HMMLikeCUDA] RunHMMOnDevice: size mismatch");
  detail::check(glp_run_hmm_on_device(detail::need(), hapPanel.data(), hapPanel.size(),
                                      extraPropHaps.data(), numSites, numSamples, numCycles,
                                      hapIdxs.data(), (uint64_t)seed),
                "RunHMMOnDevice");
}

// src/hmmLike.cu:385-397 (without the device reset)
HMMLIKE_CUDA_SHIM_FN void Cleanup() {
  if (detail::context()) {
    glp_destroy(detail::context());
    detail::context() = 0;
  }
}

}  // namespace HMMLikeCUDA

#endif
