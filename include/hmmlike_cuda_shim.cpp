// The one translation unit a reference build compiles in place of
// src/hmmLike.cu: the HMMLikeCUDA functions declared extern by the
// reference's unchanged src/hmmLike.h (hmmLike.h:23-38), defined over the C
// ABI of libglphase_gpu.so.
#define HMMLIKE_CUDA_SHIM_OUT_OF_LINE
#include "hmmlike_cuda_shim.hpp"
