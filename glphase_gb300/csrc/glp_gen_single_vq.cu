// Instantiations of the one chunk VQ emission generation kernels.
#include "glp_launch.h"

namespace glp {
GLP_GEN_TABLE(single_kernel_vq, SingleFn, generation_kernel, EmitVQ, 1)
}  // namespace glp
