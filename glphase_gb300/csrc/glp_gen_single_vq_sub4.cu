// Instantiations of the one chunk VQ emission generation kernels that normalise every
// 4 sites.
#include "glp_launch.h"

namespace glp {
GLP_GEN_TABLE(single_kernel_vq_sub4, SingleFn, generation_kernel, EmitVQ, 2)
}  // namespace glp
