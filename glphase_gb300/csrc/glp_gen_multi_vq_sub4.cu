// Instantiations of the many chunk VQ emission generation kernels that normalise every
// 4 sites.
#include "glp_launch.h"

namespace glp {
GLP_GEN_TABLE(multi_kernel_vq_sub4, MultiFn, generation_multi_kernel, EmitVQ, 2)
}  // namespace glp
