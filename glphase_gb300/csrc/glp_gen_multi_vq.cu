// Instantiations of the many chunk VQ emission generation kernels.
#include "glp_launch.h"

namespace glp {
GLP_GEN_TABLE(multi_kernel_vq, MultiFn, generation_multi_kernel, EmitVQ, 1)
}  // namespace glp
