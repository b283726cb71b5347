// Instantiations of the many chunk float emission generation kernels that normalise every
// 4 sites.
#include "glp_launch.h"

namespace glp {
GLP_GEN_TABLE(multi_kernel_f32_sub4, MultiFn, generation_multi_kernel, EmitF32, 2)
}  // namespace glp
