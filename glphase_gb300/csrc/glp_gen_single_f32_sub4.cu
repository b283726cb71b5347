// Instantiations of the one chunk float emission generation kernels that normalise every
// 4 sites.
#include "glp_launch.h"

namespace glp {
GLP_GEN_TABLE(single_kernel_f32_sub4, SingleFn, generation_kernel, EmitF32, 2)
}  // namespace glp
