// Instantiations of the one chunk float emission generation kernels.
#include "glp_launch.h"

namespace glp {
GLP_GEN_TABLE(single_kernel_f32, SingleFn, generation_kernel, EmitF32, 1)
}  // namespace glp
