// Instantiations of the many chunk float emission generation kernels.
#include "glp_launch.h"

namespace glp {
GLP_GEN_TABLE(multi_kernel_f32, MultiFn, generation_multi_kernel, EmitF32, 1)
}  // namespace glp
