// Kernel tables of the generation kernels.
//
// Each (entry kind, emission source, normalisation block) triple is
// instantiated in its own translation unit (glp_gen_*.cu) so the
// instantiations compile in parallel; the host code picks a kernel by its
// speculation width: P lanes per sample (P/2 evaluations a round).
#pragma once

#include "glp_kernels.cuh"

namespace glp {

using SingleFn = void (*)(const GenParams);
using MultiFn = void (*)(const MultiParams);

SingleFn single_kernel_f32(uint32_t P);
SingleFn single_kernel_vq(uint32_t P);
MultiFn multi_kernel_f32(uint32_t P);
MultiFn multi_kernel_vq(uint32_t P);
// the same with normalisation every 4 sites
SingleFn single_kernel_f32_sub4(uint32_t P);
SingleFn single_kernel_vq_sub4(uint32_t P);
MultiFn multi_kernel_f32_sub4(uint32_t P);
MultiFn multi_kernel_vq_sub4(uint32_t P);

}  // namespace glp

// Body of one table: KERNEL<P, EMIT, SUB> for P = 2, 4, 8, 16, 32 (narrower
// requests get two lanes: one evaluation a round, the sequential chain).
#define GLP_GEN_TABLE(NAME, FNTYPE, KERNEL, EMIT, SUB) \
  FNTYPE NAME(uint32_t P) {                            \
    switch (P) {                                       \
      case 0:                                          \
      case 1:                                          \
      case 2: return KERNEL<2, EMIT, SUB>;             \
      case 4: return KERNEL<4, EMIT, SUB>;             \
      case 8: return KERNEL<8, EMIT, SUB>;             \
      case 16: return KERNEL<16, EMIT, SUB>;           \
      default: return KERNEL<32, EMIT, SUB>;           \
    }                                                  \
  }
