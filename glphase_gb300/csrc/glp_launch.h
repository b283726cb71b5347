// Kernel tables of the generation kernels.
//
// Each (entry kind, emission source) pair is instantiated in its own
// translation unit (glp_gen_*.cu) so the instantiations compile in parallel;
// the host code picks a kernel by speculation shape: P lanes per sample and V
// evaluations per lane (V = 2 exists for P = 2, 4, 8).
#pragma once

#include "glp_kernels.cuh"

namespace glp {

using SingleFn = void (*)(const GenParams);
using MultiFn = void (*)(const MultiParams);

SingleFn single_kernel_f32(uint32_t P, uint32_t V);
SingleFn single_kernel_vq(uint32_t P, uint32_t V);
MultiFn multi_kernel_f32(uint32_t P, uint32_t V);
MultiFn multi_kernel_vq(uint32_t P, uint32_t V);
// the same with normalisation every 4 sites (one evaluation per lane)
SingleFn single_kernel_f32_sub4(uint32_t P);
SingleFn single_kernel_vq_sub4(uint32_t P);
MultiFn multi_kernel_f32_sub4(uint32_t P);
MultiFn multi_kernel_vq_sub4(uint32_t P);

}  // namespace glp

// Body of one table: KERNEL<P, V, EMIT> for every supported shape.
#define GLP_GEN_TABLE(NAME, FNTYPE, KERNEL, EMIT)   \
  FNTYPE NAME(uint32_t P, uint32_t V) {             \
    if (V == 2) {                                   \
      switch (P) {                                  \
        case 2: return KERNEL<2, 2, EMIT>;          \
        case 4: return KERNEL<4, 2, EMIT>;          \
        default: return KERNEL<8, 2, EMIT>;         \
      }                                             \
    }                                               \
    switch (P) {                                    \
      case 1: return KERNEL<1, 1, EMIT>;            \
      case 2: return KERNEL<2, 1, EMIT>;            \
      case 4: return KERNEL<4, 1, EMIT>;            \
      case 8: return KERNEL<8, 1, EMIT>;            \
      case 16: return KERNEL<16, 1, EMIT>;          \
      default: return KERNEL<32, 1, EMIT>;          \
    }                                               \
  }

// Body of a table of the every-4-sites kernels: KERNEL<P, 1, EMIT, 2>.
#define GLP_GEN_TABLE_SUB4(NAME, FNTYPE, KERNEL, EMIT) \
  FNTYPE NAME(uint32_t P) {                           \
    switch (P) {                                      \
      case 1: return KERNEL<1, 1, EMIT, 2>;           \
      case 2: return KERNEL<2, 1, EMIT, 2>;           \
      case 4: return KERNEL<4, 1, EMIT, 2>;           \
      case 8: return KERNEL<8, 1, EMIT, 2>;           \
      case 16: return KERNEL<16, 1, EMIT, 2>;         \
      default: return KERNEL<32, 1, EMIT, 2>;         \
    }                                                 \
  }
