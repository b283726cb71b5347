// glp_tally.cuh -- per-site allele tallies of the sampling generations on the
// device: Impute::replace (src/impute.cpp:564-595) and Impute::result
// (src/impute.cpp:599-613).
//
// replace: for sample I with current haplotypes oa, ob and running tallies
// ha, hb ([2N][S] uint32), count sis = sum over alt sites of oa of ha plus
// alt sites of ob of hb, and tra the crossed sum; then add oa to ha and ob to
// hb when sis > tra, else crossed.  Integer arithmetic: bit-exact.
// One CTA per sample; the two sums are block reductions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace glp {

constexpr int kTallyThreads = 128;

__global__ void __launch_bounds__(kTallyThreads)
    replace_kernel(const uint64_t *__restrict__ haps, uint32_t N, uint32_t S, uint32_t wn,
                   uint32_t *__restrict__ hsum) {
  const uint32_t I = blockIdx.x;
  if (I >= N)
    return;
  const uint64_t *oa = haps + (size_t)2 * I * wn, *ob = oa + wn;
  uint32_t *ha = hsum + (size_t)2 * I * S, *hb = ha + S;
  unsigned long long sis = 0, tra = 0;
  for (uint32_t m = threadIdx.x; m < S; m += kTallyThreads) {
    const uint32_t a = (uint32_t)((__ldg(oa + (m >> 6)) >> (m & 63u)) & 1u);
    const uint32_t b = (uint32_t)((__ldg(ob + (m >> 6)) >> (m & 63u)) & 1u);
    const uint32_t x = ha[m], y = hb[m];
    sis += (unsigned long long)(a * x + b * y);
    tra += (unsigned long long)(a * y + b * x);
  }
  __shared__ unsigned long long r_s[kTallyThreads / 32], r_t[kTallyThreads / 32];
  for (int o = 16; o; o >>= 1) {
    sis += __shfl_xor_sync(0xffffffffu, sis, o);
    tra += __shfl_xor_sync(0xffffffffu, tra, o);
  }
  if ((threadIdx.x & 31u) == 0) {
    r_s[threadIdx.x >> 5] = sis;
    r_t[threadIdx.x >> 5] = tra;
  }
  __syncthreads();
  unsigned long long S_sum = 0, T_sum = 0;
  for (int i = 0; i < kTallyThreads / 32; ++i) {
    S_sum += r_s[i];
    T_sum += r_t[i];
  }
  // the reference sums in 32-bit unsigned arithmetic (impute.cpp:575-584)
  const bool keep = (uint32_t)S_sum > (uint32_t)T_sum;
  for (uint32_t m = threadIdx.x; m < S; m += kTallyThreads) {
    const uint32_t a = (uint32_t)((__ldg(oa + (m >> 6)) >> (m & 63u)) & 1u);
    const uint32_t b = (uint32_t)((__ldg(ob + (m >> 6)) >> (m & 63u)) & 1u);
    ha[m] += keep ? a : b;
    hb[m] += keep ? b : a;
  }
}

// result: prob_out[m][2i + h] = hsum[(2i + h)][m] * (float)(1 / sn)
// (impute.cpp:599-613), binary32.
__global__ void result_kernel(const uint32_t *__restrict__ hsum, uint32_t N, uint32_t S,
                              float norm, float *__restrict__ prob_out) {
  const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t total = (uint64_t)2 * N * S;
  if (idx >= total)
    return;
  const uint32_t m = (uint32_t)(idx / (2 * N)), h = (uint32_t)(idx % (2 * N));
  prob_out[idx] = (float)hsum[(size_t)h * S + m] * norm;
}

}  // namespace glp
