// glp_knn.cuh -- kNN surrogate restriction on the device: the reference's
// KNN::ClusterHaps (src/kNN.cpp:123-206) with the Hamming metric
// (src/haplotype.cpp:35-60) or the tract-length metric (insti -T: the number
// of common sites minus Haplotype::MaxTractLen, src/haplotype.cpp:62-90,
// kNN.cpp:157-164) over the common sites of KNN::CutDownHaps
// (src/kNN.cpp:216-257).
//
// For each sample s of the H/2 samples: the ceil(K/2) haplotypes nearest to
// haplotype 2s, then the ceil(K/2) nearest to haplotype 2s+1 that are not
// already chosen, interleaved.  The sample's own haplotypes are excluded.
// Ties are ordered by haplotype index, a total order; the reference sorts
// with the unstable std::sort (kNN.cpp:172-173), so its tie order is
// implementation-defined.
//
// Distances as tiled products of bit matrices, a chunk of samples at a time
// through global memory: Hamming (knn_dist_kernel), or the tract length
// (knn_tract_dist_kernel: each word's runs of agreeing common sites --
// before its first disagreement, after its last, the longest between --
// joined in site order, glp_tract.h).  Selection (knn_select_kernel): one
// CTA per sample with the distances of both its haplotypes to all H
// haplotypes in shared memory as uint16 (H <= kKnnMaxHaps); the ceil(K/2)
// nearest are found by binary search on the distance threshold, ties at the
// threshold are taken in index order through a block scan, and the chosen
// list is put in (distance, index) order by a bitonic sort.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "glp_tract.h"

namespace glp {

constexpr int kKnnThreads = 256;
constexpr uint32_t kKnnMaxHaps = 50000;
constexpr uint32_t kKnnMaxHalf = 1024;
constexpr uint16_t kKnnExcluded = 0xffffu;

// Bit m of mask: site m's alt-allele frequency (or MAF) lies in [lb, ub].
__global__ void common_sites_kernel(const uint64_t *__restrict__ haps, uint32_t H,
                                    uint32_t wn, uint32_t S, double lb, double ub,
                                    int use_maf, uint64_t *__restrict__ mask) {
  const uint32_t w = blockIdx.x;
  const uint32_t lane = threadIdx.x;  // 64 threads: one site each
  const uint32_t m = w * 64 + lane;
  uint32_t alt = 0;
  if (m < S)
    for (uint32_t h = 0; h < H; ++h)
      alt += (uint32_t)((__ldg(haps + (size_t)h * wn + w) >> lane) & 1u);
  double af = (double)alt / H;
  if (use_maf)
    af = fabs(fabs(af - 0.5) - 0.5);
  const bool keep = m < S && af >= lb && af <= ub;
  const unsigned lo = __ballot_sync(0xffffffffu, lane < 32 ? keep : false);
  __shared__ unsigned hi_bits;
  if (lane == 32)
    hi_bits = 0;
  __syncthreads();
  const unsigned hb = __ballot_sync(0xffffffffu, keep);
  if (lane == 32)
    hi_bits = hb;
  __syncthreads();
  if (lane == 0)
    mask[w] = (uint64_t)lo | ((uint64_t)hi_bits << 32);
}

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t *red) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o; o >>= 1)
    v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0)
    red[warp] = v;
  __syncthreads();
  uint32_t t = 0;
#pragma unroll
  for (int i = 0; i < kKnnThreads / 32; ++i)
    t += red[i];
  return t;
}

// Exclusive prefix over threads (thread order), block total in *total.
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t *red,
                                                    uint32_t *total) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t n = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= (uint32_t)o)
      inc += n;
  }
  __syncthreads();
  if (lane == 31)
    red[warp] = inc;
  __syncthreads();
  uint32_t base = 0, all = 0;
#pragma unroll
  for (int i = 0; i < kKnnThreads / 32; ++i) {
    if ((uint32_t)i < warp)
      base += red[i];
    all += red[i];
  }
  *total = all;
  return base + inc - v;
}

// Choose the `half` smallest (d, index) among entries of d that are not
// kKnnExcluded, write them sorted to out[0..half).
__device__ void select_nearest(const uint16_t *d, uint32_t H, uint32_t half, uint32_t dmax,
                               uint32_t *keys, uint32_t *red, uint32_t *out) {
  const uint32_t tid = threadIdx.x;
  // smallest t with #{d <= t} >= half
  uint32_t lo = 0, hi = dmax;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    uint32_t c = 0;
    for (uint32_t h = tid; h < H; h += kKnnThreads)
      c += (d[h] != kKnnExcluded && d[h] <= mid) ? 1u : 0u;
    if (block_sum(c, red) >= half)
      hi = mid;
    else
      lo = mid + 1;
  }
  const uint32_t t = lo;
  uint32_t below = 0;
  for (uint32_t h = tid; h < H; h += kKnnThreads)
    below += (d[h] != kKnnExcluded && d[h] < t) ? 1u : 0u;
  below = block_sum(below, red);
  const uint32_t need = half - below;  // ties at t, taken in index order
  const uint32_t chunk = (H + kKnnThreads - 1) / kKnnThreads;
  const uint32_t b0 = min(H, tid * chunk), b1 = min(H, b0 + chunk);
  uint32_t ties = 0;
  for (uint32_t h = b0; h < b1; ++h)
    ties += (d[h] == t) ? 1u : 0u;
  uint32_t total;
  uint32_t rank = block_exclusive(ties, red, &total);
  uint32_t nless = 0;
  for (uint32_t h = b0; h < b1; ++h)
    nless += (d[h] != kKnnExcluded && d[h] < t) ? 1u : 0u;
  uint32_t pos = block_exclusive(nless, red, &total);
  // entries below the threshold first (positions [0, below)), then ties
  for (uint32_t h = b0; h < b1; ++h) {
    const uint16_t v = d[h];
    if (v == kKnnExcluded)
      continue;
    if (v < t) {
      keys[pos++] = ((uint32_t)v << 16) | 0u;
      keys[kKnnMaxHalf + pos - 1] = h;
    } else if (v == t) {
      if (rank < need) {
        keys[below + rank] = ((uint32_t)v << 16);
        keys[kKnnMaxHalf + below + rank] = h;
      }
      ++rank;
    }
  }
  __syncthreads();
  // bitonic sort of (distance, index) over the next power of two
  uint32_t n2 = 1;
  while (n2 < half)
    n2 <<= 1;
  for (uint32_t i = tid; i < n2; i += kKnnThreads)
    if (i >= half) {
      keys[i] = 0xffffffffu;
      keys[kKnnMaxHalf + i] = 0xffffffffu;
    }
  __syncthreads();
  for (uint32_t k = 2; k <= n2; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = tid; i < n2; i += kKnnThreads) {
        const uint32_t l = i ^ j;
        if (l > i) {
          const uint64_t a = ((uint64_t)keys[i] << 32) | keys[kKnnMaxHalf + i];
          const uint64_t b = ((uint64_t)keys[l] << 32) | keys[kKnnMaxHalf + l];
          const bool up = (i & k) == 0;
          if ((a > b) == up) {
            keys[i] = (uint32_t)(b >> 32);
            keys[kKnnMaxHalf + i] = (uint32_t)b;
            keys[l] = (uint32_t)(a >> 32);
            keys[kKnnMaxHalf + l] = (uint32_t)a;
          }
        }
      }
      __syncthreads();
    }
  }
  for (uint32_t i = tid; i < half; i += kKnnThreads)
    out[i] = keys[kKnnMaxHalf + i];
  __syncthreads();
}

// The sample's neighbour list from the distances dA, dB of its two
// haplotypes (shared memory; its own two excluded): the `half` nearest to
// the first, then the `half` nearest to the second among those not taken,
// interleaved into out (KNN::ClusterHaps, kNN.cpp:170-206).
__device__ __forceinline__ void knn_choose(uint16_t *dA, uint16_t *dB, uint32_t H,
                                           uint32_t half, uint32_t dmax, uint32_t *keys,
                                           uint32_t *red, uint32_t *chosen, uint32_t *taken,
                                           uint32_t *out) {
  const uint32_t tid = threadIdx.x;
  select_nearest(dA, H, half, dmax, keys, red, chosen);
  for (uint32_t i = tid; i < half; i += kKnnThreads) {
    const uint32_t h = chosen[i];
    atomicOr(&taken[h >> 5], 1u << (h & 31u));
  }
  __syncthreads();
  for (uint32_t h = tid; h < H; h += kKnnThreads)
    if ((taken[h >> 5] >> (h & 31u)) & 1u)
      dB[h] = kKnnExcluded;
  __syncthreads();
  select_nearest(dB, H, half, dmax, keys, red, chosen + kKnnMaxHalf);
  for (uint32_t i = tid; i < half; i += kKnnThreads) {
    out[2 * i] = chosen[i];
    out[2 * i + 1] = chosen[kKnnMaxHalf + i];
  }
}

// Tiled Hamming distances for the kNN build, as a product of bit matrices:
// dist[q][h] = popcount((hap q0+q XOR hap h) AND mask) over the words, for
// the query haplotypes [q0, q0 + nq) (2 s and 2 s + 1 for the samples s of a
// chunk) and every haplotype h; a sample's own two are marked excluded.  A
// CTA takes 64 queries x 128 haplotypes and walks the words 8 at a time,
// staged word-major in shared memory (a warp's reads of a word are
// consecutive); each thread keeps 4 x 8 sums.  Each panel word is read from
// L2 once per 64 queries instead of once per sample.
constexpr uint32_t kDistQ = 64, kDistH = 128, kDistW = 8, kDistThreads = 256;
__global__ void __launch_bounds__(kDistThreads)
    knn_dist_kernel(const uint64_t *__restrict__ haps, uint32_t H, uint32_t wn,
                    const uint64_t *__restrict__ mask, uint32_t q0, uint32_t nq,
                    uint16_t *__restrict__ dist) {
  __shared__ uint64_t sq[kDistW][kDistQ];
  __shared__ uint64_t sh[kDistW][kDistH];
  __shared__ uint64_t smask[kDistW];
  const uint32_t tid = threadIdx.x, tx = tid & 15u, ty = tid >> 4;
  const uint32_t hb = blockIdx.x * kDistH, qb = blockIdx.y * kDistQ;
  uint32_t acc[4][8];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j)
      acc[i][j] = 0;
  for (uint32_t w0 = 0; w0 < wn; w0 += kDistW) {
    for (uint32_t i = tid; i < kDistQ * kDistW; i += kDistThreads) {
      const uint32_t r = i / kDistW, k = i % kDistW, w = w0 + k;
      sq[k][r] = (qb + r < nq && w < wn) ? __ldg(haps + (size_t)(q0 + qb + r) * wn + w) : 0ull;
    }
    for (uint32_t i = tid; i < kDistH * kDistW; i += kDistThreads) {
      const uint32_t r = i / kDistW, k = i % kDistW, w = w0 + k;
      sh[k][r] = (hb + r < H && w < wn) ? __ldg(haps + (size_t)(hb + r) * wn + w) : 0ull;
    }
    if (tid < kDistW)
      smask[tid] = w0 + tid < wn ? __ldg(mask + w0 + tid) : 0ull;
    __syncthreads();
#pragma unroll
    for (uint32_t k = 0; k < kDistW; ++k) {
      const uint64_t mk = smask[k];
      uint64_t qv[4], hv[8];
#pragma unroll
      for (int i = 0; i < 4; ++i)
        qv[i] = sq[k][4 * ty + i] & mk;
#pragma unroll
      for (int j = 0; j < 8; ++j)
        hv[j] = sh[k][tx + 16 * j] & mk;
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j)
          acc[i][j] += __popcll(qv[i] ^ hv[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const uint32_t q = qb + 4 * ty + i;
    if (q >= nq)
      continue;
    const uint32_t s = (q0 + q) >> 1;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint32_t h = hb + tx + 16 * j;
      if (h < H)
        dist[(size_t)q * H + h] = (h >> 1) == s ? kKnnExcluded : (uint16_t)acc[i][j];
    }
  }
}

// Tiled tract-length distances (-T), laid out as knn_dist_kernel's: each
// pair carries the runs of agreeing common sites of the words so far --
// before the first disagreement, after the last, the longest -- and joins
// every next word's (tract_word) to them in site order; the distance is the
// common sites minus the longest run.  A CTA takes 32 queries x 64
// haplotypes, each thread 2 x 4 pairs.
constexpr uint32_t kTractQ = 32, kTractH = 64;
__global__ void __launch_bounds__(kDistThreads)
    knn_tract_dist_kernel(const uint64_t *__restrict__ haps, uint32_t H, uint32_t wn,
                          const uint64_t *__restrict__ mask, uint32_t q0, uint32_t nq,
                          uint16_t *__restrict__ dist) {
  __shared__ uint64_t sq[kDistW][kTractQ];
  __shared__ uint64_t sh[kDistW][kTractH];
  __shared__ uint64_t smask[kDistW];
  const uint32_t tid = threadIdx.x, tx = tid & 15u, ty = tid >> 4;
  const uint32_t hb = blockIdx.x * kTractH, qb = blockIdx.y * kTractQ;
  Tract run[2][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
      run[i][j] = Tract{0, 0, 0, 0};
  for (uint32_t w0 = 0; w0 < wn; w0 += kDistW) {
    for (uint32_t i = tid; i < kTractQ * kDistW; i += kDistThreads) {
      const uint32_t r = i / kDistW, k = i % kDistW, w = w0 + k;
      sq[k][r] = (qb + r < nq && w < wn) ? __ldg(haps + (size_t)(q0 + qb + r) * wn + w) : 0ull;
    }
    for (uint32_t i = tid; i < kTractH * kDistW; i += kDistThreads) {
      const uint32_t r = i / kDistW, k = i % kDistW, w = w0 + k;
      sh[k][r] = (hb + r < H && w < wn) ? __ldg(haps + (size_t)(hb + r) * wn + w) : 0ull;
    }
    if (tid < kDistW)
      smask[tid] = w0 + tid < wn ? __ldg(mask + w0 + tid) : 0ull;
    __syncthreads();
    const uint32_t kn = min(kDistW, wn - w0);
    for (uint32_t k = 0; k < kn; ++k) {
      const uint64_t m = smask[k];
      uint64_t qv[2], hv[4];
#pragma unroll
      for (int i = 0; i < 2; ++i)
        qv[i] = sq[k][2 * ty + i];
#pragma unroll
      for (int j = 0; j < 4; ++j)
        hv[j] = sh[k][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
          run[i][j] = tract_join(run[i][j], tract_word((qv[i] ^ hv[j]) & m, m));
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const uint32_t q = qb + 2 * ty + i;
    if (q >= nq)
      continue;
    const uint32_t s = (q0 + q) >> 1;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t h = hb + tx + 16 * j;
      if (h < H)
        dist[(size_t)q * H + h] =
            (h >> 1) == s ? kKnnExcluded : (uint16_t)(run[i][j].len - run[i][j].best);
    }
  }
}

// The neighbour lists of the samples s0 + blockIdx.x from their rows of
// knn_dist_kernel's distances (rows 2 i and 2 i + 1 for the chunk's i-th
// sample).  Dynamic shared memory (knn_smem_bytes): dA, dB [H] uint16, keys
// [2*kKnnMaxHalf] uint32, chosen [2*kKnnMaxHalf] uint32, taken bits
// [ceil(H/32)] uint32.
__global__ void __launch_bounds__(kKnnThreads)
    knn_select_kernel(const uint16_t *__restrict__ dist, uint32_t H, uint32_t s0, uint32_t half,
                      uint32_t dmax, uint32_t *__restrict__ neighbors) {
  extern __shared__ uint4 knn_smem[];
  uint16_t *dA = reinterpret_cast<uint16_t *>(knn_smem);
  uint16_t *dB = dA + H;
  uint32_t *keys = reinterpret_cast<uint32_t *>(dA + 2 * ((H + 1) & ~1u));
  uint32_t *chosen = keys + 2 * kKnnMaxHalf;
  uint32_t *taken = chosen + 2 * kKnnMaxHalf;
  __shared__ uint32_t red[kKnnThreads / 32];
  const uint32_t tid = threadIdx.x;
  // the two rows, 2 H uint16 in a row of the distances (H even: 4-byte units)
  const uint32_t *row = reinterpret_cast<const uint32_t *>(dist + (size_t)2 * blockIdx.x * H);
  uint32_t *d32 = reinterpret_cast<uint32_t *>(dA);
  for (uint32_t i = tid; i < H; i += kKnnThreads)
    d32[i] = __ldg(row + i);
  for (uint32_t i = tid; i < (H + 31) / 32; i += kKnnThreads)
    taken[i] = 0;
  __syncthreads();
  knn_choose(dA, dB, H, half, dmax, keys, red, chosen, taken,
             neighbors + (size_t)(s0 + blockIdx.x) * 2 * half);
}

inline size_t knn_smem_bytes(uint32_t H) {
  return sizeof(uint16_t) * 2 * ((H + 1) & ~1u) + sizeof(uint32_t) * 4 * kKnnMaxHalf +
         sizeof(uint32_t) * ((H + 31) / 32);
}

}  // namespace glp
