// GL vector quantisation on the device: Lloyd training of the (homRef, het)
// codebook (GLVQ::BuildCodeBook / AssignPoints / UpdateCodeBook,
// src/glVQ.cpp:26-146) and the packing of codes into words
// (GLPack::GetPackedGLs, src/glPack.cpp:112-165).
//
// Points are the normalised pairs rr = g0 / s, het = g1 / s with
// s = (g0 + g1) + g2 (binary32) of the GL triples [N][S][3].  A point's code
// is the entry with the smallest distance, computed as GLVQHelper::
// EuclidianDist does (glVQ.hpp:23-30): the differences in binary32, squared
// and summed in binary64, then the square root; the first such entry wins.
//
// One training iteration = one vq_assign_kernel launch (assign every point
// and accumulate, per entry, the sums of rr and het, the count, and the
// total squared distance) + one vq_update_kernel launch (new entries).  Sums
// are binary64 in a fixed order, so they do not depend on scheduling: run r
// of block b holds points b*B + r + 256*j, j = 0..63 (B = 16,384), summed in
// j order; a block adds its 256 runs in r order; the update adds the blocks
// in b order.  (The reference sums in binary32 in point order; the host
// restatement in glphase_gb300/glpack.py uses this order.)
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace glp {

constexpr int kVQMaxCodes = 16;
constexpr int kVQRun = 64;                          // points per thread
constexpr int kVQThreads = 256;                     // runs per block
constexpr uint32_t kVQBlock = kVQRun * kVQThreads;  // points per block

__device__ __forceinline__ void vq_point(const float *__restrict__ gl, uint64_t p, float &rr,
                                         float &het) {
  const float g0 = gl[3 * p], g1 = gl[3 * p + 1], g2 = gl[3 * p + 2];
  const float s = __fadd_rn(__fadd_rn(g0, g1), g2);
  rr = __fdiv_rn(g0, s);
  het = __fdiv_rn(g1, s);
}

// Squared distance of EuclidianDist before the square root.
__device__ __forceinline__ double vq_d2(float cr, float ch, float rr, float het) {
  const double dx = (double)__fsub_rn(cr, rr), dy = (double)__fsub_rn(ch, het);
  return __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
}

// Index of the first entry with the smallest sqrt(distance).  The square
// root is monotonic, so the first smallest squared distance is the answer
// unless an earlier entry's squared distance rounds to the same square root;
// those (within a few ulps) are checked with the root itself.
__device__ __forceinline__ uint32_t vq_nearest(const float2 *cb, uint32_t K, float rr,
                                               float het) {
  double best = vq_d2(cb[0].x, cb[0].y, rr, het);
  uint32_t kb = 0;
  for (uint32_t k = 1; k < K; ++k) {
    const double d = vq_d2(cb[k].x, cb[k].y, rr, het);
    if (d < best) {
      best = d;
      kb = k;
    }
  }
  if (kb > 0) {
    const double rb = __dsqrt_rn(best);
    const double near = best * (1.0 + 0x1p-48);
    for (uint32_t k = 0; k < kb; ++k) {
      const double d = vq_d2(cb[k].x, cb[k].y, rr, het);
      if (d <= near && __dsqrt_rn(d) == rb)
        return k;
    }
  }
  return kb;
}

// Per block: sums[b][0..K) rr, [K..2K) het, [2K] squared distance (binary64),
// counts[b][0..K).  Dynamic shared memory: kVQThreads * (2K + 1) doubles +
// kVQThreads * K uint32.
__global__ void __launch_bounds__(kVQThreads)
    vq_assign_kernel(const float *__restrict__ gl, uint64_t P, const float2 *__restrict__ codebook,
                     uint32_t K, double *__restrict__ sums, uint32_t *__restrict__ counts) {
  extern __shared__ __align__(16) unsigned char vq_smem[];
  double *acc = reinterpret_cast<double *>(vq_smem);                       // [2K+1][256]
  uint32_t *cnt = reinterpret_cast<uint32_t *>(acc + (2 * K + 1) * kVQThreads);  // [K][256]
  __shared__ float2 cb[kVQMaxCodes];
  const uint32_t t = threadIdx.x;
  if (t < K)
    cb[t] = codebook[t];
  for (uint32_t i = 0; i < 2 * K + 1; ++i)
    acc[i * kVQThreads + t] = 0.0;
  for (uint32_t k = 0; k < K; ++k)
    cnt[k * kVQThreads + t] = 0;
  __syncthreads();
  const uint64_t base = (uint64_t)blockIdx.x * kVQBlock + t;
  double var = 0.0;
  for (uint32_t j = 0; j < (uint32_t)kVQRun; ++j) {
    const uint64_t p = base + (uint64_t)j * kVQThreads;
    if (p >= P)
      break;
    float rr, het;
    vq_point(gl, p, rr, het);
    const uint32_t k = vq_nearest(cb, K, rr, het);
    double *a = acc + k * kVQThreads + t;
    *a = __dadd_rn(*a, (double)rr);
    a += K * kVQThreads;
    *a = __dadd_rn(*a, (double)het);
    cnt[k * kVQThreads + t] += 1;
    // AssignPoints' term: the differences point - entry in binary32, squared
    // and summed in binary64
    const double dx = (double)__fsub_rn(rr, cb[k].x), dy = (double)__fsub_rn(het, cb[k].y);
    var = __dadd_rn(var, __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
  }
  acc[2 * K * kVQThreads + t] = var;
  __syncthreads();
  // runs in r order: one thread per sum
  if (t < 2 * K + 1) {
    double s = 0.0;
    const double *row = acc + t * kVQThreads;
    for (uint32_t r = 0; r < (uint32_t)kVQThreads; ++r)
      s = __dadd_rn(s, row[r]);
    sums[(uint64_t)blockIdx.x * (2 * K + 1) + t] = s;
  }
  if (t < K) {
    uint32_t c = 0;
    const uint32_t *row = cnt + t * kVQThreads;
    for (uint32_t r = 0; r < (uint32_t)kVQThreads; ++r)
      c += row[r];
    counts[(uint64_t)blockIdx.x * K + t] = c;
  }
}

// SplitMix64 (Steele, Lea, Flood 2014): the point an entry with no points
// moves to, for training iteration `it` (UpdateCodeBook draws a random point
// there, glVQ.cpp:127-133).
__host__ __device__ inline uint64_t vq_splitmix64(uint64_t x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}
// Shared memory of vq_assign_kernel for K entries.
__host__ __device__ constexpr size_t vq_assign_smem(uint32_t K) {
  return (size_t)kVQThreads * ((2 * K + 1) * sizeof(double) + K * sizeof(uint32_t));
}

__host__ __device__ inline uint64_t vq_empty_point(uint64_t seed, uint32_t it, uint32_t k,
                                                   uint64_t P) {
  return vq_splitmix64(seed ^ (((uint64_t)it << 16) | k)) % P;
}

// New entries from the block sums (blocks in b order): mean of the points
// of an entry rounded to binary32, or an empty entry moved onto a point.
// out_var = the total squared distance of the assignment the sums came from.
// One block of 64 threads.
__global__ void vq_update_kernel(const float *__restrict__ gl, uint64_t P, uint32_t nblocks,
                                 const double *__restrict__ sums,
                                 const uint32_t *__restrict__ counts, uint32_t K, uint64_t seed,
                                 uint32_t it, float2 *__restrict__ codebook,
                                 double *__restrict__ out_var) {
  __shared__ double tot[2 * kVQMaxCodes + 1];
  __shared__ unsigned long long num[kVQMaxCodes];
  const uint32_t t = threadIdx.x;
  if (t < 2 * K + 1) {
    double s = 0.0;
    for (uint32_t b = 0; b < nblocks; ++b)
      s = __dadd_rn(s, sums[(uint64_t)b * (2 * K + 1) + t]);
    tot[t] = s;
  }
  if (t < K) {
    unsigned long long c = 0;
    for (uint32_t b = 0; b < nblocks; ++b)
      c += counts[(uint64_t)b * K + t];
    num[t] = c;
  }
  __syncthreads();
  if (t == 0)
    *out_var = tot[2 * K];
  if (codebook && t < K) {
    float2 e;
    if (num[t] > 0) {
      e.x = (float)__ddiv_rn(tot[t], (double)num[t]);
      e.y = (float)__ddiv_rn(tot[K + t], (double)num[t]);
    } else {
      vq_point(gl, vq_empty_point(seed, it, t, P), e.x, e.y);
    }
    codebook[t] = e;
  }
}

// Codes of sites w*per .. w*per+per-1 of sample n packed into one word,
// first site in the most significant bits; sites past S use the array's
// first GL (glPack.cpp:147-149).  packed is [ceil(S/per)][N].
struct VQBook {
  float2 e[kVQMaxCodes];
};

__global__ void vq_pack_kernel(const float *__restrict__ gl, uint32_t N, uint32_t S,
                               const VQBook book, uint32_t K, uint32_t bits,
                               uint32_t *__restrict__ packed) {
  __shared__ float2 cb[kVQMaxCodes];
  if (threadIdx.x < K)
    cb[threadIdx.x] = book.e[threadIdx.x];
  __syncthreads();
  const uint32_t per = 32u / bits;
  const uint32_t nw = (S + per - 1) / per;
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint64_t)nw * N)
    return;
  const uint32_t w = (uint32_t)(i / N), n = (uint32_t)(i % N);
  uint32_t word = 0;
  for (uint32_t k = 0; k < per; ++k) {
    const uint32_t m = w * per + k;
    const uint64_t p = m < S ? (uint64_t)n * S + m : 0;
    float rr, het;
    vq_point(gl, p, rr, het);
    word |= vq_nearest(cb, K, rr, het) << (32u - bits * (k + 1));
  }
  packed[(uint64_t)w * N + n] = word;
}

}  // namespace glp
