// glp_kernels.cuh -- sm_103a kernels for one MH generation of GLPhase's
// haplotype sampler: per-sample Metropolis-Hastings over surrogate-parent
// quadruples scored by the 4-state HMM forward likelihood, with the final
// haplotype sampling (hmm_work) fused into the same launch.
//
// Reference semantics (paths relative to the reference project root):
//   likelihood  Impute::hmm_like      src/impute.cpp:327-376 (CPU, float emit)
//               HMMLikeCUDA::hmmLike  src/hmmLike.cu:53-142  (GPU, VQ GLs)
//   MH chain    findHapSet            src/hmmLike.cu:145-217
//               Insti::solve          src/insti.cpp:1478-1551
//               MHSampler::SampleHap  src/MHSampler.hpp:81-96
//   sampling    Impute::hmm_work      src/impute.cpp:380-485
//
// Work decomposition (one warp = 32/P groups of P lanes, one sample per group):
//  * A sample's MH chain is inherently sequential, so its parallelism comes
//    from speculation: the P/2 lane pairs of a group evaluate the next P/2
//    evaluations of the chain (the current quadruple and the next proposals),
//    each built on the current state, i.e. assuming all earlier ones are
//    rejected.  The group then replays the accept rule in order; evaluations
//    after the first accepted proposal are discarded and re-evaluated from the
//    new state.  Decisions are exactly those of the sequential chain.
//  * A pair computes one likelihood: its even lane a forward pass over the
//    lower half of the sites, its odd lane a backward pass over the upper
//    half, both in one code path (x <- D T x), joined by a 4-term dot product
//    L = alpha_h . beta_h.  Half the sites per lane means half as many
//    speculative positions per round for the same lanes per sample, so fewer
//    of them are discarded.
//  * Scaling is by exact powers of two with an integer exponent per half;
//    the log-likelihood is assembled in binary64 (log(dot) + k*ln2).
//  * hmm_work runs one sample per thread in a second kernel over the final
//    quadruples, in the reference's exact binary32 operation order (no
//    contraction), so its output bits match the CPU reference.
//
// Memory (all resident in HBM across generations):
//   haps/hnew  uint64 [H][wn] hap-major   (parent words: L2-resident gathers)
//   emit       float4 [N][S]              (streamed, shared by a group)
//   packed     uint32 [ceil(S/8)][N]      (VQ codes; 16-entry table in smem)
//   tran4      float4 [S + 1]             (t0, t1, t2, t0 - t2); rows 0 and S = identity
//   tranp      float4 [S + 1]             (t1, t2, t0 - t2, t0 - t2), the pair rows the
//                                         blocked recursion stages (follows tran4)
//   beta       float4 [N][S]              (hmm_work scratch)
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "glp_rng.h"

namespace glp {

#ifndef GLP_GEN_WARPS
#define GLP_GEN_WARPS 4
#endif
constexpr int kWarps = GLP_GEN_WARPS;  // warps per generation block
constexpr int kThreads = 32 * kWarps;
// Resident blocks per SM the generation kernels are compiled for (the
// launch bound's minimum): with 3 the compiler may use up to 168 registers
// a thread and schedules the loop in 119-127, so 4 blocks (16 warps) still
// fit; measured 1.2 % faster than the bound of 4 (a cap of 128) on 10,000
// samples x 4,096 sites.  5 (a cap of 96) was 16 % slower.
#ifndef GLP_MIN_BLOCKS
#define GLP_MIN_BLOCKS 3
#endif
constexpr int kMinBlocks = GLP_MIN_BLOCKS;
constexpr uint32_t kNone = 0xffffffffu;
// Generation counters (GenParams::stats): scored evaluations, speculative
// rounds, accepted proposals, evaluations redone site by site after a block
// left the normalisation range, warp rounds, and active lanes summed over
// warp rounds.
constexpr int kStats = 6;
constexpr float kTiny = 0x1p-64f;
constexpr float kHuge = 0x1p64f;

struct GenParams {
  uint32_t N, S, C, H, wn, emit_mode;
  const uint64_t *__restrict__ haps;
  uint64_t *__restrict__ hnew;
  const float4 *__restrict__ emit;
  const float *__restrict__ prob;
  const float4 *__restrict__ tran4;
  const float4 *__restrict__ tranp;  // tran4's rows as (t1, t2, t0 - t2, t0 - t2)
  const uint32_t *__restrict__ packed;
  const float4 *__restrict__ vq_table;
  const uint32_t *__restrict__ quad_in;
  uint32_t *__restrict__ quad_out;
  const uint32_t *__restrict__ props;
  const uint8_t *__restrict__ tr_slot;
  const double *__restrict__ tr_u;
  const float *__restrict__ tr_work;
  double *__restrict__ like_out;
  double *__restrict__ eval_trace;
  uint8_t *__restrict__ accept_trace;
  float4 *__restrict__ beta;
  uint32_t *__restrict__ counter;
  unsigned long long *__restrict__ stats;
  int *__restrict__ error;
  const uint32_t *__restrict__ nbr;  // [N][klen] surrogate table, or null
  uint32_t klen, samp_lo, samp_hi;   // uniform surrogates over [samp_lo, samp_hi)
  uint32_t burnin;                   // >0: advance_kernel sets pen = min((g+1)/burnin,1)^2
  uint32_t kick;                     // 1: surrogates from [samp_lo, H) in generation 0 only
  uint32_t kick_first;               // 1: every chain's first proposal from the panel rows
  float pc[16];
  float pen;
  uint64_t seed;
  uint32_t generation;
  uint32_t do_work;
};

// ---------------------------------------------------------------------------
// Emission sources.  Both hand out the 4 emission values of a site,
// e[(father_bit << 1) | mother_bit] (impute.cpp:338-342).

// L1 prefetch of the line holding `ptr` (no register is held; the later
// load of the same line then hits L1).
__device__ __forceinline__ void prefetch_l1(const void *ptr) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(ptr));
}

// Bulk prefetch of [ptr, ptr + bytes) into L2 (a hint: nothing is written);
// ptr and bytes must be multiples of 16 and the range inside one allocation.
__device__ __forceinline__ void prefetch_l2_bulk(const void *ptr, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(ptr), "r"(bytes) : "memory");
}

// Asynchronous global -> shared copies (cp.async): the data lands in shared
// memory without occupying registers; cp_async_wait<n> returns once at most n
// of this thread's committed copy groups are still in flight.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int n>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(n));
}

// Staging of 8-site blocks: one slot = 8 transition rows followed by the 8
// sites' emission data (8 float4, or the block's VQ word in the first 4
// bytes).  A forward slot holds sites m0 .. m0+7 in order with the rows
// T_m0 .. T_m0+7 the forward recursion applies there; a backward slot holds
// sites n0+7 .. n0 (row j is site n0 + 7 - j) with the rows T_{n0+8-j} the
// backward recursion applies there, so both directions read slot row j at
// step j of a block.
constexpr int kSlotF4 = 16;
// Slots per direction: block t uses slot t mod 4, so within the 4-block
// quarter words the loop runs, every slot offset is a constant; two blocks
// are in flight while one is read.
constexpr int kRing = 4;
// A group's ring: forward slots at [0, 64) and backward slots at [68, 132)
// float4, so the forward and the backward row a group reads at one step are 4
// float4 (16 banks) apart; rings of neighbouring groups are 137 float4 apart
// (1 mod 8), so the 16-byte reads of the four 8-lane groups of a warp -- two
// rows a group -- fall in eight distinct bank quads.
constexpr int kBwdOffF4 = kRing * kSlotF4 + 4;
constexpr int kGroupF4 = kBwdOffF4 + kRing * kSlotF4;
constexpr int kGroupStrideF4 = kGroupF4 + 5;
static_assert(kGroupStrideF4 % 8 == 1 && kBwdOffF4 % 8 == 4, "ring bank layout");

// The rows of an 8-row block that lane li of a P-lane group copies: nr rows
// from rb.  From P = 8 up lanes 0..7 take one row each; narrower groups take
// 8/P consecutive rows per lane, so that one copy instruction of the warp
// writes rows 8/P apart in each group: with the groups' rings 1 mod 8 float4
// apart, the 16-byte writes of the groups in a quarter warp then fall in
// disjoint banks (consecutive rows per instruction would overlap).
struct StageRows {
  uint32_t rb, nr;
};
template <int kMaxRows>
__device__ __forceinline__ StageRows stage_rows(uint32_t li, uint32_t P) {
  StageRows r;
  if (kMaxRows == 1 || P >= 8) {  // kMaxRows == 1: the kernel's groups never narrow below 8
    r.rb = li;
    r.nr = li < 8 ? 1u : 0u;
  } else {
    r.nr = 8u >> (__ffs(P) - 1);  // 8 / P, P a power of two
    r.rb = li * r.nr;
  }
  return r;
}

// Copies 8 consecutive float4 from src into dst (stage8) or into dst in
// reverse order, dst[7 - i] = src[i] (stage8_rev): this lane's rows of the
// block (kMaxRows = 8/P bounds nr for the group size P the kernel starts
// with; a group only widens later).
template <int kMaxRows>
__device__ __forceinline__ void stage8(float4 *dst, const float4 *src, StageRows r) {
#pragma unroll
  for (uint32_t k = 0; k < (uint32_t)kMaxRows; ++k)
    if (k < r.nr)
      cp_async16(dst + r.rb + k, src + r.rb + k);
}
template <int kMaxRows>
__device__ __forceinline__ void stage8_rev(float4 *dst, const float4 *src, StageRows r) {
#pragma unroll
  for (uint32_t k = 0; k < (uint32_t)kMaxRows; ++k)
    if (k < r.nr)
      cp_async16(dst + 7 - (r.rb + k), src + r.rb + k);
}

// Emission sources.  stage / stage_rev copy one block's emission data into
// a forward / backward slot; block(src, rev) prepares a staged block and
// at(b, j) returns the emission of the slot's row j; get1(m) reads site m
// directly (the sites above the last full block, and the site-by-site pass).
struct EmitF32 {
  const float4 *row;
  using Blk = const float4 *;
  __device__ __forceinline__ void init(const GenParams &p, uint32_t s, const float4 *) {
    row = p.emit + (size_t)s * p.S;
  }
  __device__ __forceinline__ float4 get1(uint32_t m) const { return __ldg(row + m); }
  // copy block t (sites 8t .. 8t+7) into a forward / backward slot
  template <int kMaxRows>
  __device__ __forceinline__ void stage(float4 *dst, uint32_t t, StageRows r) const {
    stage8<kMaxRows>(dst, row + 8 * (size_t)t, r);
  }
  template <int kMaxRows>
  __device__ __forceinline__ void stage_rev(float4 *dst, uint32_t t, StageRows r) const {
    stage8_rev<kMaxRows>(dst, row + 8 * (size_t)t, r);
  }
  __device__ __forceinline__ Blk block(const float4 *src, bool) const { return src; }
  __device__ __forceinline__ float4 at(Blk b, uint32_t j) const { return b[j]; }
};

// 4-bit VQ codes, eight per uint32, most significant nibble first
// (glPack.cpp:104-109, hmmLike.cu:20-24), so one block of 8 sites is one
// word; table[c] = FillEmit(decode(c)) computed once on the host.  A backward
// slot holds the same word; block() reverses its nibbles so that code j is
// the site of row j.
struct EmitVQ {
  const uint32_t *col;
  const float4 *table;
  uint32_t stride;
  using Blk = uint32_t;
  __device__ __forceinline__ void init(const GenParams &p, uint32_t s, const float4 *tab) {
    col = p.packed + s;
    stride = p.N;
    table = tab;
  }
  __device__ __forceinline__ float4 get1(uint32_t m) const {
    const uint32_t w = __ldg(col + (size_t)(m >> 3) * stride);
    return table[(w >> (28u - 4u * (m & 7u))) & 15u];
  }
  template <int kMaxRows>
  __device__ __forceinline__ void stage(float4 *dst, uint32_t t, StageRows r) const {
    if (r.rb == 0 && r.nr != 0)  // lane 0 of the group
      cp_async4(dst, col + (size_t)t * stride);
  }
  template <int kMaxRows>
  __device__ __forceinline__ void stage_rev(float4 *dst, uint32_t t, StageRows r) const {
    stage<kMaxRows>(dst, t, r);
  }
  __device__ __forceinline__ Blk block(const float4 *src, bool rev) const {
    const uint32_t w = *reinterpret_cast<const uint32_t *>(src);
    const uint32_t b = __byte_perm(w, 0u, 0x0123u);  // bytes reversed
    const uint32_t r = ((b >> 4) & 0x0f0f0f0fu) | ((b & 0x0f0f0f0fu) << 4);
    return rev ? r : w;
  }
  __device__ __forceinline__ float4 at(Blk w, uint32_t j) const {
    return table[(w >> (28u - 4u * j)) & 15u];
  }
};

// ---------------------------------------------------------------------------
// The 4-state recursion (impute.cpp:353-373).
//
// Both halves of an evaluation run in one form, x <- D_m (T x): the forward
// half carries alpha_m = D_m T_m alpha_{m-1} up from site 0 (T_0 = I on the
// uniform start); the backward half carries v_m = D_m beta_m = D_m T_{m+1}
// v_{m+1} down from the top site (T_S = I on the all-ones start).  The two
// meet at L = alpha_h . (T_{h+1} v_{h+1}).  T is symmetric, so this is the
// reference's likelihood; one code path serves both halves.

// The state in register pairs for the packed binary32 instructions of
// sm_100+ (__ffma2_rn and friends round each component as the scalar
// instruction does): X = (l00, l01), Y = (l11, l10), P = (p2, p1) with
// p1 = l01 + l10 and p2 = l00 + l11, so that X + Y = P.
struct FState {
  float2 X, Y, P;
  int k;
};

__device__ __forceinline__ void fstate_fill(FState &f, float l, int k) {
  f.X = f.Y = make_float2(l, l);
  f.P = make_float2(l + l, l + l);
  f.k = k;
}

__device__ __forceinline__ void select4(const float4 e, bool a0, bool a1, bool c0,
                                        bool c1, float &s00, float &s01, float &s10,
                                        float &s11) {
  const float lo0 = a0 ? e.z : e.x, hi0 = a0 ? e.w : e.y;
  const float lo1 = a1 ? e.z : e.x, hi1 = a1 ? e.w : e.y;
  s00 = c0 ? hi0 : lo0;
  s01 = c1 ? hi0 : lo0;
  s10 = c0 ? hi1 : lo1;
  s11 = c1 ? hi1 : lo1;
}

__device__ __forceinline__ void fstate_scale(FState &f, float sc) {
  const float2 s2 = make_float2(sc, sc);
  f.X = __fmul2_rn(f.X, s2);
  f.Y = __fmul2_rn(f.Y, s2);
  f.P = __fmul2_rn(f.P, s2);
}

// One step with per-site power-of-two rescaling (the site-by-site pass), for
// t = (x, y, z, x - z).
__device__ __forceinline__ void fwd_step(FState &f, const float4 t, float s00, float s01,
                                         float s10, float s11) {
  const float l00 = f.X.x, l01 = f.X.y, l10 = f.Y.y, l11 = f.Y.x, p1 = f.P.y, p2 = f.P.x;
  const float b00 = fmaf(l11, t.z, fmaf(p1, t.y, l00 * t.x));
  const float b01 = fmaf(l10, t.z, fmaf(p2, t.y, l01 * t.x));
  const float b10 = fmaf(l01, t.z, fmaf(p2, t.y, l10 * t.x));
  const float b11 = fmaf(l00, t.z, fmaf(p1, t.y, l11 * t.x));
  f.X = make_float2(b00 * s00, b01 * s01);
  f.Y = make_float2(b11 * s11, b10 * s10);
  f.P = __fadd2_rn(f.X, f.Y);
  if (f.P.x + f.P.y < kTiny) {
    fstate_scale(f, kHuge);
    f.k -= 64;
  }
}

// The same step without rescaling, in a shared-term form of T: with
// p1 = l01 + l10 and p2 = l00 + l11,
//   (T l)_00 = (x - z) l00 + c1,  (T l)_11 = (x - z) l11 + c1,  c1 = y p1 + z p2
//   (T l)_01 = (x - z) l01 + c2,  (T l)_10 = (x - z) l10 + c2,  c2 = y p2 + z p1
// so that X <- (w X + c) * sx and Y <- (w Y + c) * sy for c = (c1, c2),
// w = x - z: four scalar and five packed instructions a site.  t is a row of
// the pair table, (y, z, w, w), whose last two components form the pair
// (w, w).  The caller keeps the state in range by normalising at block
// boundaries.
__device__ __forceinline__ void fwd_fast(FState &f, const float4 t, float2 sx, float2 sy) {
  const float2 c = make_float2(fmaf(t.y, f.P.x, t.x * f.P.y), fmaf(t.y, f.P.y, t.x * f.P.x));
  const float2 w = make_float2(t.z, t.w);
  f.X = __fmul2_rn(__ffma2_rn(w, f.X, c), sx);
  f.Y = __fmul2_rn(__ffma2_rn(w, f.Y, c), sy);
  f.P = __fadd2_rn(f.X, f.Y);
}

// x <- T x alone (the backward half's last step, T_{h+1} v_{h+1}), for
// t = (x, y, z, x - z).
__device__ __forceinline__ void apply_tran(FState &f, const float4 t) {
  const float2 c = make_float2(fmaf(t.z, f.P.x, t.y * f.P.y), fmaf(t.z, f.P.y, t.y * f.P.x));
  const float2 w = make_float2(t.w, t.w);
  f.X = __ffma2_rn(w, f.X, c);
  f.Y = __ffma2_rn(w, f.Y, c);
}

// Exact power-of-two normalisation at a block boundary: scales the state so
// that its sum lies in [2^62, 2^63).  Starting a block of 8 sites in that
// range, the sums stay normal floats as long as the block shrinks them by less
// than 2^-124 (emissions are at most 1, so sums never grow).  The return
// value is e - 65 for the sum's biased exponent e: it lies outside [0, 127]
// exactly when the sum left [2^-62, 2^66), i.e. when range may have been lost
// in the block just computed (the scale is then meaningless too) and the
// evaluation must be redone with per-site rescaling.
__device__ __forceinline__ uint32_t fwd_norm(FState &f) {
  const uint32_t eb = __float_as_uint(f.P.x + f.P.y) & 0x7f800000u;
  fstate_scale(f, __uint_as_float(0x9e000000u - eb));  // 2^(189 - e)
  const int e = (int)(eb >> 23);
  f.k += e - 189;
  return (uint32_t)(e - 65);
}
// The same for a state kept in range site by site (any sum down to 2^-65 is
// legitimate there): the exponent is clamped so the scale stays a normal float.
__device__ __forceinline__ void fwd_renorm(FState &f) {
  const int e = (int)((__float_as_uint(f.P.x + f.P.y) >> 23) & 0xffu);
  const int ec = max(e, 62);
  fstate_scale(f, __uint_as_float((uint32_t)(316 - ec) << 23));  // 2^(189 - ec)
  f.k += ec - 189;
}

// Overflow guard of the site-by-site pass (emissions above 1 could grow it).
__device__ __forceinline__ void fwd_guard(FState &f) {
  if (f.P.x + f.P.y > kHuge) {
    fstate_scale(f, kTiny);
    f.k += 64;
  }
}

struct Parents {
  uint64_t f0, f1, m0, m1;
};

__device__ __forceinline__ Parents load_parents(const uint64_t *haps, uint32_t wn, uint4 q,
                                                uint32_t w) {
  Parents r;
  r.f0 = __ldg(haps + (size_t)q.x * wn + w);
  r.f1 = __ldg(haps + (size_t)q.y * wn + w);
  r.m0 = __ldg(haps + (size_t)q.z * wn + w);
  r.m1 = __ldg(haps + (size_t)q.w * wn + w);
  return r;
}

// Bit-reversed parent words: bit 63 - i holds site i of the word, so the
// backward half reads its descending sites as ascending bits.
__device__ __forceinline__ Parents reverse_parents(const Parents &p) {
  Parents r;
  r.f0 = __brevll(p.f0);
  r.f1 = __brevll(p.f1);
  r.m0 = __brevll(p.m0);
  r.m1 = __brevll(p.m1);
  return r;
}

__device__ __forceinline__ void prefetch_parents(const uint64_t *haps, uint32_t wn, uint4 q,
                                                 uint32_t w) {
  prefetch_l1(haps + (size_t)q.x * wn + w);
  prefetch_l1(haps + (size_t)q.y * wn + w);
  prefetch_l1(haps + (size_t)q.z * wn + w);
  prefetch_l1(haps + (size_t)q.w * wn + w);
}

// 32-bit halves of the four parent words: the bits of four 8-site blocks.
struct Bits32 {
  uint32_t f0, f1, m0, m1;
};

__device__ __forceinline__ Bits32 half_words(const Parents &pw, uint32_t h) {
  Bits32 r;
  r.f0 = (uint32_t)(pw.f0 >> (32 * h));
  r.f1 = (uint32_t)(pw.f1 >> (32 * h));
  r.m0 = (uint32_t)(pw.m0 >> (32 * h));
  r.m1 = (uint32_t)(pw.m1 >> (32 * h));
  return r;
}

// The emissions of one site as the pairs (s00, s01) and (s11, s10) that
// multiply X and Y.
__device__ __forceinline__ void site_emission(const float4 e, const Bits32 &bw, uint32_t j,
                                              float2 &sx, float2 &sy) {
  const uint32_t bit = 1u << j;  // j is a compile-time constant in the unrolled block
  select4(e, (bw.f0 & bit) != 0u, (bw.f1 & bit) != 0u, (bw.m0 & bit) != 0u,
          (bw.m1 & bit) != 0u, sx.x, sx.y, sy.y, sy.x);
}

// One staged block of 8 sites: row j of the slot (transition rows first,
// emission data from slot + 8) with bit 8B + j of the parent halves; the
// state is normalised at the end (kSub = 2: also after the first 4 sites)
// and eacc collects the range codes.
template <int B, class E, int kSub>
__device__ __forceinline__ void block8(FState &x, const E &em, const float4 *slot,
                                       typename E::Blk eb, const Bits32 &bw, uint32_t &eacc) {
#pragma unroll
  for (uint32_t j = 0; j < 8; ++j) {
    const float4 e = em.at(eb, j), t = slot[j];
    float2 sx, sy;
    site_emission(e, bw, 8 * B + j, sx, sy);
    fwd_fast(x, t, sx, sy);
    if (kSub == 2 && j == 3)
      eacc |= fwd_norm(x);
  }
  eacc |= fwd_norm(x);
}

// Log-likelihood of one quadruple by a plain forward pass, site by site, with
// the per-site power-of-two rescaling of fwd_step (the scheme of
// impute.cpp:327-376), reading emission, transition and parent words straight
// from global memory.  Used, rarely, for an evaluation whose blocked pass may
// have lost range.
template <class E>
__device__ __noinline__ double like_forward(const uint64_t *__restrict__ haps, uint32_t wn,
                                            uint32_t S, const float4 *__restrict__ tran4,
                                            const E em, uint4 q) {
  FState f;
  fstate_fill(f, 0.25f, 0);
  for (uint32_t w = 0; w < wn; ++w) {
    const Parents pw = load_parents(haps, wn, q, w);
    const uint32_t end = min(S, (w + 1) * 64);
    for (uint32_t m = w * 64; m < end; ++m) {
      const uint32_t j = m & 63u;
      float s00, s01, s10, s11;
      select4(em.get1(m), (pw.f0 >> j) & 1, (pw.f1 >> j) & 1, (pw.m0 >> j) & 1,
              (pw.m1 >> j) & 1, s00, s01, s10, s11);
      fwd_step(f, __ldg(tran4 + m), s00, s01, s10, s11);
    }
    fwd_guard(f);
  }
  const double sum = (((double)f.X.x + (double)f.X.y) + (double)f.Y.y) + (double)f.Y.x;
  return log(sum) + (double)f.k * 0.69314718055994530942;
}

// ln(dot) + k ln 2 for a positive dot product: the binary64 exponent of dot
// joins k exactly, and the logarithm of its mantissa m in [1, 2) is taken in
// binary32 (absolute error below 3e-7, against log-likelihoods of order
// -S), so the FP64 pipe only adds the two parts.  Dots far below the block
// range (never in the blocked pass) take the binary64 logarithm.
__device__ __forceinline__ double log_scaled(double dot, int k) {
  constexpr double kLn2 = 0.69314718055994530942;
  if (!(dot > 0x1p-1000))
    return log(dot) + (double)k * kLn2;
  const long long bits = __double_as_longlong(dot);
  const int e = (int)((bits >> 52) & 0x7ff) - 1023;
  const double m = __longlong_as_double((bits & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
  return (double)logf((float)m) + (double)(e + k) * kLn2;
}

// Log-likelihood (natural log, binary64) of quadruple q, scored by a lane
// pair of a P-lane group.  Of the nw = floor(S/64) full 64-site words, the
// even lane runs the forward half over words [0, wf), wf = ceil(nw/2); the
// odd lane first runs the sites of the partial top word site by site
// (straight from global memory), then the backward half over words
// [wf, nw) from the top.  Each word is eight 8-site blocks, run four at a
// time so that ring slots and parent-bit positions are constants: step t
// stages forward block t and backward block 8 nw - 1 - t of every pair into
// the group's ring (cp.async, two steps ahead), so the arithmetic reads
// shared memory only.  With an odd word count the odd lane idles through
// the last word (it computes on stale rows and restores its state after).
// States are normalised at block boundaries (exact powers of two); a
// quadruple whose block sums left the safe range is recomputed site by site
// by the even lane.  The pair joins with two exact-product shuffles, so both
// lanes return the same value.  All P lanes of the group call this together;
// gmask names the lanes that synchronise at each step (the group, or the
// whole warp when every group runs the same loop).  tran4 and tranp hold
// S + 1 rows, rows 0 and S the identity; the ring stages tranp's.
// kFull: every lane of the warp takes part (gmask is the full mask, known to
// the compiler).
template <int kMaxRows, class E, int kSub = 1, bool kFull = false>
__device__ __forceinline__ double eval_pair(const GenParams &p, const E &em, uint4 q,
                                            float4 *stage, uint32_t li, uint32_t P,
                                            unsigned gmask_in) {
  const unsigned gmask = kFull ? 0xffffffffu : gmask_in;
  const uint32_t S = p.S, wn = p.wn;
  const float4 *tran4 = p.tran4, *tranp = p.tranp;
  const bool bwd = (li & 1u) != 0;
  const uint32_t nw = S >> 6, wf = (nw + 1) >> 1, wb = nw - wf;
  const uint32_t nbf = 8 * wf, nbb = 8 * wb, top = 8 * nw - 1;  // blocks per direction
  // block-normalised states start at sum 2^62: the forward state 1/4 scaled
  // by 2^62, the backward state 1 scaled by 2^60
  FState x;
  fstate_fill(x, 0x1p60f, bwd ? -60 : -62);
  uint32_t eacc = 0;  // OR of the blocks' range codes (fwd_norm)
  if (bwd && (S & 63u)) {
    const Parents pw = load_parents(p.haps, wn, q, nw);
#pragma unroll 1
    for (int m = (int)S - 1; m >= (int)(nw * 64); --m) {
      const uint32_t j = (uint32_t)m & 63u;
      float s00, s01, s10, s11;
      select4(em.get1((uint32_t)m), (pw.f0 >> j) & 1, (pw.f1 >> j) & 1, (pw.m0 >> j) & 1,
              (pw.m1 >> j) & 1, s00, s01, s10, s11);
      fwd_step(x, __ldg(tran4 + m + 1), s00, s01, s10, s11);
    }
    fwd_renorm(x);
  }
  float4 *const stF = stage, *const stB = stage + kBwdOffF4;
  const StageRows rows = stage_rows<kMaxRows>(li, P);
  // block t0 + d of both directions into slot (t0 + d) mod 4: forward sites
  // 8t .. 8t+7 with rows T_8t .., backward sites of block top - t reversed
  // with the rows T_{m+1} of its sites m.  t0 is a multiple of 4 and d a
  // constant, so the sources are base pointers of the quarter word plus
  // constant offsets.
  auto issue = [&](uint32_t t0, uint32_t d) {
    const uint32_t t = t0 + d, slot = d & 3u;
    if (t < nbf) {
      stage8<kMaxRows>(stF + slot * kSlotF4, tranp + 8 * (size_t)t0 + 8 * d, rows);
      em.template stage<kMaxRows>(stF + slot * kSlotF4 + 8, t, rows);
    }
    if (t < nbb) {
      stage8_rev<kMaxRows>(stB + slot * kSlotF4, tranp + 8 * (size_t)(top - t0) + 1 - 8 * d,
                           rows);
      em.template stage_rev<kMaxRows>(stB + slot * kSlotF4 + 8, top - t, rows);
    }
    cp_async_commit();
  };
  issue(0, 0);
  issue(0, 1);
  float4 *const mine = bwd ? stB : stF;
#pragma unroll 1
  for (uint32_t i = 0; i < wf; ++i) {
    const bool act = !bwd || i < wb;
    const FState xs = x;
    const uint32_t es = eacc;
    const uint32_t w = bwd ? nw - 1 - i : i;
    const Parents raw = load_parents(p.haps, wn, q, w);
    const Parents pw = bwd ? reverse_parents(raw) : raw;
    if (i + 1 < (bwd ? wb : wf))  // this lane's next word
      prefetch_parents(p.haps, wn, q, bwd ? w - 1 : w + 1);
#pragma unroll 1
    for (uint32_t h = 0; h < 2; ++h) {
      const uint32_t t0 = 8 * i + 4 * h;
      const Bits32 bw = half_words(pw, h);
#pragma unroll
      for (uint32_t b = 0; b < 4; ++b) {
        // One barrier a block: the slot staged here, (t + 2) mod 4, was last
        // read at step t - 2, which every lane of the group finished before
        // the barrier of step t - 1 let this one go on.
        issue(t0, b + 2);
        cp_async_wait<2>();
        __syncwarp(gmask);
        const float4 *slot = mine + b * kSlotF4;
        switch (b) {  // bit positions 8b + j as constants
          case 0: block8<0, E, kSub>(x, em, slot, em.block(slot + 8, bwd), bw, eacc); break;
          case 1: block8<1, E, kSub>(x, em, slot, em.block(slot + 8, bwd), bw, eacc); break;
          case 2: block8<2, E, kSub>(x, em, slot, em.block(slot + 8, bwd), bw, eacc); break;
          default: block8<3, E, kSub>(x, em, slot, em.block(slot + 8, bwd), bw, eacc); break;
        }
      }
    }
    if (!act) {  // the odd lane's idle word
      x = xs;
      eacc = es;
    }
  }
  if (bwd)  // beta_{64 wf - 1} = T_{64 wf} v_{64 wf} (row S is the identity)
    apply_tran(x, __ldg(tran4 + 64 * (size_t)wf));
  const float y00 = __shfl_xor_sync(gmask, x.X.x, 1), y01 = __shfl_xor_sync(gmask, x.X.y, 1),
              y10 = __shfl_xor_sync(gmask, x.Y.y, 1), y11 = __shfl_xor_sync(gmask, x.Y.x, 1);
  const int yk = __shfl_xor_sync(gmask, x.k, 1);
  const uint32_t bad = (eacc | __shfl_xor_sync(gmask, eacc, 1)) & ~127u;
  // alpha . beta on both lanes: the same exact products in the same order
  const double dot = (double)x.X.x * (double)y00 + (double)x.X.y * (double)y01 +
                     (double)x.Y.y * (double)y10 + (double)x.Y.x * (double)y11;
  double L = log_scaled(dot, x.k + yk);
  if (__any_sync(gmask, bad != 0u)) {
    double Lf = L;
    if (bad && !bwd) {
      if (p.stats)
        atomicAdd(p.stats + 3, 1ull);
      Lf = like_forward(p.haps, wn, S, tran4, em, q);
    }
    L = __shfl_sync(gmask, Lf, (threadIdx.x & 31u) & ~1u);
  }
  return L;
}

// ---------------------------------------------------------------------------
// hmm_work, binary32 in the reference's operation order
// (impute.cpp:380-485): explicit _rn intrinsics keep nvcc from contracting
// products and sums into FMAs, so results are bit-identical to the CPU code.

__device__ __forceinline__ float pick(const float4 e, uint32_t i) {
  return (i & 2u) ? ((i & 1u) ? e.w : e.z) : ((i & 1u) ? e.y : e.x);
}


__device__ __forceinline__ float fma3_rn(float a0, float b0, float a1, float b1, float a2,
                                         float b2, float a3, float b3) {
  // ((a0*b0 + a1*b1) + a2*b2) + a3*b3, every product and sum rounded.
  return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(a0, b0), __fmul_rn(a1, b1)),
                             __fmul_rn(a2, b2)),
                   __fmul_rn(a3, b3));
}

// The reference's normalisation factor 1.0f / sum (impute.cpp:404, 441): the
// correctly rounded reciprocal, which is what __frcp_rn returns for every
// input, with a shorter dependency chain than the general division.
__device__ __forceinline__ float recip_rn(float x) { return __frcp_rn(x); }

// hmm_work is split in two passes with the reference's arithmetic unchanged.
// The forward state l_m of impute.cpp:416-447 does not depend on the sampled
// bits, so (1) the two sequential recursions -- the backward vectors beta_m
// (impute.cpp:389-414) and the forward l_m -- run per sample and leave
// p_m = l_m * beta_m (the products of impute.cpp:449-452) in the scratch:
// work_chains_pair runs them at the same time on two warps (a lane pair per
// recursion), work_chains one after the other on one thread (chunks mixed
// within a warp); (2) the
// sampling of impute.cpp:453-484 then runs for every site in parallel, one
// warp per part of a sample and 32 sites per instruction.

__device__ __forceinline__ uint32_t clamp_site(int m, uint32_t S) {
  return m < 0 ? 0u : ((uint32_t)m >= S ? S - 1 : (uint32_t)m);
}

// Rows of one 4-site step of pass 1: emission and transition rows (and, in
// the forward recursion, the backward vectors).  Steps are aligned to
// multiples of 4 sites, so a step never straddles a parent word; indices
// outside [0, S) are clamped (the rows loaded there are never used).
struct WorkRows {
  float4 e[4], t[4];
};
struct WorkRowsB {
  float4 e[4], t[4], b[4];
};

__device__ __forceinline__ void load_rows(WorkRows &r, const float4 *e, const float4 *tr,
                                          int m0, uint32_t S) {
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const uint32_t m = clamp_site(m0 + j, S);
    r.e[j] = __ldg(e + m);
    r.t[j] = __ldg(tr + m);
  }
}

__device__ __forceinline__ void load_rows(WorkRowsB &r, const float4 *e, const float4 *tr,
                                          const float4 *beta, int m0, uint32_t S) {
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const uint32_t m = clamp_site(m0 + j, S);
    r.e[j] = __ldg(e + m);
    r.t[j] = __ldg(tr + m);
    r.b[j] = beta[m];
  }
}

// Pass 1 of hmm_work for sample s with final quadruple q: beta_m for
// m = S-1 .. 0, then l_m for m = 0 .. S-1, leaving p_m = l_m * beta_m in
// p.beta[s][m].  The next 4-site step's rows are loaded before the current
// step is computed.
__device__ __forceinline__ void work_chains(const GenParams &p, uint32_t s, uint4 q) {
  const uint32_t S = p.S, wn = p.wn;
  const uint64_t *f0 = p.haps + (size_t)q.x * wn, *f1 = p.haps + (size_t)q.y * wn,
                 *m0 = p.haps + (size_t)q.z * wn, *m1 = p.haps + (size_t)q.w * wn;
  const float4 *e = p.emit + (size_t)s * S;
  const float4 *tr = p.tran4;
  float4 *beta = p.beta + (size_t)s * S;
  // backward recursion (impute.cpp:389-414): sites S-1 .. 1
  {
    float b0 = 1.f, b1 = 1.f, b2 = 1.f, b3 = 1.f;
    beta[S - 1] = make_float4(1.f, 1.f, 1.f, 1.f);
    const int top = (int)((S - 1) & ~3u);
    WorkRows cur, nxt;
    load_rows(cur, e, tr, top, S);
    for (int c0 = top; c0 >= 0; c0 -= 4) {
      // emission sites [c0 - 96, c0 - 64) into L2, two 32-site blocks ahead
      if ((c0 & 31) == 0 && c0 >= 96)
        prefetch_l2_bulk(e + (c0 - 96), 32 * sizeof(float4));
      load_rows(nxt, e, tr, c0 - 4, S);
      const uint32_t w = (uint32_t)c0 >> 6;
      const uint64_t A0 = __ldg(f0 + w), A1 = __ldg(f1 + w), C0 = __ldg(m0 + w),
                     C1 = __ldg(m1 + w);
#pragma unroll
      for (int j = 3; j >= 0; --j) {
        const int m = c0 + j;
        if (m >= 1 && m <= (int)S - 1) {
          const uint32_t sh = (uint32_t)m & 63u;
          const uint32_t a0 = (uint32_t)(A0 >> sh) & 1u, a1 = (uint32_t)(A1 >> sh) & 1u,
                         c0b = (uint32_t)(C0 >> sh) & 1u, c1b = (uint32_t)(C1 >> sh) & 1u;
          const float4 em = cur.e[j], t = cur.t[j];
          const float b00 = __fmul_rn(b0, pick(em, (a0 << 1) | c0b));
          const float b01 = __fmul_rn(b1, pick(em, (a0 << 1) | c1b));
          const float b10 = __fmul_rn(b2, pick(em, (a1 << 1) | c0b));
          const float b11 = __fmul_rn(b3, pick(em, (a1 << 1) | c1b));
          b0 = __fadd_rn(__fadd_rn(__fmul_rn(b00, t.x), __fmul_rn(__fadd_rn(b01, b10), t.y)),
                         __fmul_rn(b11, t.z));
          b1 = __fadd_rn(__fadd_rn(__fmul_rn(b01, t.x), __fmul_rn(__fadd_rn(b00, b11), t.y)),
                         __fmul_rn(b10, t.z));
          b2 = __fadd_rn(__fadd_rn(__fmul_rn(b10, t.x), __fmul_rn(__fadd_rn(b00, b11), t.y)),
                         __fmul_rn(b01, t.z));
          b3 = __fadd_rn(__fadd_rn(__fmul_rn(b11, t.x), __fmul_rn(__fadd_rn(b01, b10), t.y)),
                         __fmul_rn(b00, t.z));
          const float sum = __fdiv_rn(1.0f, __fadd_rn(__fadd_rn(__fadd_rn(b0, b1), b2), b3));
          b0 = __fmul_rn(b0, sum);
          b1 = __fmul_rn(b1, sum);
          b2 = __fmul_rn(b2, sum);
          b3 = __fmul_rn(b3, sum);
          beta[m - 1] = make_float4(b0, b1, b2, b3);
        }
      }
      cur = nxt;
    }
  }
  // forward recursion (impute.cpp:416-452): sites 0 .. S-1, p_m = l_m * beta_m
  float l00 = 0, l01 = 0, l10 = 0, l11 = 0;
  WorkRowsB cur, nxt;
  load_rows(cur, e, tr, beta, 0, S);
  for (uint32_t c0 = 0; c0 < S; c0 += 4) {
    // emission and backward sites [c0 + 64, c0 + 96) into L2, two blocks ahead
    if ((c0 & 31u) == 0 && c0 + 96 <= S) {
      prefetch_l2_bulk(e + c0 + 64, 32 * sizeof(float4));
      prefetch_l2_bulk(beta + c0 + 64, 32 * sizeof(float4));
    }
    load_rows(nxt, e, tr, beta, (int)c0 + 4, S);
    const uint32_t w = c0 >> 6;
    const uint64_t A0 = __ldg(f0 + w), A1 = __ldg(f1 + w), C0 = __ldg(m0 + w),
                   C1 = __ldg(m1 + w);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t m = c0 + (uint32_t)j;
      if (m < S) {
        const uint32_t sh = m & 63u;
        const uint32_t a0 = (uint32_t)(A0 >> sh) & 1u, a1 = (uint32_t)(A1 >> sh) & 1u,
                       c0b = (uint32_t)(C0 >> sh) & 1u, c1b = (uint32_t)(C1 >> sh) & 1u;
        const uint32_t s00 = (a0 << 1) | c0b, s01 = (a0 << 1) | c1b, s10 = (a1 << 1) | c0b,
                       s11 = (a1 << 1) | c1b;
        const float4 em = cur.e[j], t = cur.t[j], bb = cur.b[j];
        if (m) {
          const float b00 = fma3_rn(l00, t.x, l01, t.y, l10, t.y, l11, t.z);
          const float b01 = fma3_rn(l00, t.y, l01, t.x, l10, t.z, l11, t.y);
          const float b10 = fma3_rn(l00, t.y, l01, t.z, l10, t.x, l11, t.y);
          const float b11 = fma3_rn(l00, t.z, l01, t.y, l10, t.y, l11, t.x);
          l00 = __fmul_rn(b00, pick(em, s00));
          l01 = __fmul_rn(b01, pick(em, s01));
          l10 = __fmul_rn(b10, pick(em, s10));
          l11 = __fmul_rn(b11, pick(em, s11));
        } else {
          l00 = __fmul_rn(0.25f, pick(em, s00));
          l01 = __fmul_rn(0.25f, pick(em, s01));
          l10 = __fmul_rn(0.25f, pick(em, s10));
          l11 = __fmul_rn(0.25f, pick(em, s11));
        }
        const float sum = __fdiv_rn(1.0f, __fadd_rn(__fadd_rn(__fadd_rn(l00, l01), l10), l11));
        l00 = __fmul_rn(l00, sum);
        l01 = __fmul_rn(l01, sum);
        l10 = __fmul_rn(l10, sum);
        l11 = __fmul_rn(l11, sum);
        beta[m] = make_float4(__fmul_rn(l00, bb.x), __fmul_rn(l01, bb.y), __fmul_rn(l10, bb.z),
                              __fmul_rn(l11, bb.w));
      }
    }
    cur = nxt;
  }
}

// Staging of pass 1 for the 16 samples of a warp that share one chunk (two
// lanes a sample): each 16-site tile of the 16 per-sample rows (emission,
// and stored vectors) is copied into shared memory by the whole warp, one
// 256-byte row segment per half-warp instruction (cp.async, one tile in
// flight ahead), so every lane then reads its sample's row from shared
// memory.
constexpr int kTile = 16;
constexpr int kTileStrideF4 = kTile + 1;  // odd number of 16-byte units: no bank conflicts
constexpr int kPairRows = 16;             // samples per warp of pass 1

struct ChainTiles {
  float4 e[2][kPairRows * kTileStrideF4];
  float4 b[2][kPairRows * kTileStrideF4];
  float4 t[2][kTile];
  const float4 *erow[kPairRows];
  float4 *brow[kPairRows];
};

// Copy sites [base, base + kTile) of every row (rows with a null pointer are
// skipped); indices are clamped to [0, S).
__device__ __forceinline__ void stage_tile(float4 *dst, const float4 *const *rows, int base,
                                           uint32_t S, uint32_t lane) {
  const uint32_t half = lane >> 4, j = lane & 15u;
  const uint32_t m = clamp_site(base + (int)j, S);
#pragma unroll
  for (uint32_t r = 0; r < (uint32_t)kPairRows; r += 2) {
    const float4 *row = rows[r + half];
    if (row)
      cp_async16(dst + (r + half) * kTileStrideF4 + j, row + m);
  }
}

// The emission e[(abit << 1) | cbit] of impute.cpp:338-342 for bit j of the
// father word a and the mother word c.
__device__ __forceinline__ float pick_bits(const float4 e, uint32_t a, uint32_t c, int j) {
  const bool ab = (a >> j) & 1u, cb = (c >> j) & 1u;
  return ab ? (cb ? e.w : e.z) : (cb ? e.y : e.x);
}

// Pass 1 on lane pairs.  A generation has only 2N recursions of S
// sequential steps, so one lane a recursion leaves about one warp a
// scheduler, which then waits on each step's latency; here two lanes share a
// recursion, which doubles the warps.  Lane role 0 owns the states 00 and
// 11, role 1 the states 01 and 10: each lane computes the reference's
// formula for its own two states (impute.cpp:389-414 backward, 416-447
// forward) in the reference's binary32 operation order, one shuffle hands
// the pair the other two, and both lanes form the normalising sum in the
// reference's order, so both hold the same, bit-identical vector.
//
// The backward state is kept relative to the lane: (o1, o2) its own states,
// (p1, p2) the partner's -- role 0: (b0, b3, b1, b2), role 1: (b1, b2, b0,
// b3).  With the mother words of role 1 swapped (cf, cs), own state k picks
// its emission from (father word k, cf) for k = 1 and (father word 2, cs)
// for k = 2, and the partner's from the opposite mother word.
struct PairBwd {
  float o1, o2, p1, p2;
  __device__ __forceinline__ void step(float e_o1, float e_o2, float e_p1, float e_p2,
                                       const float4 t, bool r0) {
    const float xo1 = __fmul_rn(o1, e_o1), xo2 = __fmul_rn(o2, e_o2);
    const float pair = __fadd_rn(__fmul_rn(p1, e_p1), __fmul_rn(p2, e_p2));
    const float py = __fmul_rn(pair, t.y);
    const float A = __fadd_rn(__fadd_rn(__fmul_rn(xo1, t.x), py), __fmul_rn(xo2, t.z));
    const float B = __fadd_rn(__fadd_rn(__fmul_rn(xo2, t.x), py), __fmul_rn(xo1, t.z));
    const float pA = __shfl_xor_sync(0xffffffffu, A, 1), pB = __shfl_xor_sync(0xffffffffu, B, 1);
    // ((b0 + b1) + b2) + b3: role 0 holds b0 = A, b3 = B; role 1 b1 = A, b2 = B
    const float sum = __fadd_rn(__fadd_rn(__fadd_rn(A, pA), r0 ? pB : B), r0 ? B : pB);
    const float inv = recip_rn(sum);
    o1 = __fmul_rn(A, inv);
    o2 = __fmul_rn(B, inv);
    p1 = __fmul_rn(pA, inv);
    p2 = __fmul_rn(pB, inv);
  }
  // (b0, b1, b2, b3) for role 0
  __device__ __forceinline__ float4 vec() const { return make_float4(o1, p1, p2, o2); }
};

// The forward state is the reference's (l00, l01, l10, l11) in both lanes.
// Role 0 computes c00 and c11, role 1 c01 and c10 (the coefficient rows of
// T for those states), each times its own emission.
struct PairFwd {
  float l00, l01, l10, l11;
  __device__ __forceinline__ void finish(float A, float B, bool r0) {
    const float pA = __shfl_xor_sync(0xffffffffu, A, 1), pB = __shfl_xor_sync(0xffffffffu, B, 1);
    const float n00 = r0 ? A : pA, n01 = r0 ? pA : A, n10 = r0 ? pB : B, n11 = r0 ? B : pB;
    const float inv = recip_rn(__fadd_rn(__fadd_rn(__fadd_rn(n00, n01), n10), n11));
    l00 = __fmul_rn(n00, inv);
    l01 = __fmul_rn(n01, inv);
    l10 = __fmul_rn(n10, inv);
    l11 = __fmul_rn(n11, inv);
  }
  __device__ __forceinline__ void step(float e_o1, float e_o2, const float4 t, bool r0) {
    // role 0: c00 (x, y, y, z), c11 (z, y, y, x); role 1: c01 (y, x, z, y), c10 (y, z, x, y)
    const float cA = fma3_rn(l00, r0 ? t.x : t.y, l01, r0 ? t.y : t.x, l10, r0 ? t.y : t.z, l11,
                             r0 ? t.z : t.y);
    const float cB = fma3_rn(l00, r0 ? t.z : t.y, l01, r0 ? t.y : t.z, l10, r0 ? t.y : t.x, l11,
                             r0 ? t.x : t.y);
    finish(__fmul_rn(cA, e_o1), __fmul_rn(cB, e_o2), r0);
  }
  __device__ __forceinline__ void first(float e_o1, float e_o2, bool r0) {
    finish(__fmul_rn(0.25f, e_o1), __fmul_rn(0.25f, e_o2), r0);
  }
  __device__ __forceinline__ float4 vec() const { return make_float4(l00, l01, l10, l11); }
};

// Pass 1 split over two warps that share the same 16 samples (two lanes per
// sample in each): warp 0 runs the backward recursion from the top site and
// warp 1 the forward recursion from site 0, at the same time.  Neither
// depends on the other until p_m = l_m * beta_m, so each runs to the middle
// site mid storing its vectors -- beta_{m-1} for m >= mid (backward; index
// mid-1 upwards) and l_m for m <= mid-2 (forward; l_{mid-1} stays in
// registers) -- then, after a block barrier, each continues through the other
// half reading what the other stored and writing p there: the backward warp
// p_m for m <= mid-2 (beta_m fresh, l_m stored), the forward warp p_{mid-1}
// and p_m for m >= mid (l_m fresh, beta_m stored).  The operations on every
// vector are those of work_chains, so p is bit-identical.  Role-0 lanes store
// the vectors.  Both warps call this together, every lane (lanes of samples
// past the end compute on whatever their rows hold and store nothing).
__device__ __forceinline__ void work_chains_pair(const GenParams &p, uint32_t s, uint4 q,
                                                 bool valid, uint32_t lane, bool fwd,
                                                 ChainTiles &sm) {
  const uint32_t S = p.S, wn = p.wn;
  const float4 *tr = p.tran4;
  const bool r0 = (lane & 1u) == 0;
  const bool writer = valid && r0;
  const uint32_t row = lane >> 1;
  const uint64_t *f0 = p.haps + (size_t)q.x * wn, *f1 = p.haps + (size_t)q.y * wn,
                 *m0 = p.haps + (size_t)q.z * wn, *m1 = p.haps + (size_t)q.w * wn;
  // role 1 owns 01 and 10: its first own state takes the second mother word
  const uint64_t *mf = r0 ? m0 : m1, *ms = r0 ? m1 : m0;
  float4 *beta = p.beta + (size_t)s * S;
  if (r0) {
    sm.erow[row] = valid ? p.emit + (size_t)s * S : nullptr;
    sm.brow[row] = valid ? beta : nullptr;
  }
  if (!fwd && writer)
    beta[S - 1] = make_float4(1.f, 1.f, 1.f, 1.f);
  __syncwarp();
  const int ntiles = (int)((S + kTile - 1) / kTile);
  const int top = (int)((S - 1) & ~(uint32_t)(kTile - 1));
  const int mid = kTile * (ntiles / 2);            // first site of the upper half
  const int n_hi = (top - mid) / kTile + 1;        // tiles [mid, S)
  const int n_lo = mid / kTile;                    // tiles [0, mid)
  const float4 *const *erows = sm.erow;
  const float4 *const *brows = sm.brow;
  // emission rows of the tile at base, stored vectors from bbase (with_b)
  auto stage = [&](int buf, int base, bool with_b, int bbase) {
    stage_tile(sm.e[buf], erows, base, S, lane);
    if (with_b)
      stage_tile(sm.b[buf], brows, bbase, S, lane);
    if (lane < kTile)
      cp_async16(&sm.t[buf][lane], tr + clamp_site(base + (int)lane, S));
    cp_async_commit();
  };
  PairBwd vb;
  vb.o1 = vb.o2 = vb.p1 = vb.p2 = 1.f;
  PairFwd vf;
  vf.l00 = vf.l01 = vf.l10 = vf.l11 = 0.f;
  // the four parent words of the current 64-site word, mother words by role
  uint64_t wa0 = 0, wa1 = 0, wcf = 0, wcs = 0;
  int wcur = -1;
  auto words = [&](uint32_t w) {
    if ((int)w != wcur) {
      wa0 = __ldg(f0 + w);
      wa1 = __ldg(f1 + w);
      wcf = __ldg(mf + w);
      wcs = __ldg(ms + w);
      wcur = (int)w;
    }
  };

  // backward (impute.cpp:389-414) over n tiles from the tile at first down;
  // comb: store p_{m-1} = l_{m-1} * beta_{m-1} (l staged one site lower)
  auto run_bwd = [&](int first, int n, bool comb) {
    if (n <= 0)
      return;
    stage(0, first, comb, first - 1);
    for (int i = 0; i < n; ++i) {
      const int base = first - kTile * i, buf = i & 1;
      if (i + 1 < n)
        stage(buf ^ 1, base - kTile, comb, base - kTile - 1);
      else
        cp_async_commit();
      words((uint32_t)base >> 6);
      const uint32_t A0 = (uint32_t)(wa0 >> (base & 63)), A1 = (uint32_t)(wa1 >> (base & 63)),
                     CF = (uint32_t)(wcf >> (base & 63)), CS = (uint32_t)(wcs >> (base & 63));
      cp_async_wait<1>();
      __syncwarp();
      const float4 *erow = sm.e[buf] + row * kTileStrideF4;
      const float4 *lrow = sm.b[buf] + row * kTileStrideF4;
      auto store = [&](int j) {  // beta_{m-1} (or p_{m-1}) for site m = base + j
        if (!writer)
          return;
        const float4 v = vb.vec();
        if (comb) {
          const float4 l = lrow[j];
          beta[base + j - 1] = make_float4(__fmul_rn(l.x, v.x), __fmul_rn(l.y, v.y),
                                           __fmul_rn(l.z, v.z), __fmul_rn(l.w, v.w));
        } else {
          beta[base + j - 1] = v;
        }
      };
      auto one = [&](int j) {
        const float4 e = erow[j];
        vb.step(pick_bits(e, A0, CF, j), pick_bits(e, A1, CS, j), pick_bits(e, A0, CS, j),
                pick_bits(e, A1, CF, j), sm.t[buf][j], r0);
        store(j);
      };
      if (base >= 1 && base + kTile - 1 <= (int)S - 1) {
#pragma unroll
        for (int j = kTile - 1; j >= 0; --j)
          one(j);
      } else {
#pragma unroll 1
        for (int j = kTile - 1; j >= 0; --j)
          if (base + j >= 1 && base + j <= (int)S - 1)
            one(j);
      }
      __syncwarp();  // the buffer is refilled next iteration
    }
  };

  // forward (impute.cpp:416-452) over n tiles from the tile at first up;
  // comb: store p_m = l_m * beta_m (beta staged), else l_m for m <= mid - 2
  auto run_fwd = [&](int first, int n, bool comb) {
    if (n <= 0)
      return;
    stage(0, first, comb, first);
    for (int i = 0; i < n; ++i) {
      const int base = first + kTile * i, buf = i & 1;
      if (i + 1 < n)
        stage(buf ^ 1, base + kTile, comb, base + kTile);
      else
        cp_async_commit();
      words((uint32_t)base >> 6);
      const uint32_t A0 = (uint32_t)(wa0 >> (base & 63)), A1 = (uint32_t)(wa1 >> (base & 63)),
                     CF = (uint32_t)(wcf >> (base & 63)), CS = (uint32_t)(wcs >> (base & 63));
      cp_async_wait<1>();
      __syncwarp();
      const float4 *erow = sm.e[buf] + row * kTileStrideF4;
      const float4 *brow = sm.b[buf] + row * kTileStrideF4;
      auto store = [&](int j) {  // l_m (or p_m) for site m = base + j
        const int m = base + j;
        if (!writer)
          return;
        const float4 v = vf.vec();
        if (comb) {
          const float4 bb = brow[j];
          beta[m] = make_float4(__fmul_rn(v.x, bb.x), __fmul_rn(v.y, bb.y),
                                __fmul_rn(v.z, bb.z), __fmul_rn(v.w, bb.w));
        } else if (m <= mid - 2) {
          beta[m] = v;
        }
      };
      auto one = [&](int j) {
        const float4 e = erow[j];
        const float e1 = pick_bits(e, A0, CF, j), e2 = pick_bits(e, A1, CS, j);
        if (base + j == 0)
          vf.first(e1, e2, r0);
        else
          vf.step(e1, e2, sm.t[buf][j], r0);
        store(j);
      };
      if (base >= 1 && base + kTile <= (int)S) {
#pragma unroll
        for (int j = 0; j < kTile; ++j)
          one(j);
      } else {
#pragma unroll 1
        for (int j = 0; j < kTile; ++j)
          if (base + j < (int)S)
            one(j);
      }
      __syncwarp();
    }
  };

  if (fwd)
    run_fwd(0, n_lo, false);
  else
    run_bwd(top, n_hi, false);
  // both halves' vectors are stored (block barrier: the two warps)
  __syncthreads();
  if (fwd) {
    if (writer && mid >= 1) {  // p_{mid-1}: l_{mid-1} still in registers
      const float4 bb = beta[mid - 1];
      const float4 v = vf.vec();
      beta[mid - 1] = make_float4(__fmul_rn(v.x, bb.x), __fmul_rn(v.y, bb.y),
                                  __fmul_rn(v.z, bb.z), __fmul_rn(v.w, bb.w));
    }
    run_fwd(mid, n_hi, true);
  } else {
    run_bwd(mid - kTile, n_lo, true);
  }
}

// Pass 2 of hmm_work: the sampling of impute.cpp:453-484 for site m of
// sample s, from p_m (pass 1), the genotype probabilities, the
// mutation-matrix rows pcr (pc[i][0..3] as float4) and the site's uniform
// u_bits (the draw's 32 bits; the trace's value when one is given).  Returns
// the two haplotype bits of the site as bits 0 and 1 (0 for sites past S).
__device__ __forceinline__ uint32_t work_sample_site(const GenParams &p, const float4 *pcr,
                                                     uint32_t s, uint32_t m, uint64_t A0,
                                                     uint64_t A1, uint64_t C0, uint64_t C1,
                                                     uint32_t u_bits) {
  const uint32_t S = p.S;
  if (m >= S)
    return 0;
  const uint32_t sh = m & 63u;
  const uint32_t a0 = (uint32_t)(A0 >> sh) & 1u, a1 = (uint32_t)(A1 >> sh) & 1u,
                 c0b = (uint32_t)(C0 >> sh) & 1u, c1b = (uint32_t)(C1 >> sh) & 1u;
  const uint32_t s00 = (a0 << 1) | c0b, s01 = (a0 << 1) | c1b, s10 = (a1 << 1) | c0b,
                 s11 = (a1 << 1) | c1b;
  const float4 pp = p.beta[(size_t)s * S + m];
  const float *pr = p.prob + ((size_t)s * S + m) * 3;
  const float g0 = __ldg(pr), g1 = __ldg(pr + 1), g2 = __ldg(pr + 2);
  const float4 r00 = pcr[s00], r01 = pcr[s01], r10 = pcr[s10], r11 = pcr[s11];
  const float inner0 = fma3_rn(pp.x, r00.x, pp.y, r01.x, pp.z, r10.x, pp.w, r11.x);
  const float inner1 = fma3_rn(pp.x, r00.y, pp.y, r01.y, pp.z, r10.y, pp.w, r11.y);
  const float inner2 = fma3_rn(pp.x, r00.z, pp.y, r01.z, pp.z, r10.z, pp.w, r11.z);
  const float inner3 = fma3_rn(pp.x, r00.w, pp.y, r01.w, pp.z, r10.w, pp.w, r11.w);
  float c[4] = {__fmul_rn(g0, inner0), __fmul_rn(g1, inner1), __fmul_rn(g1, inner2),
                __fmul_rn(g2, inner3)};
  if (p.pen != 1.0f) {
#pragma unroll
    for (int k = 0; k < 4; ++k)
      c[k] = powf(c[k], p.pen);
  }
  const float u = p.tr_work ? __ldg(p.tr_work + (size_t)s * S + m) : glp_u24(u_bits);
  const float c01 = __fadd_rn(c[0], c[1]);
  const float c012 = __fadd_rn(c01, c[2]);
  const float r = __fmul_rn(u, __fadd_rn(c012, c[3]));
  if (r < c[0])
    return 0u;  // (0, 0)
  if (r < c01)
    return 2u;  // (0, 1)
  if (r < c012)
    return 1u;  // (1, 0)
  return 3u;    // (1, 1)
}

// Pass 2 for words [w_lo, w_hi) of sample s (called by a whole warp; w_lo
// even), two words at a time: lane l draws the four uniforms of the l-th
// 4-site group of the
// 128-site span (one draw per group, as the reference draws them) into
// u[4 l .. 4 l + 3], so u[o] is the uniform of span site o; then the bits
// of sites w*64 + lane and w*64 + 32 + lane of each word are gathered into
// the two new haplotype words with ballots.
__device__ __forceinline__ void work_sample(const GenParams &p, const float4 *pcr, uint32_t s,
                                            uint4 q, uint32_t lane, uint32_t *u, uint32_t w_lo,
                                            uint32_t w_hi) {
  const uint32_t wn = p.wn;
  const uint64_t *f0 = p.haps + (size_t)q.x * wn, *f1 = p.haps + (size_t)q.y * wn,
                 *m0 = p.haps + (size_t)q.z * wn, *m1 = p.haps + (size_t)q.w * wn;
  uint64_t *ha = p.hnew + (size_t)2 * s * wn, *hb = ha + wn;
  for (uint32_t w2 = w_lo; w2 < w_hi; w2 += 2) {
    if (!p.tr_work) {
      const glp_u32x4 ux = glp_draw(p.seed, p.generation, s, 16 * w2 + lane, GLP_TAG_WORK);
      reinterpret_cast<uint4 *>(u)[lane] = make_uint4(ux.v[0], ux.v[1], ux.v[2], ux.v[3]);
    }
    __syncwarp();
#pragma unroll
    for (uint32_t t = 0; t < 2; ++t) {
      const uint32_t w = w2 + t;
      if (w >= w_hi)
        break;
      const uint64_t A0 = __ldg(f0 + w), A1 = __ldg(f1 + w), C0 = __ldg(m0 + w),
                     C1 = __ldg(m1 + w);
      const uint32_t lo = work_sample_site(p, pcr, s, w * 64 + lane, A0, A1, C0, C1,
                                           u[64 * t + lane]);
      const uint32_t hi = work_sample_site(p, pcr, s, w * 64 + 32 + lane, A0, A1, C0, C1,
                                           u[64 * t + 32 + lane]);
      const uint32_t alo = __ballot_sync(0xffffffffu, lo & 1u),
                     ahi = __ballot_sync(0xffffffffu, hi & 1u);
      const uint32_t blo = __ballot_sync(0xffffffffu, lo & 2u),
                     bhi = __ballot_sync(0xffffffffu, hi & 2u);
      if (lane == 0) {
        ha[w] = ((uint64_t)ahi << 32) | alo;
        hb[w] = ((uint64_t)bhi << 32) | blo;
      }
    }
    __syncwarp();  // u is redrawn next span
  }
}

// ---------------------------------------------------------------------------
// The generation kernels.

__device__ __forceinline__ void set_slot(uint4 &q, uint32_t r, uint32_t v) {
  if (r == 0)
    q.x = v;
  else if (r == 1)
    q.y = v;
  else if (r == 2)
    q.z = v;
  else
    q.w = v;
}

// Work sources.  One chunk: the kernel parameter.  Many chunks: a descriptor
// table in global memory; the samples of all chunks form one queue, chunk by
// chunk, so a group's neighbours in the queue usually share its chunk.
// Pass 2 of one chunk splits each sample's words into parts of
// kSampleWords, one warp a part, so that its warps are many and short and the
// last of them leave little of the GPU idle (many chunks: one part a sample).
#ifndef GLP_SAMPLE_WORDS
#define GLP_SAMPLE_WORDS 16
#endif
constexpr uint32_t kSampleWords = GLP_SAMPLE_WORDS;
static_assert(kSampleWords % 2 == 0, "a part starts a two-word span");
__host__ __device__ inline uint32_t sample_parts(uint32_t wn) {
  return (wn + kSampleWords - 1) / kSampleWords;
}

struct OneChunk {
  static constexpr bool kMulti = false;
  const GenParams &p;
  __device__ __forceinline__ uint32_t total() const { return p.N; }
  __device__ __forceinline__ uint32_t parts() const { return sample_parts(p.wn); }
  __device__ __forceinline__ const GenParams &chunk(uint32_t) const { return p; }
  __device__ __forceinline__ void locate(uint32_t g, uint32_t &c, uint32_t &s) const {
    c = 0;
    s = g;
  }
};

struct MultiParams {
  const GenParams *chunks;   // [nchunks]
  const uint32_t *offsets;   // [nchunks + 1] prefix sums of the chunks' N
  uint32_t nchunks;
  uint32_t *counter;
  unsigned long long *stats;
  int *error;
};

struct ManyChunks {
  static constexpr bool kMulti = true;
  const MultiParams &mp;
  __device__ __forceinline__ uint32_t total() const { return __ldg(mp.offsets + mp.nchunks); }
  __device__ __forceinline__ uint32_t parts() const { return 1; }
  __device__ __forceinline__ const GenParams &chunk(uint32_t c) const { return mp.chunks[c]; }
  __device__ __forceinline__ void locate(uint32_t g, uint32_t &c, uint32_t &s) const {
    uint32_t lo = 0, hi = mp.nchunks;  // largest c with offsets[c] <= g
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (__ldg(mp.offsets + mid) <= g)
        lo = mid;
      else
        hi = mid;
    }
    c = lo;
    s = g - __ldg(mp.offsets + lo);
  }
};

// Lane groups of a warp.  A warp starts as 32/P groups of P lanes (P is the
// smallest group size the kernel is instantiated for).  Once the sample queue
// is exhausted and some of the warp's groups have no sample left, the warp's
// 32 lanes are re-partitioned among its remaining samples: na samples get
// groups of p = 32 / nextpow2(na) or 2p lanes (the 2p-groups first, every
// group aligned to its size), so the longest chains of a generation finish
// with wider speculation instead of leaving lanes idle.
struct LaneGroups {
  uint32_t size, base, index, count;
};

__device__ __forceinline__ LaneGroups regroup(uint32_t lane, uint32_t na) {
  const uint32_t np2 = 1u << (32 - __clz(na - 1u));  // nextpow2(na), na >= 1
  const uint32_t p = 32u / (na > 1 ? np2 : 1u);
  const uint32_t nbig = 32u / p - na;  // groups of 2p lanes
  LaneGroups g;
  g.count = na;
  if (lane < nbig * 2 * p) {
    g.size = 2 * p;
    g.index = lane / (2 * p);
    g.base = g.index * 2 * p;
  } else {
    g.size = p;
    g.index = nbig + (lane - nbig * 2 * p) / p;
    g.base = nbig * 2 * p + (g.index - nbig) * p;
  }
  return g;
}

// The accept rule of MHSampler<T>::SampleHap (MHSampler.hpp:86-93) for a
// uniform u in [0, 1) with 53-bit resolution: accept when prop >= curr or
// u < exp((prop - curr) pen).  For d = (prop - curr) pen in (-37, 0) the
// exponential is taken in binary32 (relative error below 3e-6: a decision can
// differ from the binary64 one only where |d - ln u| < 3e-6); below -37 it
// is under 2^-53, so only u = 0 accepts, as in binary64.
__device__ __forceinline__ bool mh_accept(double prop, double curr, float pen, double u) {
  if (prop >= curr)
    return true;
  const double d = (prop - curr) * (double)pen;
  if (d > -37.0)
    return u < (double)expf((float)d);
  return u == 0.0 && u < exp(d);
}

template <int P, class E, class Src, int kSub = 1>
__device__ __forceinline__ void generation_body(const Src &src, uint32_t *counter,
                                                unsigned long long *stats, int *error,
                                                const float4 *vq_smem) {
  static_assert(P == 2 || P == 4 || P == 8 || P == 16 || P == 32, "P");
  constexpr unsigned FULL = 0xffffffffu;
  constexpr uint32_t G0 = 32u / P;  // group slots (staging rings) per warp
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  // current partition of the warp's lanes
  uint32_t Pc = P, gbase = lane - lane % P, gidx = lane / P, ngroups = G0;
  uint32_t li = lane - gbase;
  extern __shared__ float4 glp_stage[];  // kWarps * (32/P) * kGroupStrideF4 float4

  const uint32_t total = src.total();
  // The first sample of group slot g of global warp w is g * W + w, which
  // spreads the samples evenly over the warps; later samples come from the
  // queue counter, offset past those.
  const uint32_t nwarps = gridDim.x * (uint32_t)kWarps;
  const uint32_t gwarp = blockIdx.x * (uint32_t)kWarps + warp;
  const uint32_t spread = (uint32_t)min((unsigned long long)total,
                                        (unsigned long long)G0 * nwarps);
  bool first = true;
  uint32_t c = 0, s = kNone, e = 0;
  uint4 q = make_uint4(0, 0, 0, 0);
  double curr = 0.0;
  bool exhausted = false;
  unsigned long long n_evals = 0, n_rounds = 0, n_acc = 0;
  unsigned long long n_warp_rounds = 0, n_active_lanes = 0;

  while (true) {
    // idle groups take the next sample from the generation's queue
    const bool need = (s == kNone) && !exhausted;
    uint32_t ns = 0;
    if (need && li == 0) {
      if (first) {
        const unsigned long long f = (unsigned long long)gidx * nwarps + gwarp;
        ns = f < spread ? (uint32_t)f : total;
      } else {
        ns = spread + atomicAdd(counter, 1u);
      }
    }
    first = false;
    ns = __shfl_sync(FULL, ns, gbase);
    if (need) {
      if (ns < total) {
        src.locate(ns, c, s);
        e = 0;
        const GenParams &p = src.chunk(c);
        const uint32_t N = p.N;
        if (p.quad_in) {
          q = make_uint4(__ldg(p.quad_in + s), __ldg(p.quad_in + N + s),
                         __ldg(p.quad_in + 2 * (size_t)N + s),
                         __ldg(p.quad_in + 3 * (size_t)N + s));
        } else {
          // fresh quadruple from the sampler, as RunHMMOnSamples draws one
          // every generation (hmmLike.cpp:90-95)
          q.x = glp_surrogate(p.seed, p.generation, s, 0, GLP_TAG_INIT, p.samp_lo, p.samp_hi,
                              p.nbr, p.klen);
          q.y = glp_surrogate(p.seed, p.generation, s, 1, GLP_TAG_INIT, p.samp_lo, p.samp_hi,
                              p.nbr, p.klen);
          q.z = glp_surrogate(p.seed, p.generation, s, 2, GLP_TAG_INIT, p.samp_lo, p.samp_hi,
                              p.nbr, p.klen);
          q.w = glp_surrogate(p.seed, p.generation, s, 3, GLP_TAG_INIT, p.samp_lo, p.samp_hi,
                              p.nbr, p.klen);
        }
        const uint32_t H = p.H;
        if (q.x >= H || q.y >= H || q.z >= H || q.w >= H) {
          atomicOr(error, 1);
          q = make_uint4(0, 0, 0, 0);
        }
      } else {
        exhausted = true;
      }
    }
    // groups still without a sample cannot get one any more: hand their
    // lanes to the warp's remaining samples
    const unsigned lead = __ballot_sync(FULL, li == 0 && s != kNone);
    if (lead == 0)
      break;
    const uint32_t na = __popc(lead);
    if (na < ngroups) {
      const LaneGroups ng = regroup(lane, na);
      const uint32_t from = __fns(lead, 0, (int)ng.index + 1);
      c = __shfl_sync(FULL, c, from);
      s = __shfl_sync(FULL, s, from);
      e = __shfl_sync(FULL, e, from);
      q.x = __shfl_sync(FULL, q.x, from);
      q.y = __shfl_sync(FULL, q.y, from);
      q.z = __shfl_sync(FULL, q.z, from);
      q.w = __shfl_sync(FULL, q.w, from);
      curr = __shfl_sync(FULL, curr, from);
      Pc = ng.size;
      gbase = ng.base;
      gidx = ng.index;
      ngroups = ng.count;
      li = lane - gbase;
      exhausted = true;
    }
    const bool active = s != kNone;
    const unsigned amask = __ballot_sync(FULL, active);
    if (lane == 0) {
      ++n_warp_rounds;
      n_active_lanes += __popc(amask);
    }

    const GenParams &p = src.chunk(c);
    const uint32_t N = p.N, C = p.C, H = p.H;
    // One speculative round: the group's Pc/2 lane pairs score the next Pc/2
    // positions of the chain, pair r = li/2 position e + r (its even lane the
    // forward half, its odd lane the backward half of the evaluation).
    const uint32_t npos = Pc >> 1, r = li >> 1, ev = e + r;
    const bool lead_lane = (li & 1u) == 0;
    const uint32_t k = active ? min(npos, C + 1 - e) : 0u;
    uint32_t slot = 0, phap = 0;
    double u = 0.0;
    uint4 myq = q;
    if (r < k && ev > 0) {
      const uint32_t cyc = ev - 1;
      if (p.tr_slot) {
        slot = p.tr_slot[(size_t)s * C + cyc] & 3u;
        u = p.tr_u[(size_t)s * C + cyc];
      } else {
        glp_mh_draw(p.seed, p.generation, s, cyc, &slot, &u);
      }
      phap = p.props ? __ldg(p.props + (size_t)cyc * N + s)
             : (p.kick_first && cyc == 0)
                 ? glp_surrogate_ref(p.seed, p.generation, s, cyc, GLP_TAG_PROP, 2u * N, H,
                                     p.nbr, p.klen)
                 : glp_surrogate(p.seed, p.generation, s, cyc, GLP_TAG_PROP, p.samp_lo,
                                 p.samp_hi, p.nbr, p.klen);
      if (phap >= H) {
        atomicOr(error, 1);
        phap = 0;
      }
      set_slot(myq, slot, phap);
    }
    double L = 0.0;
    // When every lane of the warp scores a chunk of the same length, all
    // groups run the same block loop and synchronise as one warp: a
    // group-masked __syncwarp would let the groups drift apart and issue the
    // loop body once per group.
    unsigned same = 0;
    __match_all_sync(FULL, active ? p.S : 0u, (int *)&same);
    const bool warp_lockstep = same && amask == FULL;
    if (active) {
      // every pair of an active group evaluates (positions past k score the
      // base quadruple and drop the result) so the group shares its ring
      E em;
      em.init(p, s, Src::kMulti ? p.vq_table : vq_smem);
      const unsigned gm = (Pc == 32 || warp_lockstep) ? FULL : (((1u << Pc) - 1u) << gbase);
      float4 *ring = glp_stage + ((size_t)warp * G0 + gidx) * kGroupStrideF4;
      L = (gm == FULL)
              ? eval_pair<(P >= 8 ? 1 : 8 / P), E, kSub, true>(p, em, myq, ring, li, Pc, gm)
              : eval_pair<(P >= 8 ? 1 : 8 / P), E, kSub, false>(p, em, myq, ring, li, Pc, gm);
      if (r >= k)
        L = 0.0;
    }
    // The accept rule of MHSampler.hpp:86-93 in chain order.  Every
    // evaluation of the round was built on the round's starting state, and
    // until the first acceptance the chain's current likelihood is the
    // starting one, so each position tests its own proposal against it in
    // parallel and the first accepting position (in chain order) wins: the
    // same decisions as the sequential loop.  The even lanes vote.
    const double L0 = __shfl_sync(FULL, L, gbase);
    const double curr0 = (e == 0) ? L0 : curr;
    const bool acc = lead_lane && r < k && ev > 0 && mh_accept(L, curr0, p.pen, u);
    const unsigned gmask = (Pc == 32) ? FULL : (((1u << Pc) - 1u) << gbase);
    const unsigned abal = __ballot_sync(FULL, acc) & gmask;
    const uint32_t srcl = abal ? (uint32_t)(__ffs(abal) - 1) : gbase;
    const uint32_t first_acc = abal ? (srcl - gbase) >> 1 : npos;
    const double La = __shfl_sync(FULL, L, srcl);
    const uint32_t sla = __shfl_sync(FULL, slot, srcl);
    const uint32_t pha = __shfl_sync(FULL, phap, srcl);
    // The positions after the first acceptance that replace the same slot
    // scored exactly the quadruple the sequential chain builds there (it
    // differs from the round's start only in that slot), so the chain goes on
    // through them -- each tested against the likelihood accepted last --
    // up to the first position that replaces another slot.
    uint32_t last = first_acc, hap = pha;
    uint32_t more = 0;  // accepted positions after first_acc
    double cur = La;
    bool go = active && abal != 0;
    for (uint32_t d = 1; d < 16u; ++d) {
      const uint32_t r2 = first_acc + d;
      go = go && r2 < k;
      const uint32_t from = gbase + 2u * (go ? r2 : 0u);
      const uint32_t sl_r = __shfl_sync(FULL, slot, from);
      go = go && sl_r == sla;
      if (!__any_sync(FULL, go))
        break;
      const double L_r = __shfl_sync(FULL, L, from), u_r = __shfl_sync(FULL, u, from);
      const uint32_t ph_r = __shfl_sync(FULL, phap, from);
      if (go) {
        last = r2;
        if (mh_accept(L_r, cur, p.pen, u_r)) {
          cur = L_r;
          hap = ph_r;
          more |= 1u << r2;
        }
      }
    }
    if (active) {
      curr = curr0;
      if (abal) {
        set_slot(q, sla, hap);
        curr = cur;
      }
    }
    if (lead_lane && r < k && r <= last) {
      if (p.eval_trace)
        p.eval_trace[(size_t)s * (C + 1) + ev] = L;
      if (ev > 0 && p.accept_trace)
        p.accept_trace[(size_t)s * C + ev - 1] =
            (uint8_t)(r == first_acc || ((more >> r) & 1u));
    }
    if (active) {
      e = (first_acc < npos) ? e + last + 1 : e + k;
      if (li == 0) {
        n_evals += k;
        ++n_rounds;
        n_acc += first_acc < npos ? 1u + (uint32_t)__popc(more) : 0u;
      }
    }

    // finished chains: publish (hmm_work_kernel samples their haplotypes)
    const bool done = active && e > C;
    if (done && li == 0) {
      p.quad_out[s] = q.x;
      p.quad_out[N + s] = q.y;
      p.quad_out[2 * (size_t)N + s] = q.z;
      p.quad_out[3 * (size_t)N + s] = q.w;
      if (p.like_out)
        p.like_out[s] = curr;
    }
    if (done)
      s = kNone;
  }
  if (stats && n_rounds) {  // per-lane counts of the rounds this lane led
    atomicAdd(stats, n_evals);
    atomicAdd(stats + 1, n_rounds);
    atomicAdd(stats + 2, n_acc);
  }
  if (stats && n_warp_rounds) {
    atomicAdd(stats + 4, n_warp_rounds);
    atomicAdd(stats + 5, n_active_lanes);
  }
}

// Dynamic shared memory of a generation kernel with P lanes per sample: one
// staging ring (both directions) per group.
__host__ __device__ constexpr size_t stage_bytes(int P) {
  return sizeof(float4) * (size_t)kWarps * (32 / P) * kGroupStrideF4;
}

// One chunk per launch (the reference's RunHMMOnDevice granularity).  P lanes
// per sample (P/2 evaluations a round); kSub = 2 normalises every 4 sites
// instead of every 8 (for GLs confident enough that 8-site blocks often leave
// the normalisation range).
template <int P, class E, int kSub = 1>
__global__ void __launch_bounds__(kThreads, kMinBlocks) generation_kernel(const GenParams p) {
  __shared__ float4 s_vq[16];
  if (threadIdx.x < 16 && p.vq_table)
    s_vq[threadIdx.x] = p.vq_table[threadIdx.x];
  __syncthreads();
  const OneChunk src{p};
  generation_body<P, E, OneChunk, kSub>(src, p.counter, p.stats, p.error, s_vq);
}

// Many chunks of uneven size in one persistent launch: one queue over all
// samples of all chunks.
template <int P, class E, int kSub = 1>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
    generation_multi_kernel(const MultiParams mp) {
  const ManyChunks src{mp};
  generation_body<P, E, ManyChunks, kSub>(src, mp.counter, mp.stats, mp.error, nullptr);
}

// hmm_work after the generation kernel, over the published final
// quadruples.  Pass 1: blocks of two warps over 16 samples, a lane pair per
// sample and recursion direction in each warp (work_chains_pair), so the
// thousand-odd blocks of a generation spread over every SM.  Pass 2: one
// warp per part of a sample (kSampleWords words) samples its sites.  Chunks
// without hmm_work skip both.
constexpr int kWorkThreads = 32;
constexpr int kChainThreads = 64;
constexpr size_t kChainSmem = 2 * sizeof(ChainTiles);  // dynamic: one per warp

template <class Src>
__device__ __forceinline__ uint4 final_quad(const Src &, const GenParams &p, uint32_t s) {
  const uint32_t N = p.N;
  return make_uint4(p.quad_out[s], p.quad_out[N + s], p.quad_out[2 * (size_t)N + s],
                    p.quad_out[3 * (size_t)N + s]);
}

template <class Src>
__device__ __forceinline__ void chains_body(const Src &src) {
  extern __shared__ __align__(16) unsigned char glp_chain_smem[];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  ChainTiles &s_tiles = reinterpret_cast<ChainTiles *>(glp_chain_smem)[warp];
  // both warps: the block's 16 samples, two lanes each
  const uint32_t g = blockIdx.x * (uint32_t)kPairRows + (lane >> 1);
  const uint32_t total = src.total();
  uint32_t c = 0, s = 0;
  if (g < total)
    src.locate(g, c, s);
  else
    src.locate(total - 1, c, s);  // idle lanes borrow a valid chunk (they skip the work)
  const GenParams &p = src.chunk(c);
  const bool valid = g < total && p.do_work;
  // the warps stage rows together when all their lanes share one chunk (the
  // two warps see the same samples, so they take the same branch and either
  // both or neither reach the barrier in work_chains_pair)
  int same = 0;
  __match_all_sync(0xffffffffu, c, &same);
  if (same) {
    if (__any_sync(0xffffffffu, valid))
      work_chains_pair(p, s, valid ? final_quad(src, p, s) : make_uint4(0, 0, 0, 0), valid,
                       lane, warp == 1, s_tiles);
  } else if (valid && warp == 0 && (lane & 1u) == 0) {
    work_chains(p, s, final_quad(src, p, s));
  }
}

template <class Src>
__device__ __forceinline__ void sample_body(const Src &src) {
  __shared__ float4 s_pcr[kWorkThreads / 32][4];  // the warp's mutation-matrix rows
  __shared__ __align__(16) uint32_t s_u[kWorkThreads / 32][128];  // a span's uniforms
  const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
  // one part of one sample per warp
  const uint64_t g = (uint64_t)blockIdx.x * (blockDim.x >> 5) + wib;
  const uint32_t parts = src.parts();
  if (g >= (uint64_t)src.total() * parts)
    return;
  const uint32_t gs = (uint32_t)(g / parts), part = (uint32_t)(g % parts);
  uint32_t c, s;
  src.locate(gs, c, s);
  const GenParams &p = src.chunk(c);
  if (!p.do_work)
    return;
  const uint32_t w_lo = parts > 1 ? part * kSampleWords : 0u;
  const uint32_t w_hi = parts > 1 ? min(p.wn, w_lo + kSampleWords) : p.wn;
  if (lane < 4)
    s_pcr[wib][lane] = make_float4(p.pc[4 * lane], p.pc[4 * lane + 1], p.pc[4 * lane + 2],
                                   p.pc[4 * lane + 3]);
  __syncwarp();
  work_sample(p, s_pcr[wib], s, final_quad(src, p, s), lane, s_u[wib], w_lo, w_hi);
}

template <int = 0>
__global__ void __launch_bounds__(kChainThreads) work_chains_kernel(const GenParams p) {
  const OneChunk src{p};
  chains_body(src);
}

template <int = 0>
__global__ void __launch_bounds__(kChainThreads) work_chains_multi_kernel(const MultiParams mp) {
  const ManyChunks src{mp};
  chains_body(src);
}

template <int = 0>
__global__ void __launch_bounds__(kWorkThreads) work_sample_kernel(const GenParams p) {
  const OneChunk src{p};
  sample_body(src);
}

template <int = 0>
__global__ void __launch_bounds__(kWorkThreads) work_sample_multi_kernel(const MultiParams mp) {
  const ManyChunks src{mp};
  sample_body(src);
}

}  // namespace glp
