/*
 * glp_oracle.c -- CPU oracle for the GLPhase MH/HMM hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see glp_oracle.h).  Compiled with
 * -ffp-contract=off so that every product and sum is rounded exactly as the
 * reference's scalar code rounds it on a machine without fused multiply-add;
 * the same object therefore gives identical bits on x86-64 and aarch64.
 */
#include "glp_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../glphase_gb300/csrc/glp_rng.h"

#ifdef _OPENMP
#include <omp.h>
#endif

/* impute.hpp:64-66 */
static inline unsigned bit_test(const uint64_t *P, unsigned I) {
  return (unsigned)((P[I >> 6] >> (I & 63)) & 1u);
}

float glpo_norm(void) { return powf(FLT_MIN, 2.0f / 3.0f); }

/* impute.cpp:327-376 */
float glpo_hmm_like_f32(const float *emit_row, const float *tran,
                        const uint64_t *haps, uint32_t wn, uint32_t S,
                        const uint32_t P[4]) {
  const float norm = glpo_norm();
  const uint64_t *f0 = haps + (size_t)P[0] * wn, *f1 = haps + (size_t)P[1] * wn,
                 *m0 = haps + (size_t)P[2] * wn, *m1 = haps + (size_t)P[3] * wn;
  const float *e = emit_row, *t = tran;
  float sum, score = 0;
  float l00 = 0.25f * e[(bit_test(f0, 0) << 1) | bit_test(m0, 0)];
  float l01 = 0.25f * e[(bit_test(f0, 0) << 1) | bit_test(m1, 0)];
  float l10 = 0.25f * e[(bit_test(f1, 0) << 1) | bit_test(m0, 0)];
  float l11 = 0.25f * e[(bit_test(f1, 0) << 1) | bit_test(m1, 0)];
  float b00, b01, b10, b11;
  e += 4;
  t += 3;
  for (unsigned m = 1; m < S; m++, e += 4, t += 3) {
    b00 = l00 * t[0] + (l01 + l10) * t[1] + l11 * t[2];
    b01 = l01 * t[0] + (l00 + l11) * t[1] + l10 * t[2];
    b10 = l10 * t[0] + (l00 + l11) * t[1] + l01 * t[2];
    b11 = l11 * t[0] + (l01 + l10) * t[1] + l00 * t[2];
    l00 = b00 * e[(bit_test(f0, m) << 1) | bit_test(m0, m)];
    l01 = b01 * e[(bit_test(f0, m) << 1) | bit_test(m1, m)];
    l10 = b10 * e[(bit_test(f1, m) << 1) | bit_test(m0, m)];
    l11 = b11 * e[(bit_test(f1, m) << 1) | bit_test(m1, m)];
    if ((sum = l00 + l01 + l10 + l11) < norm) {
      sum = 1.0f / sum;
      score -= logf(sum);
      l00 *= sum;
      l01 *= sum;
      l10 *= sum;
      l11 *= sum;
    }
  }
  return score + logf(l00 + l01 + l10 + l11);
}

/* The recursion of impute.cpp:327-376 in binary64, rescaled whenever the
 * state sum drops below 2^-500: the error yardstick for both FP32 forms. */
double glpo_hmm_like_f64(const float *emit_row, const float *tran,
                         const uint64_t *haps, uint32_t wn, uint32_t S,
                         const uint32_t P[4]) {
  const uint64_t *f0 = haps + (size_t)P[0] * wn, *f1 = haps + (size_t)P[1] * wn,
                 *m0 = haps + (size_t)P[2] * wn, *m1 = haps + (size_t)P[3] * wn;
  const float *e = emit_row, *t = tran;
  double score = 0, sum;
  double l00 = 0.25 * e[(bit_test(f0, 0) << 1) | bit_test(m0, 0)];
  double l01 = 0.25 * e[(bit_test(f0, 0) << 1) | bit_test(m1, 0)];
  double l10 = 0.25 * e[(bit_test(f1, 0) << 1) | bit_test(m0, 0)];
  double l11 = 0.25 * e[(bit_test(f1, 0) << 1) | bit_test(m1, 0)];
  e += 4;
  t += 3;
  for (unsigned m = 1; m < S; m++, e += 4, t += 3) {
    const double t0 = t[0], t1 = t[1], t2 = t[2];
    const double b00 = l00 * t0 + (l01 + l10) * t1 + l11 * t2;
    const double b01 = l01 * t0 + (l00 + l11) * t1 + l10 * t2;
    const double b10 = l10 * t0 + (l00 + l11) * t1 + l01 * t2;
    const double b11 = l11 * t0 + (l01 + l10) * t1 + l00 * t2;
    l00 = b00 * e[(bit_test(f0, m) << 1) | bit_test(m0, m)];
    l01 = b01 * e[(bit_test(f0, m) << 1) | bit_test(m1, m)];
    l10 = b10 * e[(bit_test(f1, m) << 1) | bit_test(m0, m)];
    l11 = b11 * e[(bit_test(f1, m) << 1) | bit_test(m1, m)];
    if ((sum = l00 + l01 + l10 + l11) < 0x1p-500) {
      score += log(sum);
      sum = 1.0 / sum;
      l00 *= sum;
      l01 *= sum;
      l10 *= sum;
      l11 *= sum;
    }
  }
  return score + log(l00 + l01 + l10 + l11);
}

/* hmmLike.cu:12-28: code slot k sits at bits [32-4k-4, 32-4k). */
void glpo_unpack_gl_codebook(uint32_t word, const float *codebook,
                             uint32_t slot, float gl[3]) {
  const uint32_t code = (word >> (32u - 4u * slot - 4u)) & 15u;
  gl[0] = codebook[2 * code];
  gl[1] = codebook[2 * code + 1];
  const float rest = 1 - gl[0] - gl[1];
  gl[2] = rest > 0.0f ? rest : 0.0f;
}

/* hmmLike.cu:39-44 */
void glpo_fill_emit(const float gl[3], const float M[16], float emit[4]) {
  for (unsigned i = 0; i < 4; ++i)
    emit[i] = M[i] * gl[0] + M[i + 4] * gl[1] + M[i + 8] * gl[1] +
              M[i + 12] * gl[2];
}

/* hmmLike.cu:341-344 */
void glpo_mutation_to_device_layout(const float pc[16], float M[16]) {
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j)
      M[i + 4 * j] = pc[i * 4 + j];
}

/* hmmLike.cu:53-142, with logf standing in for __logf. */
float glpo_hmm_like_vq(const uint32_t *packed, uint32_t stride, uint32_t sample,
                       const float *codebook, const float M[16],
                       const float *tran, const uint64_t *haps, uint32_t wn,
                       uint32_t S, const uint32_t P[4]) {
  const float norm = glpo_norm();
  const uint64_t *f0 = haps + (size_t)P[0] * wn, *f1 = haps + (size_t)P[1] * wn,
                 *m0 = haps + (size_t)P[2] * wn, *m1 = haps + (size_t)P[3] * wn;
  float gl[3], emit[4];
  glpo_unpack_gl_codebook(packed[sample], codebook, 0, gl);
  glpo_fill_emit(gl, M, emit);
  float sum, score = 0;
  float l00 = 0.25f * emit[(bit_test(f0, 0) << 1) | bit_test(m0, 0)];
  float l01 = 0.25f * emit[(bit_test(f0, 0) << 1) | bit_test(m1, 0)];
  float l10 = 0.25f * emit[(bit_test(f1, 0) << 1) | bit_test(m0, 0)];
  float l11 = 0.25f * emit[(bit_test(f1, 0) << 1) | bit_test(m1, 0)];
  for (uint32_t site = 1; site < S; ++site) {
    const uint32_t w = packed[sample + (size_t)(site >> 3) * stride];
    glpo_unpack_gl_codebook(w, codebook, site & 7u, gl);
    glpo_fill_emit(gl, M, emit);
    const float *t = tran + (size_t)site * 3;
    const float b00 = l00 * t[0] + (l01 + l10) * t[1] + l11 * t[2];
    const float b01 = l01 * t[0] + (l00 + l11) * t[1] + l10 * t[2];
    const float b10 = l10 * t[0] + (l00 + l11) * t[1] + l01 * t[2];
    const float b11 = l11 * t[0] + (l01 + l10) * t[1] + l00 * t[2];
    l00 = b00 * emit[(bit_test(f0, site) << 1) | bit_test(m0, site)];
    l01 = b01 * emit[(bit_test(f0, site) << 1) | bit_test(m1, site)];
    l10 = b10 * emit[(bit_test(f1, site) << 1) | bit_test(m0, site)];
    l11 = b11 * emit[(bit_test(f1, site) << 1) | bit_test(m1, site)];
    if ((sum = l00 + l01 + l10 + l11) < norm) {
      sum = 1.0f / sum;
      score -= logf(sum);
      l00 *= sum;
      l01 *= sum;
      l10 *= sum;
      l11 *= sum;
    }
  }
  return score + logf(l00 + l01 + l10 + l11);
}

static inline void set_bit(uint64_t *P, unsigned I, unsigned v) {
  const uint64_t mask = (uint64_t)1 << (I & 63);
  if (v)
    P[I >> 6] |= mask;
  else
    P[I >> 6] &= ~mask;
}

/* impute.cpp:380-485 */
void glpo_hmm_work(const float *emit_row, const float *prob_row,
                   const float *tran, const float pc_flat[16],
                   const uint64_t *haps, uint32_t wn, uint32_t S,
                   const uint32_t P[4], float pen, const float *u, uint64_t *ha,
                   uint64_t *hb, float *beta) {
  const float(*pc)[4] = (const float(*)[4])pc_flat;
  const uint64_t *f0 = haps + (size_t)P[0] * wn, *f1 = haps + (size_t)P[1] * wn,
                 *m0 = haps + (size_t)P[2] * wn, *m1 = haps + (size_t)P[3] * wn;
  const float *e = emit_row + (size_t)(S - 1) * 4, *t = tran + (size_t)(S - 1) * 3;
  float *b = beta + (size_t)(S - 1) * 4;
  float sum, l00 = 0, l01 = 0, l10 = 0, l11 = 0, b00, b01, b10, b11;
  b[0] = b[1] = b[2] = b[3] = 1;
  for (unsigned m = S - 1; m; m--, e -= 4, t -= 3) {
    b00 = b[0] * e[(bit_test(f0, m) << 1) | bit_test(m0, m)];
    b01 = b[1] * e[(bit_test(f0, m) << 1) | bit_test(m1, m)];
    b10 = b[2] * e[(bit_test(f1, m) << 1) | bit_test(m0, m)];
    b11 = b[3] * e[(bit_test(f1, m) << 1) | bit_test(m1, m)];
    b -= 4;
    b[0] = b00 * t[0] + (b01 + b10) * t[1] + b11 * t[2];
    b[1] = b01 * t[0] + (b00 + b11) * t[1] + b10 * t[2];
    b[2] = b10 * t[0] + (b00 + b11) * t[1] + b01 * t[2];
    b[3] = b11 * t[0] + (b01 + b10) * t[1] + b00 * t[2];
    sum = 1.0f / (b[0] + b[1] + b[2] + b[3]);
    b[0] *= sum;
    b[1] *= sum;
    b[2] *= sum;
    b[3] *= sum;
  }
  const float *p = prob_row;
  e = emit_row;
  t = tran;
  b = beta;
  for (unsigned m = 0; m < S; m++, e += 4, t += 3, p += 3, b += 4) {
    const unsigned s00 = (bit_test(f0, m) << 1) | bit_test(m0, m);
    const unsigned s01 = (bit_test(f0, m) << 1) | bit_test(m1, m);
    const unsigned s10 = (bit_test(f1, m) << 1) | bit_test(m0, m);
    const unsigned s11 = (bit_test(f1, m) << 1) | bit_test(m1, m);
    if (m) {
      b00 = l00 * t[0] + l01 * t[1] + l10 * t[1] + l11 * t[2];
      b01 = l00 * t[1] + l01 * t[0] + l10 * t[2] + l11 * t[1];
      b10 = l00 * t[1] + l01 * t[2] + l10 * t[0] + l11 * t[1];
      b11 = l00 * t[2] + l01 * t[1] + l10 * t[1] + l11 * t[0];
      l00 = b00 * e[s00];
      l01 = b01 * e[s01];
      l10 = b10 * e[s10];
      l11 = b11 * e[s11];
    } else {
      l00 = 0.25f * e[s00];
      l01 = 0.25f * e[s01];
      l10 = 0.25f * e[s10];
      l11 = 0.25f * e[s11];
    }
    sum = 1.0f / (l00 + l01 + l10 + l11);
    l00 *= sum;
    l01 *= sum;
    l10 *= sum;
    l11 *= sum;
    const float p00 = l00 * b[0], p01 = l01 * b[1], p10 = l10 * b[2],
                p11 = l11 * b[3];
    const float c00 = powf(p[0] * (p00 * pc[s00][0] + p01 * pc[s01][0] +
                                   p10 * pc[s10][0] + p11 * pc[s11][0]),
                           pen);
    const float c01 = powf(p[1] * (p00 * pc[s00][1] + p01 * pc[s01][1] +
                                   p10 * pc[s10][1] + p11 * pc[s11][1]),
                           pen);
    const float c10 = powf(p[1] * (p00 * pc[s00][2] + p01 * pc[s01][2] +
                                   p10 * pc[s10][2] + p11 * pc[s11][2]),
                           pen);
    const float c11 = powf(p[2] * (p00 * pc[s00][3] + p01 * pc[s01][3] +
                                   p10 * pc[s10][3] + p11 * pc[s11][3]),
                           pen);
    /* impute.cpp:470: a double uniform times a float sum, stored in float. */
    sum = (float)((double)u[m] * (double)(c00 + c01 + c10 + c11));
    if (sum < c00) {
      set_bit(ha, m, 0);
      set_bit(hb, m, 0);
    } else if (sum < c00 + c01) {
      set_bit(ha, m, 0);
      set_bit(hb, m, 1);
    } else if (sum < c00 + c01 + c10) {
      set_bit(ha, m, 1);
      set_bit(hb, m, 0);
    } else {
      set_bit(ha, m, 1);
      set_bit(hb, m, 1);
    }
  }
}

/* MHSampler.hpp:81-96 (MH variant): accept a better or equal proposal, else
 * accept when u < exp((proposal - current) * pen), all in binary64. */
int glpo_mh_accept(double proposal, double current, double pen, double u) {
  if (proposal >= current)
    return 1;
  return u < exp((proposal - current) * pen) ? 1 : 0;
}

static float like_of(const glpo_problem *pb, uint32_t sample,
                     const uint32_t P[4]) {
  if (pb->emit_mode == GLPO_EMIT_VQ) {
    float M[16];
    glpo_mutation_to_device_layout(pb->pc, M);
    return glpo_hmm_like_vq(pb->packed, pb->N, sample, pb->codebook, M,
                            pb->tran, pb->haps, pb->wn, pb->S, P);
  }
  return glpo_hmm_like_f32(pb->emit + (size_t)sample * pb->S * 4, pb->tran,
                           pb->haps, pb->wn, pb->S, P);
}

static void mh_draw(const glpo_problem *pb, const glpo_trace *tr,
                    uint32_t sample, uint32_t cycle, uint32_t *slot,
                    double *u) {
  if (tr->slot) {
    *slot = tr->slot[(size_t)sample * pb->C + cycle] & 3u;
    *u = tr->u_mh[(size_t)sample * pb->C + cycle];
  } else {
    glp_mh_draw(tr->seed, tr->generation, sample, cycle, slot, u);
  }
}

static void work_uniforms(const glpo_problem *pb, const glpo_trace *tr,
                          uint32_t sample, float *u) {
  if (tr->u_work) {
    memcpy(u, tr->u_work + (size_t)sample * pb->S, sizeof(float) * pb->S);
  } else {
    for (uint32_t m = 0; m < pb->S; ++m)
      u[m] = glp_work_uniform(tr->seed, tr->generation, sample, m);
  }
}

/* insti.cpp:1478-1551 with the CUDA path's pre-drawn proposals
 * (hmmLike.cpp:90-102, hmmLike.cu:185-207) and MHSampler's accept. */
double glpo_solve_sample(const glpo_problem *pb, const glpo_trace *tr,
                         uint32_t sample, const uint32_t *quad_in,
                         const uint32_t *props, float pen,
                         uint32_t quad_out[4], float *like_trace,
                         uint8_t *accept, int do_work, uint64_t *ha,
                         uint64_t *hb, float *beta_scratch) {
  const uint32_t N = pb->N;
  uint32_t q[4];
  for (int i = 0; i < 4; ++i)
    q[i] = quad_in[sample + (size_t)N * i];
  double curr = like_of(pb, sample, q);
  if (like_trace)
    like_trace[0] = (float)curr;
  for (uint32_t c = 0; c < pb->C; ++c) {
    uint32_t r;
    double u;
    mh_draw(pb, tr, sample, c, &r, &u);
    const uint32_t old = q[r];
    q[r] = props[(size_t)c * N + sample];
    const double prop = like_of(pb, sample, q);
    if (like_trace)
      like_trace[c + 1] = (float)prop;
    const int acc = glpo_mh_accept(prop, curr, pen, u);
    if (accept)
      accept[c] = (uint8_t)acc;
    if (acc)
      curr = prop;
    else
      q[r] = old;
  }
  for (int i = 0; i < 4; ++i)
    quad_out[i] = q[i];
  if (do_work) {
    float *u = (float *)malloc(sizeof(float) * pb->S);
    if (u) {
      work_uniforms(pb, tr, sample, u);
      glpo_hmm_work(pb->emit + (size_t)sample * pb->S * 4,
                    pb->prob + (size_t)sample * pb->S * 3, pb->tran, pb->pc,
                    pb->haps, pb->wn, pb->S, q, pen, u, ha, hb, beta_scratch);
      free(u);
    }
  }
  return curr;
}

int glpo_generation(const glpo_problem *pb, const glpo_trace *tr,
                    const uint32_t *quad_in, const uint32_t *props, float pen,
                    uint32_t first, uint32_t last, int do_work,
                    uint32_t *quad_out, uint64_t *hnew, double *like_out,
                    int nthreads) {
  int failed = 0;
  const uint32_t N = pb->N, wn = pb->wn;
#ifdef _OPENMP
  if (nthreads <= 0)
    nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads) reduction(| : failed)
#endif
  {
    float *beta = (float *)malloc(sizeof(float) * 4 * (size_t)pb->S);
    if (!beta) {
      failed = 1;
    } else {
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
      for (long s = (long)first; s < (long)last; ++s) {
        uint32_t q[4];
        uint64_t *ha = hnew + (size_t)2 * s * wn, *hb = ha + wn;
        if (do_work) {
          memset(ha, 0, sizeof(uint64_t) * wn);
          memset(hb, 0, sizeof(uint64_t) * wn);
        }
        const double curr =
            glpo_solve_sample(pb, tr, (uint32_t)s, quad_in, props, pen, q, NULL,
                              NULL, do_work, ha, hb, beta);
        for (int i = 0; i < 4; ++i)
          quad_out[s + (size_t)N * i] = q[i];
        if (like_out)
          like_out[s] = curr;
      }
      free(beta);
    }
  }
  (void)nthreads;
  return failed ? -1 : 0;
}

void glpo_replay_sample(const glpo_problem *pb, const glpo_trace *tr,
                        uint32_t sample, const uint32_t *quad_in,
                        const uint32_t *props, float pen,
                        const uint8_t *gpu_accept, float *like32,
                        double *like64, uint8_t *own_accept,
                        uint32_t quad_out[4]) {
  const uint32_t N = pb->N;
  const float *er = pb->emit ? pb->emit + (size_t)sample * pb->S * 4 : NULL;
  uint32_t q[4];
  for (int i = 0; i < 4; ++i)
    q[i] = quad_in[sample + (size_t)N * i];
  double curr = like_of(pb, sample, q);
  like32[0] = (float)curr;
  if (like64)
    like64[0] = er ? glpo_hmm_like_f64(er, pb->tran, pb->haps, pb->wn, pb->S, q)
                   : 0.0;
  for (uint32_t c = 0; c < pb->C; ++c) {
    uint32_t r;
    double u;
    mh_draw(pb, tr, sample, c, &r, &u);
    const uint32_t old = q[r];
    q[r] = props[(size_t)c * N + sample];
    const double prop = like_of(pb, sample, q);
    like32[c + 1] = (float)prop;
    if (like64)
      like64[c + 1] =
          er ? glpo_hmm_like_f64(er, pb->tran, pb->haps, pb->wn, pb->S, q) : 0.0;
    own_accept[c] = (uint8_t)glpo_mh_accept(prop, curr, pen, u);
    if (gpu_accept[c])
      curr = prop;
    else
      q[r] = old;
  }
  for (int i = 0; i < 4; ++i)
    quad_out[i] = q[i];
}

void glpo_mh_draws(uint64_t seed, uint32_t generation, uint32_t sample, uint32_t C,
                   uint8_t *slot, double *u) {
  for (uint32_t c = 0; c < C; ++c) {
    uint32_t r;
    glp_mh_draw(seed, generation, sample, c, &r, &u[c]);
    slot[c] = (uint8_t)r;
  }
}

void glpo_work_uniforms(uint64_t seed, uint32_t generation, uint32_t sample, uint32_t S,
                        float *u) {
  for (uint32_t m = 0; m < S; ++m)
    u[m] = glp_work_uniform(seed, generation, sample, m);
}

/* Insti::solve's kick-start (insti.cpp:1505-1511): the first proposal comes
 * from Sampler::SampleHap(I, true) (sampler.cpp:12-27), which redraws until
 * the index is a panel haplotype (>= 2N).  With counter-based draws: a
 * uniform pick among the neighbour list's panel entries, in list order, or
 * uniform over [2N, H) without a list or panel entries. */
static uint32_t kick_proposal(uint64_t seed, uint32_t generation, uint32_t s, uint32_t N,
                              uint32_t H, const uint32_t *nbr, uint32_t klen) {
  const glp_u32x4 x = glp_draw(seed, generation, s, 0, GLP_TAG_PROP);
  const uint32_t ref_lo = 2 * N;
  if (nbr) {
    uint32_t panel[1024], n = 0;
    for (uint32_t k = 0; k < klen && n < 1024; ++k)
      if (nbr[(size_t)s * klen + k] >= ref_lo)
        panel[n++] = nbr[(size_t)s * klen + k];
    if (n)
      return panel[glp_below(x.v[2], x.v[3], n)];
  }
  return glp_uniform_hap(x, s, ref_lo, H);
}

void glpo_sample_surrogates(uint64_t seed, uint32_t generation, uint32_t N, uint32_t C,
                            uint32_t lo, uint32_t hi, const uint32_t *nbr, uint32_t klen,
                            int kick_first, uint32_t H, uint32_t *quad, uint32_t *props) {
  for (uint32_t s = 0; s < N; ++s) {
    for (uint32_t j = 0; j < 4; ++j)
      quad[(size_t)j * N + s] =
          glp_surrogate(seed, generation, s, j, GLP_TAG_INIT, lo, hi, nbr, klen);
    for (uint32_t c = 0; c < C; ++c)
      props[(size_t)c * N + s] =
          (kick_first && c == 0)
              ? kick_proposal(seed, generation, s, N, H, nbr, klen)
              : glp_surrogate(seed, generation, s, c, GLP_TAG_PROP, lo, hi, nbr, klen);
  }
}

/* kNN.cpp:216-257 */
void glpo_common_sites(const uint64_t *haps, uint32_t H, uint32_t wn, uint32_t S,
                       double lb, double ub, int use_maf, uint64_t *mask) {
  memset(mask, 0, sizeof(uint64_t) * wn);
  for (uint32_t m = 0; m < S; ++m) {
    uint32_t alt = 0;
    for (uint32_t h = 0; h < H; ++h)
      alt += bit_test(haps + (size_t)h * wn, m);
    double af = (double)alt / H;
    if (use_maf)
      af = fabs(fabs(af - 0.5) - 0.5);
    if (af >= lb && af <= ub)
      mask[m >> 6] |= (uint64_t)1 << (m & 63);
  }
}

typedef struct {
  uint32_t d, idx;
} knn_pair;

static int knn_cmp(const void *a, const void *b) {
  const knn_pair *x = (const knn_pair *)a, *y = (const knn_pair *)b;
  if (x->d != y->d)
    return x->d < y->d ? -1 : 1;
  return x->idx < y->idx ? -1 : (x->idx > y->idx ? 1 : 0);
}

static uint32_t hamming_masked(const uint64_t *a, const uint64_t *b,
                               const uint64_t *mask, uint32_t wn) {
  uint32_t d = 0;
  for (uint32_t w = 0; w < wn; ++w)
    d += (uint32_t)__builtin_popcountll((a[w] ^ b[w]) & mask[w]);
  return d;
}

/* Haplotype::MaxTractLen (haplotype.cpp:62-90) over the common sites of
   KNN::CutDownHaps (kNN.cpp:216-257): the longest run of consecutive common
   sites at which a and b agree; sites outside the mask are not part of the
   cut-down haplotypes, so they neither extend nor break a run. */
uint32_t glpo_max_tract(const uint64_t *a, const uint64_t *b, const uint64_t *mask,
                        uint32_t wn) {
  uint32_t best = 0, run = 0;
  for (uint32_t w = 0; w < wn; ++w)
    for (uint32_t j = 0; j < 64; ++j) {
      if (!((mask[w] >> j) & 1u))
        continue;
      if (((a[w] ^ b[w]) >> j) & 1u) {
        if (run > best)
          best = run;
        run = 0;
      } else {
        ++run;
      }
    }
  return run > best ? run : best;
}

/* kNN.cpp:123-206 with the Hamming metric */
int glpo_knn(const uint64_t *haps, uint32_t H, uint32_t wn, const uint64_t *mask,
             uint32_t K, uint32_t *neighbors) {
  return glpo_knn_metric(haps, H, wn, mask, K, 0, neighbors);
}

/* kNN.cpp:123-206; metric 0: Hamming distance (kNN.cpp:151-153), 1: the
   number of common sites minus the longest shared tract (kNN.cpp:157-164) */
int glpo_knn_metric(const uint64_t *haps, uint32_t H, uint32_t wn, const uint64_t *mask,
                    uint32_t K, int metric, uint32_t *neighbors) {
  uint32_t ncommon = 0;
  for (uint32_t w = 0; w < wn; ++w)
    ncommon += (uint32_t)__builtin_popcountll(mask[w]);
  const uint32_t half = (K + 1) / 2, len = 2 * half, ns = H / 2;
  if (H < 2 || H - 2 < len)
    return -1;
  int failed = 0;
#ifdef _OPENMP
#pragma omp parallel reduction(| : failed)
#endif
  {
    knn_pair *da = (knn_pair *)malloc(sizeof(knn_pair) * H);
    knn_pair *db = (knn_pair *)malloc(sizeof(knn_pair) * H);
    uint8_t *taken = (uint8_t *)malloc(H);
    if (!da || !db || !taken) {
      failed = 1;
    } else {
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
      for (long s = 0; s < (long)ns; ++s) {
        const uint64_t *ha = haps + (size_t)2 * s * wn, *hb = ha + wn;
        uint32_t n = 0;
        for (uint32_t h = 0; h < H; ++h) {
          if ((h >> 1) == (uint32_t)s)
            continue;
          const uint64_t *o = haps + (size_t)h * wn;
          if (metric == 1) {
            da[n].d = ncommon - glpo_max_tract(ha, o, mask, wn);
            db[n].d = ncommon - glpo_max_tract(hb, o, mask, wn);
          } else {
            da[n].d = hamming_masked(ha, o, mask, wn);
            db[n].d = hamming_masked(hb, o, mask, wn);
          }
          da[n].idx = h;
          db[n].idx = h;
          ++n;
        }
        qsort(da, n, sizeof(knn_pair), knn_cmp);
        qsort(db, n, sizeof(knn_pair), knn_cmp);
        memset(taken, 0, H);
        uint32_t *out = neighbors + (size_t)s * len;
        for (uint32_t i = 0; i < half; ++i) {
          out[2 * i] = da[i].idx;
          taken[da[i].idx] = 1;
        }
        uint32_t j = 0;
        for (uint32_t i = 0; i < half; ++i) {
          while (taken[db[j].idx])
            ++j;
          out[2 * i + 1] = db[j].idx;
          taken[db[j].idx] = 1;
          ++j;
        }
      }
    }
    free(da);
    free(db);
    free(taken);
  }
  return failed ? -1 : 0;
}

/* impute.cpp:564-595 */
void glpo_replace(const uint64_t *haps, uint32_t wn, uint32_t S,
                  uint32_t sample, uint32_t *hsum) {
  const uint64_t *oa = haps + (size_t)sample * 2 * wn, *ob = oa + wn;
  uint32_t *ha = hsum + (size_t)sample * 2 * S, *hb = ha + S;
  uint32_t sis = 0, tra = 0;
  for (uint32_t m = 0; m < S; m++) {
    if (bit_test(oa, m)) {
      sis += ha[m];
      tra += hb[m];
    }
    if (bit_test(ob, m)) {
      sis += hb[m];
      tra += ha[m];
    }
  }
  if (sis > tra)
    for (uint32_t m = 0; m < S; m++) {
      ha[m] += bit_test(oa, m);
      hb[m] += bit_test(ob, m);
    }
  else
    for (uint32_t m = 0; m < S; m++) {
      ha[m] += bit_test(ob, m);
      hb[m] += bit_test(oa, m);
    }
}

/* impute.cpp:599-613 */
void glpo_result(const uint32_t *hsum, uint32_t N, uint32_t S, uint32_t sn,
                 float *prob_out) {
  const float norm = (float)(1.0 / sn);
  const uint32_t hn = 2 * N;
  for (uint32_t m = 0; m < S; m++) {
    float *p = prob_out + (size_t)m * hn;
    for (uint32_t i = 0; i < N; i++, p += 2) {
      p[0] = hsum[(size_t)i * 2 * S + m] * norm;
      p[1] = hsum[(size_t)(i * 2 + 1) * S + m] * norm;
    }
  }
}
