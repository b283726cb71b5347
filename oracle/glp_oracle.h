/*
 * glp_oracle.h -- CPU oracle for the GLPhase MH/HMM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library and its
 * host-side mirror) may call into this file; only the tests, the smoke check
 * and the CPU-baseline leg of bench.py use it, and only as the checker or as
 * the timed CPU reference.
 *
 * Every function restates one piece of the reference's arithmetic in plain C,
 * in the reference's operation order, and cites the file:line it follows
 * (paths relative to the reference project root).  The restatement is pinned
 * two ways: (1) against the reference's own impute.cpp compiled from source
 * (oracle/_ref, built by oracle/Makefile where the reference tree exists),
 * bit-for-bit on hmm_like and hmm_work; (2) against the known-answer vectors
 * of the reference's unit tests (codebook decode, FillEmit, mutation-matrix
 * transpose, GL packing, MH semantics, planted parents).
 *
 * Layouts (all row-major, all shared with the CUDA path):
 *   haps   uint64 [H][wn]     site m -> word m>>6, bit m&63 (impute.hpp:53-66)
 *   emit   float  [N][S][4]   (insti.cpp:1226-1227, 1376-1378)
 *   prob   float  [N][S][3]   (homRef, het, homAlt) after initialize
 *                             (insti.cpp:1345-1350, 1382)
 *   tran   float  [S][3]      row 0 unused (insti.cpp:1277-1300)
 *   pc     float  [4][4]      pc[i][j] (insti.cpp:1307-1315)
 *   quad   uint32 [4][N]      hapIdxs layout of RunHMMOnDevice (hmmLike.cpp:81)
 *   props  uint32 [C][N]      extraPropHaps layout (hmmLike.cpp:86)
 *   packed uint32 [ceil(S/8)][N] 4-bit VQ codes, MSB-first (glPack.cpp:129-156)
 *   codebook float [16][2]    (RR, Het) pairs (hmmLike.cu:369-383)
 */
#ifndef GLP_ORACLE_H
#define GLP_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* norm = powf(FLT_MIN, 2/3) (impute.cpp:11-13, hmmLike.cu:233). */
float glpo_norm(void);

/* Impute::hmm_like, FP32 in the reference's op order (impute.cpp:327-376). */
float glpo_hmm_like_f32(const float *emit_row, const float *tran,
                        const uint64_t *haps, uint32_t wn, uint32_t S,
                        const uint32_t P[4]);

/* The same recursion in FP64 with per-site rescaling: the error yardstick. */
double glpo_hmm_like_f64(const float *emit_row, const float *tran,
                         const uint64_t *haps, uint32_t wn, uint32_t S,
                         const uint32_t P[4]);

/* UnpackGLsWithCodeBook (hmmLike.cu:12-28): code slot k of a packed word. */
void glpo_unpack_gl_codebook(uint32_t word, const float *codebook,
                             uint32_t slot, float gl[3]);

/* FillEmit (hmmLike.cu:39-44) with M[i + 4j] = pc[i][j] (hmmLike.cu:341-344). */
void glpo_fill_emit(const float gl[3], const float M[16], float emit[4]);

/* Mutation matrix transpose of CopyMutationMatToDevice (hmmLike.cu:339-344). */
void glpo_mutation_to_device_layout(const float pc[16], float M[16]);

/* Device hmmLike with VQ-decoded emissions (hmmLike.cu:53-142). */
float glpo_hmm_like_vq(const uint32_t *packed, uint32_t stride, uint32_t sample,
                       const float *codebook, const float M[16],
                       const float *tran, const uint64_t *haps, uint32_t wn,
                       uint32_t S, const uint32_t P[4]);

/* Impute::hmm_work (impute.cpp:380-485): backward beta, forward sampling.
 * u[m] is the uniform of site m; beta is scratch [S][4]; ha/hb are the two
 * output rows [wn] (bits of sites >= S are left at zero). */
void glpo_hmm_work(const float *emit_row, const float *prob_row,
                   const float *tran, const float pc[16], const uint64_t *haps,
                   uint32_t wn, uint32_t S, const uint32_t P[4], float pen,
                   const float *u, uint64_t *ha, uint64_t *hb, float *beta);

/* MHSampler<T>::SampleHap accept rule, MH variant (MHSampler.hpp:81-96). */
int glpo_mh_accept(double proposal, double current, double pen, double u);

/* Emission sources of the MH likelihood. */
#define GLPO_EMIT_FLOAT 0 /* emit [N][S][4], the CPU path */
#define GLPO_EMIT_VQ 1    /* packed codes + codebook, the reference GPU path */

typedef struct glpo_problem {
  uint32_t N, S, C, H, wn;
  const uint64_t *haps; /* [H][wn] */
  const float *emit;    /* [N][S][4] */
  const float *prob;    /* [N][S][3] */
  const float *tran;    /* [S][3] */
  const float *pc;      /* [16] row-major pc[i][j] */
  const uint32_t *packed;   /* [ceil(S/8)][N] or NULL */
  const float *codebook;    /* [16][2] or NULL */
  int emit_mode;
} glpo_problem;

typedef struct glpo_trace {
  /* Either explicit per-draw arrays, or (when all are NULL) the Philox
   * streams of glp_rng.h keyed by (seed, generation). */
  const uint8_t *slot;  /* [N][C] */
  const double *u_mh;   /* [N][C] */
  const float *u_work;  /* [N][S] */
  uint64_t seed;
  uint32_t generation;
} glpo_trace;

/* One sample of one generation: the MH chain of Insti::solve restricted to
 * the CUDA path's semantics (proposals pre-drawn, hmmLike.cpp:90-102;
 * accept of MHSampler.hpp:81-96 with pen), then hmm_work.  like_trace (C+1,
 * nullable) receives every evaluated log-likelihood, accept (C, nullable) the
 * decisions.  Writes quad_out[4], rows ha/hb when do_work, returns curr. */
double glpo_solve_sample(const glpo_problem *pb, const glpo_trace *tr,
                         uint32_t sample, const uint32_t *quad_in /*[4][N]*/,
                         const uint32_t *props /*[C][N]*/, float pen,
                         uint32_t quad_out[4], float *like_trace,
                         uint8_t *accept, int do_work, uint64_t *ha,
                         uint64_t *hb, float *beta_scratch);

/* A whole generation over samples [first, last), OpenMP over samples with
 * nthreads threads (0 = all).  quad_out [4][N], hnew [H][wn] (only rows of
 * processed samples written), like_out [N] (nullable).  This is the timed
 * multi-core CPU baseline.  Returns 0, or -1 if scratch could not be
 * allocated. */
int glpo_generation(const glpo_problem *pb, const glpo_trace *tr,
                    const uint32_t *quad_in, const uint32_t *props, float pen,
                    uint32_t first, uint32_t last, int do_work,
                    uint32_t *quad_out, uint64_t *hnew, double *like_out,
                    int nthreads);

/* Replay a GPU chain: follow the given accept decisions, evaluate every
 * proposal with the FP32 reference-order likelihood (like32) and the FP64
 * yardstick (like64), and report the oracle's own decision (own_accept) for
 * each cycle under the same uniforms. */
void glpo_replay_sample(const glpo_problem *pb, const glpo_trace *tr,
                        uint32_t sample, const uint32_t *quad_in,
                        const uint32_t *props, float pen,
                        const uint8_t *gpu_accept /*[C]*/, float *like32,
                        double *like64, uint8_t *own_accept,
                        uint32_t quad_out[4]);

/* The counter-based draws of glp_rng.h for one sample, so that the checker
 * can replay a generation that ran on the Philox streams. */
void glpo_mh_draws(uint64_t seed, uint32_t generation, uint32_t sample, uint32_t C,
                   uint8_t *slot, double *u);
void glpo_work_uniforms(uint64_t seed, uint32_t generation, uint32_t sample, uint32_t S,
                        float *u);

/* The surrogates a generation draws on the device (glp_surrogate of
 * glp_rng.h), materialised: quad [4][N] and props [C][N]; nbr [N][klen] or
 * NULL for uniform over [lo, hi) minus the sample's own pair. */
void glpo_sample_surrogates(uint64_t seed, uint32_t generation, uint32_t N, uint32_t C,
                            uint32_t lo, uint32_t hi, const uint32_t *nbr, uint32_t klen,
                            int kick_first, uint32_t H, uint32_t *quad, uint32_t *props);

/* KNN::CalculateVarAfs + CutDownHaps (kNN.cpp:216-257): bit m of mask is
 * set when site m's alt-allele frequency over all H haplotypes (or its minor
 * allele frequency) lies in [lb, ub].  mask is [wn] uint64. */
void glpo_common_sites(const uint64_t *haps, uint32_t H, uint32_t wn, uint32_t S,
                       double lb, double ub, int use_maf, uint64_t *mask);

/* KNN::ClusterHaps (kNN.cpp:123-206), Hamming metric over the masked sites:
 * for each of the H/2 samples, the ceil(K/2) haplotypes nearest to its first
 * haplotype, then the ceil(K/2) nearest to its second that are not already
 * chosen, interleaved (first, second, first, ...).  Ties are ordered by
 * haplotype index (the reference's std::sort is unstable, kNN.cpp:172-173).
 * neighbors is [H/2][2*ceil(K/2)].  Returns 0, or -1 when H - 2 < the list
 * length. */
int glpo_knn(const uint64_t *haps, uint32_t H, uint32_t wn, const uint64_t *mask,
             uint32_t K, uint32_t *neighbors);
int glpo_knn_metric(const uint64_t *haps, uint32_t H, uint32_t wn, const uint64_t *mask,
                    uint32_t K, int metric, uint32_t *neighbors);
uint32_t glpo_max_tract(const uint64_t *a, const uint64_t *b, const uint64_t *mask,
                        uint32_t wn);

/* Impute::replace (impute.cpp:564-595): per-site allele tallies, hsum is
 * [2N][S] uint32. */
void glpo_replace(const uint64_t *haps, uint32_t wn, uint32_t S,
                  uint32_t sample, uint32_t *hsum);

/* Impute::result (impute.cpp:599-613): prob_out [S][2N]. */
void glpo_result(const uint32_t *hsum, uint32_t N, uint32_t S, uint32_t sn,
                 float *prob_out);

#ifdef __cplusplus
}
#endif
#endif
