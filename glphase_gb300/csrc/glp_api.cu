// glp_api.cu -- host side of the C ABI declared in include/glphase_gpu.h.
//
// A context owns a device, a stream and the per-generation work buffers.  A
// problem (one phasing chunk) owns its device-resident model inputs:
// transition table, mutation matrix, emissions or VQ codes, genotype
// probabilities and the hmm_work scratch.  The context's own model (the
// glp_set_* calls that replace HMMLikeCUDA's Copy*ToDevice) is its default
// problem.  Every entry point returns a status code; nothing exits, throws
// across the boundary or resets the device (the reference's HMMLikeCUDA calls
// exit(EXIT_FAILURE) on CUDA errors, src/hmmLike.cu:240-300, and
// cudaDeviceReset in Cleanup, src/hmmLike.cu:396).
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/glphase_gpu.h"
#include "glp_server_core.h"
#include "glp_knn.cuh"
#include "glp_launch.h"
#include "glp_tally.cuh"
#include "glp_vq.cuh"

namespace glp {

// Moves every chunk of a prepared batch to its next generation in place, so
// a captured CUDA graph can replay generation after generation: the new
// haplotypes become the current ones (Insti::cudaSolve's swap,
// insti.cpp:1455), the generation counter advances, the annealing penalty
// follows Insti::estimate (insti.cpp:1670-1671, binary32), and the
// kick-start restriction of the surrogates ends after generation 0.
__global__ void advance_kernel(GenParams *__restrict__ table, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  GenParams &p = table[i];
  if (p.do_work) {
    uint64_t *cur = const_cast<uint64_t *>(p.haps);
    p.haps = p.hnew;
    p.hnew = cur;
  }
  p.generation += 1;
  if (p.burnin) {
    const float x = fminf(__fdiv_rn((float)p.generation + 1.0f, (float)p.burnin), 1.0f);
    p.pen = x * x;
  }
  if (p.kick) {
    p.samp_lo = 0;
    p.kick = 0;
  }
}

}  // namespace glp

struct glp_problem {
  glp_ctx *ctx = nullptr;
  uint32_t S = 0;  // sites of tran
  float4 *d_tran4 = nullptr;
  float pc[16] = {0};
  bool have_pc = false;
  float codebook[32] = {0};
  bool have_codebook = false;
  float4 *d_vq = nullptr;  // [16] emission per VQ code
  uint32_t *d_packed = nullptr;
  size_t packed_words = 0;
  float4 *d_emit = nullptr;
  float *d_prob = nullptr;
  uint32_t eN = 0, eS = 0;  // shape of emit/prob
  bool borrowed = false;     // emit/prob belong to the caller
  float4 *d_beta = nullptr;  // hmm_work scratch [N][S]
  size_t beta_cap = 0;
};

struct glp_ctx {
  int device = 0;
  int sms = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  std::string err;
  glp_problem def;  // the model set by glp_set_* (HMMLikeCUDA semantics)
  // work buffers
  uint32_t *d_counter = nullptr;
  unsigned long long *d_stats = nullptr;
  int *d_error = nullptr;
  glp::GenParams *d_table = nullptr;  // batch descriptors
  uint32_t *d_offsets = nullptr;
  size_t table_cap = 0, offsets_cap = 0;
  glp::GenParams *h_table = nullptr;  // pinned staging
  uint32_t *h_offsets = nullptr;
  size_t h_cap = 0;
  // staging for the host-pointer entry points
  uint64_t *d_haps = nullptr, *d_hnew = nullptr;
  size_t haps_cap = 0, hnew_cap = 0;
  uint32_t *d_quad = nullptr, *d_quad_out = nullptr, *d_props = nullptr, *d_nbr = nullptr;
  size_t quad_cap = 0, quad_out_cap = 0, props_cap = 0, nbr_cap = 0;
  uint64_t *d_mask = nullptr;  // kNN common-site mask
  size_t mask_cap = 0;
  uint16_t *d_knn_dist = nullptr;  // kNN distances of a chunk of samples [2 n][H]
  size_t knn_dist_cap = 0;
  uint8_t *d_tr_slot = nullptr, *d_acc = nullptr;
  double *d_tr_u = nullptr, *d_like = nullptr, *d_evals = nullptr;
  float *d_tr_work = nullptr;
  size_t tr_slot_cap = 0, acc_cap = 0, tr_u_cap = 0, like_cap = 0, evals_cap = 0,
         tr_work_cap = 0;
  // tuning and statistics
  uint32_t lanes = 0;  // 0 = automatic
  uint32_t evals = 0;  // evaluations per lane and round, 0 = automatic
  // sites per normalisation block (8 or 4), 0 = automatic: 8 until a
  // generation recomputes more than 0.1 % of its evaluations site by site,
  // then 4 for the rest of the context's life
  uint32_t block_sites = 0;
  int knn_metric = GLP_KNN_HAMMING;  // glp_set_knn_metric
  bool short_blocks = false;
  // resident threads per lane width (1 .. 32), per [multi-chunk][VQ] kernel
  double resident[2][2][6] = {};
  bool resident_known[2][2] = {};
  uint32_t lanes_used = 4;
  double last_accept = -1.0;  // acceptance rate of the last generation
  // annealing penalty of the last launch, and of the generation last_accept
  // was measured on: the acceptance rate only predicts a generation run at
  // the same penalty (it falls several-fold while the penalty ramps up)
  float launch_pen = -1.0f, accept_pen = -2.0f;
  uint64_t last_chain_cycles = 0;
  unsigned long long last_stats[glp::kStats] = {};
  // device-time record of the last kTimed generations launched from the host
  // (glp_run_generation, glp_run_batch): events before the generation kernel,
  // after it and after the hmm_work kernels, on the launching stream
  static constexpr uint32_t kTimed = 64;
  cudaEvent_t ev[kTimed][3] = {};
  uint64_t ev_count = 0;
};

namespace {

int fail(glp_ctx *c, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (c)
    c->err = buf;
  return code;
}

#define GLP_CUDA(c, call)                                                                   \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      return fail((c), e_ == cudaErrorMemoryAllocation ? GLP_ERR_NOMEM : GLP_ERR_CUDA,     \
                  "%s failed: %s", #call, cudaGetErrorString(e_));                          \
  } while (0)

template <class T>
int ensure(glp_ctx *c, T *&ptr, size_t &cap, size_t count) {
  if (count <= cap && ptr)
    return GLP_OK;
  if (ptr)
    cudaFree(ptr);
  ptr = nullptr;
  cap = 0;
  GLP_CUDA(c, cudaMalloc((void **)&ptr, std::max<size_t>(count, 1) * sizeof(T)));
  cap = count;
  return GLP_OK;
}

template <class T>
void release(T *&p) {
  if (p)
    cudaFree(p);
  p = nullptr;
}

void drop_emission(glp_problem *pb) {
  if (pb->borrowed) {
    pb->d_emit = nullptr;
    pb->d_prob = nullptr;
  } else {
    release(pb->d_emit);
    release(pb->d_prob);
  }
  pb->borrowed = false;
  pb->eN = pb->eS = 0;
}

void release_problem(glp_problem *pb) {
  release(pb->d_tran4);
  release(pb->d_vq);
  release(pb->d_packed);
  drop_emission(pb);
  release(pb->d_beta);
  pb->S = pb->eN = pb->eS = 0;
  pb->packed_words = pb->beta_cap = 0;
}

int check_ctx(glp_ctx *c) {
  if (!c)
    return GLP_ERR_ARG;
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess)
    return fail(c, GLP_ERR_CUDA, "cudaSetDevice(%d): %s", c->device, cudaGetErrorString(e));
  return GLP_OK;
}

// The model set-up calls overwrite device buffers with synchronous copies,
// which are not ordered with the context's (non-blocking) stream: they first
// wait for the work already enqueued there, which reads the old contents.
int quiesce(glp_ctx *c) {
  GLP_CUDA(c, cudaStreamSynchronize(c->stream));
  return GLP_OK;
}

// FillEmit of every codebook entry (hmmLike.cu:12-44): G = (cb0, cb1,
// max(1 - cb0 - cb1, 0)), emit[i] = pc[i][0] G0 + pc[i][1] G1 + pc[i][2] G1
// + pc[i][3] G2.  Host code is built with -ffp-contract=off, so each term is
// rounded exactly as in the CPU reference.
int upload_vq_table(glp_problem *pb) {
  glp_ctx *c = pb->ctx;
  if (!pb->have_pc || !pb->have_codebook)
    return GLP_OK;
  float4 tab[16];
  for (int code = 0; code < 16; ++code) {
    const float g0 = pb->codebook[2 * code], g1 = pb->codebook[2 * code + 1];
    const float rest = 1 - g0 - g1;
    const float g2 = rest > 0.0f ? rest : 0.0f;
    float em[4];
    for (int i = 0; i < 4; ++i) {
      const float a = pb->pc[i * 4 + 0] * g0;
      const float b = pb->pc[i * 4 + 1] * g1;
      const float d = pb->pc[i * 4 + 2] * g1;
      const float f = pb->pc[i * 4 + 3] * g2;
      em[i] = ((a + b) + d) + f;
    }
    tab[code] = make_float4(em[0], em[1], em[2], em[3]);
  }
  if (!pb->d_vq)
    GLP_CUDA(c, cudaMalloc((void **)&pb->d_vq, sizeof(tab)));
  else if (int rc = quiesce(c))
    return rc;
  GLP_CUDA(c, cudaMemcpy(pb->d_vq, tab, sizeof(tab), cudaMemcpyHostToDevice));
  return GLP_OK;
}

int set_tran(glp_problem *pb, const float *tran, uint32_t S) {
  glp_ctx *c = pb->ctx;
  if (!tran || S == 0)
    return fail(c, GLP_ERR_ARG, "tran must be non-null with num_sites > 0");
  // rows 0 and S are the identity: row 0 is unused by the reference's
  // recursion (the forward pass starts from it), row S ends the backward pass
  // followed by the same rows as (t1, t2, t0 - t2, t0 - t2) for the blocked
  // recursion
  std::vector<float4> t4(2 * (size_t)(S + 1));
  t4[0] = make_float4(1.f, 0.f, 0.f, 1.f);
  for (uint32_t m = 1; m < S; ++m)
    t4[m] = make_float4(tran[3 * m], tran[3 * m + 1], tran[3 * m + 2],
                        tran[3 * m] - tran[3 * m + 2]);
  t4[S] = make_float4(1.f, 0.f, 0.f, 1.f);
  for (uint32_t m = 0; m <= S; ++m)
    t4[S + 1 + m] = make_float4(t4[m].y, t4[m].z, t4[m].w, t4[m].w);
  if (int rc = quiesce(c))
    return rc;
  if (pb->S != S) {
    release(pb->d_tran4);
    pb->S = 0;
    GLP_CUDA(c, cudaMalloc((void **)&pb->d_tran4, sizeof(float4) * t4.size()));
    pb->S = S;
  }
  GLP_CUDA(c, cudaMemcpy(pb->d_tran4, t4.data(), sizeof(float4) * t4.size(),
                         cudaMemcpyHostToDevice));
  return GLP_OK;
}

int set_pc(glp_problem *pb, const float *pc16) {
  if (!pc16)
    return fail(pb->ctx, GLP_ERR_ARG, "pc must be non-null");
  std::memcpy(pb->pc, pc16, sizeof(pb->pc));
  pb->have_pc = true;
  return upload_vq_table(pb);
}

int set_codebook(glp_problem *pb, const float *codebook, uint32_t entries) {
  if (!codebook || entries != 16)
    return fail(pb->ctx, GLP_ERR_ARG, "codebook must hold 16 (RR, Het) entries, got %u",
                entries);
  std::memcpy(pb->codebook, codebook, sizeof(pb->codebook));
  pb->have_codebook = true;
  return upload_vq_table(pb);
}

int set_packed(glp_problem *pb, const uint32_t *packed, size_t n) {
  glp_ctx *c = pb->ctx;
  if (!packed || n == 0)
    return fail(c, GLP_ERR_ARG, "packed GLs must be non-empty");
  if (int rc = quiesce(c))
    return rc;
  if (n != pb->packed_words) {
    release(pb->d_packed);
    pb->packed_words = 0;
    GLP_CUDA(c, cudaMalloc((void **)&pb->d_packed, sizeof(uint32_t) * n));
    pb->packed_words = n;
  }
  GLP_CUDA(c, cudaMemcpy(pb->d_packed, packed, sizeof(uint32_t) * n, cudaMemcpyHostToDevice));
  return GLP_OK;
}

int set_emission(glp_problem *pb, const float *emit, const float *prob, uint32_t N,
                 uint32_t S) {
  glp_ctx *c = pb->ctx;
  if (!emit || N == 0 || S == 0)
    return fail(c, GLP_ERR_ARG, "emit must be non-null with positive N and S");
  if (int rc = quiesce(c))
    return rc;
  const size_t ns = (size_t)N * S;
  if (pb->eN != N || pb->eS != S || pb->borrowed) {
    drop_emission(pb);
    GLP_CUDA(c, cudaMalloc((void **)&pb->d_emit, sizeof(float4) * ns));
    pb->eN = N;
    pb->eS = S;
  }
  GLP_CUDA(c, cudaMemcpy(pb->d_emit, emit, sizeof(float4) * ns, cudaMemcpyHostToDevice));
  if (!prob) {
    // no genotype probabilities with these emissions (earlier ones belong to
    // other GLs): a generation that runs hmm_work is refused
    release(pb->d_prob);
    return GLP_OK;
  }
  if (!pb->d_prob)
    GLP_CUDA(c, cudaMalloc((void **)&pb->d_prob, sizeof(float) * 3 * ns));
  GLP_CUDA(c, cudaMemcpy(pb->d_prob, prob, sizeof(float) * 3 * ns, cudaMemcpyHostToDevice));
  return GLP_OK;
}

using glp::MultiFn;
using glp::SingleFn;

// Speculation shape of a launch: P lanes per sample (P/2 lane pairs, one
// evaluation each per round).
struct Shape {
  uint32_t P = 2;
  uint32_t sub = 1;  // normalisations per 8-site block (2: every 4 sites)
};

SingleFn single_kernel(Shape sh, bool vq) {
  if (sh.sub == 2)
    return vq ? glp::single_kernel_vq_sub4(sh.P) : glp::single_kernel_f32_sub4(sh.P);
  return vq ? glp::single_kernel_vq(sh.P) : glp::single_kernel_f32(sh.P);
}
MultiFn multi_kernel(Shape sh, bool vq) {
  if (sh.sub == 2)
    return vq ? glp::multi_kernel_vq_sub4(sh.P) : glp::multi_kernel_f32_sub4(sh.P);
  return vq ? glp::multi_kernel_vq(sh.P) : glp::multi_kernel_f32(sh.P);
}

// hmm_work of a generation: the recursions (blocks of two warps over 32
// samples, backward and forward at once), then the sampling (one warp per
// sample).  The recursions' staging tiles take more than the default 48 KB
// of shared memory: allow_chain_smem opts the kernels in on the current
// device (at context creation, before any launch or graph capture).
cudaError_t allow_chain_smem() {
  cudaError_t e = cudaFuncSetAttribute(glp::work_chains_kernel<>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)glp::kChainSmem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(glp::work_chains_multi_kernel<>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)glp::kChainSmem);
  return e;
}
void launch_work(const glp::GenParams &p, uint64_t samples, cudaStream_t st) {
  glp::work_chains_kernel<><<<(unsigned)((samples + glp::kPairRows - 1) / glp::kPairRows),
                              glp::kChainThreads, glp::kChainSmem, st>>>(p);
  glp::work_sample_kernel<><<<(unsigned)(samples * glp::sample_parts(p.wn)), 32, 0, st>>>(p);
}
void launch_work(const glp::MultiParams &mp, uint64_t samples, cudaStream_t st) {
  glp::work_chains_multi_kernel<><<<(unsigned)((samples + glp::kPairRows - 1) / glp::kPairRows),
                                    glp::kChainThreads, glp::kChainSmem, st>>>(mp);
  glp::work_sample_multi_kernel<><<<(unsigned)samples, 32, 0, st>>>(mp);
}

// Threads of the generation kernel with P lanes per sample that the GPU keeps
// resident (registers and the per-group staging rings limit the blocks per
// SM), or 0 when the occupancy query fails.
template <class Fn>
double resident_threads(Fn fn, uint32_t P, int sms) {
  const size_t smem = glp::stage_bytes((int)P);
  int occ = 0;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
          cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, glp::kThreads, smem) !=
          cudaSuccess)
    return 0.0;
  return (double)occ * glp::kThreads * sms;
}

// Speculation width for N samples at acceptance rate a.  A group of P lanes
// scores n = P/2 positions of the chain a round (one per lane pair), of which
// (1 - (1-a)^n) / (a n) are useful.  A lane-round costs kLaneRoundCost[P]
// relative to P = 8 when the GPU is full (narrow groups stage more rows per
// lane, and at 2 lanes the staging rings cap the resident blocks).  The
// kernels are issue-bound, so lane-rounds run at a rate that saturates with
// the share u = min(N P, threads resident with P lanes) / the most resident
// for any P: rate(u) = u (1 + h) / (u + h), h = 0.08 (0.93 of the full rate
// at half the warps).  The score is useful fraction x rate / cost.
constexpr double kLaneRoundCost[6] = {0.0, 2.44, 1.34, 1.0, 0.955, 0.953};

template <class FnOf>
uint32_t pick_lanes(double a, uint64_t N, int sms, FnOf kernel_for, double *cache = nullptr,
                    bool *known = nullptr) {
  double local[6] = {};
  double *res = cache ? cache : local;
  if (!known || !*known) {
    res[0] = 0.0;
    for (int i = 1; i < 6; ++i)
      res[i] = resident_threads(kernel_for(1u << i), 1u << i, sms);
    if (known)
      *known = true;
  }
  double most = 0;
  for (int i = 1; i < 6; ++i)
    most = std::max(most, res[i]);
  if (most <= 0)
    return 8;
  uint32_t best = 2;
  double best_score = 0;
  for (int i = 1; i < 6; ++i) {
    const uint32_t P = 1u << i;
    const double n = P / 2;
    const double eff = (1.0 - std::pow(1.0 - a, n)) / (a * n);
    const double u = std::min((double)N * P, res[i]) / most;
    constexpr double h = 0.08;
    const double rate = u * (1.0 + h) / (u + h);
    const double score = eff * rate / kLaneRoundCost[i];
    if (score > best_score * 1.02) {
      best_score = score;
      best = P;
    }
  }
  return best;
}

uint32_t choose_lanes(glp_ctx *c, uint64_t N, bool multi, bool vq, float pen) {
  if (c->lanes)
    return c->lanes;
  const double a = (c->last_accept < 0 || pen != c->accept_pen)
                       ? 0.12
                       : std::max(c->last_accept, 1e-3);
  return pick_lanes(
      a, N, c->sms,
      [&](uint32_t P) {
        Shape sh;
        sh.P = P;
        return multi ? (const void *)multi_kernel(sh, vq) : (const void *)single_kernel(sh, vq);
      },
      c->resident[multi][vq], &c->resident_known[multi][vq]);
}

// Lanes from choose_lanes (a request below two lanes gets two: one
// evaluation a round), normalisation block from the context's rule.
Shape choose_shape(glp_ctx *c, uint64_t N, bool multi, bool vq, float pen) {
  Shape sh;
  sh.P = std::max<uint32_t>(2u, choose_lanes(c, N, multi, vq, pen));
  c->launch_pen = pen;
  if (c->block_sites == 4 || (c->block_sites == 0 && c->short_blocks))
    sh.sub = 2;
  return sh;
}

// Validate one (problem, generation) pair and fill its kernel descriptor.
int make_params(glp_ctx *c, glp_problem *pb, const glp_generation_args *a,
                glp::GenParams *p) {
  const bool vq = (a->flags & GLP_GEN_VQ) != 0;
  const bool work = (a->flags & GLP_GEN_NO_WORK) == 0;
  const uint32_t N = a->num_samples, S = a->num_sites, C = a->num_cycles, H = a->num_haps;
  if (N == 0 || S == 0)
    return fail(c, GLP_ERR_ARG, "num_samples and num_sites must be positive");
  if (H < 2 || (uint64_t)2 * N > H)
    return fail(c, GLP_ERR_ARG, "num_haps=%u must be >= 2*num_samples=%u", H, 2 * N);
  if (!a->haps || !a->hap_idxs_out)
    return fail(c, GLP_ERR_ARG, "haps and hap_idxs_out are required");
  uint32_t lo = a->sample_lo, hi = a->sample_hi;
  if (lo == 0 && hi == 0)
    hi = H;
  const bool draws = !a->hap_idxs_in || (C && !a->props);
  if (draws) {
    if (a->neighbors && a->neighbors_per_sample == 0)
      return fail(c, GLP_ERR_ARG, "neighbors_per_sample must be positive");
    if (!a->neighbors && (hi > H || lo >= hi || hi - lo < 3))
      return fail(c, GLP_ERR_ARG, "surrogate range [%u, %u) must hold 3+ of %u haplotypes",
                  lo, hi, H);
  }
  const bool kick_first = (a->flags & GLP_GEN_KICK_FIRST) != 0;
  if (kick_first && draws && C && H < 2 * N + 1)
    return fail(c, GLP_ERR_ARG,
                "GLP_GEN_KICK_FIRST needs panel haplotypes after the 2*num_samples=%u rows", 2 * N);
  if (work && !a->hnew)
    return fail(c, GLP_ERR_ARG, "hnew is required unless GLP_GEN_NO_WORK is set");
  if (!pb->d_tran4 || pb->S != S)
    return fail(c, GLP_ERR_STATE, "transition matrix not set for %u sites", S);
  if (!pb->have_pc)
    return fail(c, GLP_ERR_STATE, "mutation matrix not set");
  if (vq) {
    if (!pb->d_packed || !pb->d_vq)
      return fail(c, GLP_ERR_STATE, "packed GLs and codebook are required in VQ mode");
    const size_t want = (size_t)N * ((S + 7) / 8);
    if (pb->packed_words != want)
      return fail(c, GLP_ERR_ARG, "packed GLs have %zu words, expected %zu", pb->packed_words,
                  want);
  }
  if (!vq || work) {
    if (!pb->d_emit || pb->eN != N || pb->eS != S)
      return fail(c, GLP_ERR_STATE, "emission not set for N=%u S=%u", N, S);
  }
  if (work && !pb->d_prob)
    return fail(c, GLP_ERR_STATE, "genotype probabilities not set (needed by hmm_work)");
  const bool tr = a->trace_slot || a->trace_accept || a->trace_work;
  if (tr && !(a->trace_slot && a->trace_accept && a->trace_work))
    return fail(c, GLP_ERR_ARG, "a replay trace needs slot, accept and work arrays");
  if (!(a->pen > 0.0f) || !std::isfinite(a->pen))
    return fail(c, GLP_ERR_ARG, "pen must be positive and finite");
  if (work) {
    int rc = ensure(c, pb->d_beta, pb->beta_cap, (size_t)N * S);
    if (rc)
      return rc;
  }
  std::memset(p, 0, sizeof(*p));
  p->N = N;
  p->S = S;
  p->C = C;
  p->H = H;
  p->wn = (S + 63) / 64;
  p->emit_mode = vq ? GLP_EMIT_VQ : GLP_EMIT_FLOAT;
  p->haps = a->haps;
  p->hnew = a->hnew;
  p->emit = pb->d_emit;
  p->prob = pb->d_prob;
  p->tran4 = pb->d_tran4;
  p->tranp = pb->d_tran4 + (S + 1);
  p->packed = pb->d_packed;
  p->vq_table = vq ? pb->d_vq : nullptr;
  p->quad_in = a->hap_idxs_in;
  p->quad_out = a->hap_idxs_out;
  p->props = a->props;
  p->tr_slot = a->trace_slot;
  p->tr_u = a->trace_accept;
  p->tr_work = a->trace_work;
  p->like_out = a->like_out;
  p->eval_trace = a->eval_trace;
  p->accept_trace = a->accept_trace;
  p->beta = pb->d_beta;
  p->counter = c->d_counter;
  p->stats = c->d_stats;
  p->error = c->d_error;
  p->nbr = a->neighbors;
  p->klen = a->neighbors_per_sample;
  p->samp_lo = lo;
  p->samp_hi = hi;
  std::memcpy(p->pc, pb->pc, sizeof(p->pc));
  p->pen = a->pen;
  p->seed = a->seed;
  p->generation = a->generation;
  p->do_work = work ? 1u : 0u;
  p->burnin = a->burnin;
  p->kick = a->kick_start ? 1u : 0u;
  p->kick_first = kick_first ? 1u : 0u;
  return GLP_OK;
}

template <class Fn>
unsigned grid_for(glp_ctx *c, Fn fn, uint64_t samples, uint32_t P, int *rc) {
  const size_t smem = glp::stage_bytes((int)P);
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int occ = 0;
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, glp::kThreads, smem);
  if (e != cudaSuccess) {
    *rc = fail(c, GLP_ERR_CUDA, "occupancy query failed: %s", cudaGetErrorString(e));
    return 0;
  }
  occ = std::max(occ, 1);
  const uint64_t groups_per_block = (uint64_t)glp::kThreads / P;
  const uint64_t want = (samples + groups_per_block - 1) / groups_per_block;
  const uint64_t cap = (uint64_t)occ * c->sms;
  *rc = GLP_OK;
  return (unsigned)std::max<uint64_t>(1, std::min(want, cap));
}

int launch_single(glp_ctx *c, glp_problem *pb, const glp_generation_args *a) {
  glp::GenParams p;
  int rc = make_params(c, pb, a, &p);
  if (rc)
    return rc;
  const bool vq = (a->flags & GLP_GEN_VQ) != 0;
  const Shape sh = choose_shape(c, a->num_samples, false, vq, a->pen);
  const uint32_t P = sh.P;
  SingleFn fn = single_kernel(sh, vq);
  const unsigned grid = grid_for(c, fn, a->num_samples, P, &rc);
  if (rc)
    return rc;
  GLP_CUDA(c, cudaMemsetAsync(c->d_counter, 0, sizeof(uint32_t), c->stream));
  GLP_CUDA(c, cudaMemsetAsync(c->d_stats, 0, glp::kStats * sizeof(unsigned long long), c->stream));
  cudaEvent_t *ev = c->ev[c->ev_count++ % glp_ctx::kTimed];
  GLP_CUDA(c, cudaEventRecord(ev[0], c->stream));
  fn<<<grid, glp::kThreads, glp::stage_bytes((int)P), c->stream>>>(p);
  GLP_CUDA(c, cudaGetLastError());
  GLP_CUDA(c, cudaEventRecord(ev[1], c->stream));
  if (p.do_work) {
    launch_work(p, a->num_samples, c->stream);
    GLP_CUDA(c, cudaGetLastError());
  }
  GLP_CUDA(c, cudaEventRecord(ev[2], c->stream));
  c->lanes_used = P;
  c->last_chain_cycles = (uint64_t)a->num_samples * a->num_cycles;
  return GLP_OK;
}

}  // namespace

extern "C" {

int glp_check_device(int device, int *device_count, int *cc_major, int *cc_minor,
                     int *sm_count) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (device_count)
    *device_count = (e == cudaSuccess) ? n : 0;
  if (e != cudaSuccess || n == 0)
    return GLP_ERR_DEVICE;
  if (device < 0 || device >= n)
    return GLP_ERR_ARG;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess)
    return GLP_ERR_CUDA;
  if (cc_major)
    *cc_major = prop.major;
  if (cc_minor)
    *cc_minor = prop.minor;
  if (sm_count)
    *sm_count = prop.multiProcessorCount;
  return (prop.major == 10 && prop.minor == 3) ? GLP_OK : GLP_ERR_DEVICE;
}

int glp_create(int device, glp_ctx **out) {
  if (!out)
    return GLP_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
    return GLP_ERR_DEVICE;
  if (device < 0 || device >= n)
    return GLP_ERR_ARG;
  glp_ctx *c = new glp_ctx();
  c->device = device;
  c->def.ctx = c;
  int rc = check_ctx(c);
  if (rc) {
    delete c;
    return rc;
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc((void **)&c->d_counter, sizeof(uint32_t)) != cudaSuccess ||
      cudaMalloc((void **)&c->d_stats, glp::kStats * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc((void **)&c->d_error, sizeof(int)) != cudaSuccess ||
      cudaMemset(c->d_error, 0, sizeof(int)) != cudaSuccess ||
      allow_chain_smem() != cudaSuccess) {
    glp_destroy(c);
    return GLP_ERR_CUDA;
  }
  for (uint32_t i = 0; i < glp_ctx::kTimed; ++i)
    for (int j = 0; j < 3; ++j)
      if (cudaEventCreate(&c->ev[i][j]) != cudaSuccess) {
        glp_destroy(c);
        return GLP_ERR_CUDA;
      }
  c->sms = prop.multiProcessorCount;
  c->stream = c->own_stream;
  *out = c;
  return GLP_OK;
}

void glp_destroy(glp_ctx *c) {
  if (!c)
    return;
  cudaSetDevice(c->device);
  if (c->stream)
    cudaStreamSynchronize(c->stream);
  release_problem(&c->def);
  release(c->d_counter);
  release(c->d_stats);
  release(c->d_error);
  release(c->d_table);
  release(c->d_offsets);
  if (c->h_table)
    cudaFreeHost(c->h_table);
  if (c->h_offsets)
    cudaFreeHost(c->h_offsets);
  release(c->d_haps);
  release(c->d_hnew);
  release(c->d_quad);
  release(c->d_quad_out);
  release(c->d_props);
  release(c->d_nbr);
  release(c->d_mask);
  release(c->d_knn_dist);
  release(c->d_tr_slot);
  release(c->d_acc);
  release(c->d_tr_u);
  release(c->d_like);
  release(c->d_evals);
  release(c->d_tr_work);
  for (uint32_t i = 0; i < glp_ctx::kTimed; ++i)
    for (int j = 0; j < 3; ++j)
      if (c->ev[i][j])
        cudaEventDestroy(c->ev[i][j]);
  if (c->own_stream)
    cudaStreamDestroy(c->own_stream);
  delete c;
}

const char *glp_last_error(const glp_ctx *c) {
  if (!c)
    return "null context";
  return c->err.c_str();
}

int glp_set_stream(glp_ctx *c, void *stream) {
  if (!c)
    return GLP_ERR_ARG;
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return GLP_OK;
}

int glp_set_tran(glp_ctx *c, const float *tran, uint32_t S) {
  int rc = check_ctx(c);
  return rc ? rc : set_tran(&c->def, tran, S);
}

int glp_set_mutation_mat(glp_ctx *c, const float *pc16) {
  int rc = check_ctx(c);
  return rc ? rc : set_pc(&c->def, pc16);
}

int glp_set_codebook(glp_ctx *c, const float *codebook, uint32_t entries) {
  int rc = check_ctx(c);
  return rc ? rc : set_codebook(&c->def, codebook, entries);
}

int glp_set_packed_gls(glp_ctx *c, const uint32_t *packed, size_t n) {
  int rc = check_ctx(c);
  return rc ? rc : set_packed(&c->def, packed, n);
}

int glp_set_emission(glp_ctx *c, const float *emit, const float *prob, uint32_t N, uint32_t S) {
  int rc = check_ctx(c);
  return rc ? rc : set_emission(&c->def, emit, prob, N, S);
}

int glp_problem_create(glp_ctx *c, glp_problem **out) {
  int rc = check_ctx(c);
  if (rc)
    return rc;
  if (!out)
    return fail(c, GLP_ERR_ARG, "out must be non-null");
  glp_problem *pb = new glp_problem();
  pb->ctx = c;
  *out = pb;
  return GLP_OK;
}

void glp_problem_destroy(glp_problem *pb) {
  if (!pb)
    return;
  if (pb->ctx) {
    cudaSetDevice(pb->ctx->device);
    if (pb->ctx->stream)
      cudaStreamSynchronize(pb->ctx->stream);
  }
  release_problem(pb);
  delete pb;
}

int glp_problem_set_model(glp_problem *pb, const float *tran, const float *pc16,
                          const float *emit, const float *prob, uint32_t num_samples,
                          uint32_t num_sites) {
  if (!pb || !pb->ctx)
    return GLP_ERR_ARG;
  int rc = check_ctx(pb->ctx);
  if (rc || (rc = set_tran(pb, tran, num_sites)) || (rc = set_pc(pb, pc16)) ||
      (rc = set_emission(pb, emit, prob, num_samples, num_sites)))
    return rc;
  return GLP_OK;
}

int glp_problem_set_model_device(glp_problem *pb, const float *tran, const float *pc16,
                                 const float *emit_dev, const float *prob_dev,
                                 uint32_t num_samples, uint32_t num_sites) {
  if (!pb || !pb->ctx)
    return GLP_ERR_ARG;
  glp_ctx *c = pb->ctx;
  int rc = check_ctx(c);
  if (rc || (rc = set_tran(pb, tran, num_sites)) || (rc = set_pc(pb, pc16)))
    return rc;
  if (!emit_dev || num_samples == 0 || num_sites == 0)
    return fail(c, GLP_ERR_ARG, "emit must be non-null with positive N and S");
  if (((uintptr_t)emit_dev & 15u) || ((uintptr_t)prob_dev & 3u))
    return fail(c, GLP_ERR_ARG, "emit must be 16-byte and prob 4-byte aligned");
  drop_emission(pb);
  pb->d_emit = (float4 *)emit_dev;
  pb->d_prob = (float *)prob_dev;
  pb->borrowed = true;
  pb->eN = num_samples;
  pb->eS = num_sites;
  return GLP_OK;
}

int glp_problem_set_vq(glp_problem *pb, const uint32_t *packed, size_t num_words,
                       const float *codebook) {
  if (!pb || !pb->ctx)
    return GLP_ERR_ARG;
  int rc = check_ctx(pb->ctx);
  if (rc || (rc = set_codebook(pb, codebook, 16)) || (rc = set_packed(pb, packed, num_words)))
    return rc;
  return GLP_OK;
}

int glp_run_generation(glp_ctx *c, const glp_generation_args *a) {
  int rc = check_ctx(c);
  if (rc)
    return rc;
  if (!a)
    return fail(c, GLP_ERR_ARG, "args must be non-null");
  return launch_single(c, &c->def, a);
}

int glp_run_batch(glp_ctx *c, uint32_t count, glp_problem *const *problems,
                  const glp_generation_args *args) {
  int rc = check_ctx(c);
  if (rc)
    return rc;
  if (count == 0 || !problems || !args)
    return fail(c, GLP_ERR_ARG, "a batch needs count > 0, problems and args");
  const bool vq = (args[0].flags & GLP_GEN_VQ) != 0;
  if (count > c->h_cap) {
    if (c->h_table)
      cudaFreeHost(c->h_table);
    if (c->h_offsets)
      cudaFreeHost(c->h_offsets);
    c->h_table = nullptr;
    c->h_offsets = nullptr;
    c->h_cap = 0;
    GLP_CUDA(c, cudaMallocHost((void **)&c->h_table, sizeof(glp::GenParams) * count));
    GLP_CUDA(c, cudaMallocHost((void **)&c->h_offsets, sizeof(uint32_t) * (count + 1)));
    c->h_cap = count;
  }
  // the staging buffers are reused: wait for the previous batch's upload
  GLP_CUDA(c, cudaStreamSynchronize(c->stream));
  uint64_t total = 0, chain_cycles = 0;
  c->h_offsets[0] = 0;
  for (uint32_t i = 0; i < count; ++i) {
    glp_problem *pb = problems[i];
    if (!pb || pb->ctx != c)
      return fail(c, GLP_ERR_ARG, "problem %u does not belong to this context", i);
    if (((args[i].flags & GLP_GEN_VQ) != 0) != vq)
      return fail(c, GLP_ERR_ARG, "all chunks of a batch must use the same emission source");
    if ((rc = make_params(c, pb, &args[i], &c->h_table[i])))
      return rc;
    total += args[i].num_samples;
    chain_cycles += (uint64_t)args[i].num_samples * args[i].num_cycles;
    if (total > 0xffffffffull)
      return fail(c, GLP_ERR_ARG, "a batch holds at most 2^32-1 samples");
    c->h_offsets[i + 1] = (uint32_t)total;
  }
  if ((rc = ensure(c, c->d_table, c->table_cap, count)) ||
      (rc = ensure(c, c->d_offsets, c->offsets_cap, (size_t)count + 1)))
    return rc;
  GLP_CUDA(c, cudaMemcpyAsync(c->d_table, c->h_table, sizeof(glp::GenParams) * count,
                              cudaMemcpyHostToDevice, c->stream));
  GLP_CUDA(c, cudaMemcpyAsync(c->d_offsets, c->h_offsets, sizeof(uint32_t) * (count + 1),
                              cudaMemcpyHostToDevice, c->stream));
  glp::MultiParams mp;
  mp.chunks = c->d_table;
  mp.offsets = c->d_offsets;
  mp.nchunks = count;
  mp.counter = c->d_counter;
  mp.stats = c->d_stats;
  mp.error = c->d_error;
  const Shape sh = choose_shape(c, total, true, vq, c->h_table[0].pen);
  const uint32_t P = sh.P;
  MultiFn fn = multi_kernel(sh, vq);
  const unsigned grid = grid_for(c, fn, total, P, &rc);
  if (rc)
    return rc;
  GLP_CUDA(c, cudaMemsetAsync(c->d_counter, 0, sizeof(uint32_t), c->stream));
  GLP_CUDA(c, cudaMemsetAsync(c->d_stats, 0, glp::kStats * sizeof(unsigned long long), c->stream));
  cudaEvent_t *ev = c->ev[c->ev_count++ % glp_ctx::kTimed];
  GLP_CUDA(c, cudaEventRecord(ev[0], c->stream));
  fn<<<grid, glp::kThreads, glp::stage_bytes((int)P), c->stream>>>(mp);
  GLP_CUDA(c, cudaGetLastError());
  GLP_CUDA(c, cudaEventRecord(ev[1], c->stream));
  launch_work(mp, total, c->stream);
  GLP_CUDA(c, cudaEventRecord(ev[2], c->stream));
  GLP_CUDA(c, cudaGetLastError());
  c->lanes_used = P;
  c->last_chain_cycles = chain_cycles;
  return GLP_OK;
}

}  // extern "C"

struct glp_batch {
  glp_ctx *c = nullptr;
  uint32_t count = 0;
  uint64_t total = 0, chain_cycles = 0;
  uint32_t P = 8;
  unsigned grid = 1;
  glp::GenParams *d_table = nullptr;
  uint32_t *d_offsets = nullptr;
  glp::MultiParams mp;
  MultiFn fn = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

int batch_enqueue(glp_batch *b, cudaStream_t st) {
  glp_ctx *c = b->c;
  GLP_CUDA(c, cudaMemsetAsync(c->d_counter, 0, sizeof(uint32_t), st));
  GLP_CUDA(c, cudaMemsetAsync(c->d_stats, 0, glp::kStats * sizeof(unsigned long long), st));
  b->fn<<<b->grid, glp::kThreads, glp::stage_bytes((int)b->P), st>>>(b->mp);
  GLP_CUDA(c, cudaGetLastError());
  launch_work(b->mp, b->total, st);
  GLP_CUDA(c, cudaGetLastError());
  glp::advance_kernel<<<(b->count + 127) / 128, 128, 0, st>>>(b->d_table, b->count);
  GLP_CUDA(c, cudaGetLastError());
  return GLP_OK;
}

}  // namespace

extern "C" {

void glp_batch_destroy(glp_batch *b) {
  if (!b)
    return;
  if (b->c) {
    cudaSetDevice(b->c->device);
    cudaStreamSynchronize(b->c->stream);
  }
  if (b->exec)
    cudaGraphExecDestroy(b->exec);
  if (b->graph)
    cudaGraphDestroy(b->graph);
  release(b->d_table);
  release(b->d_offsets);
  delete b;
}

int glp_batch_prepare(glp_ctx *c, uint32_t count, glp_problem *const *problems,
                      const glp_generation_args *args, glp_batch **out) {
  int rc = check_ctx(c);
  if (rc)
    return rc;
  if (!out || count == 0 || !problems || !args)
    return fail(c, GLP_ERR_ARG, "a batch needs count > 0, problems, args and out");
  *out = nullptr;
  const bool vq = (args[0].flags & GLP_GEN_VQ) != 0;
  std::vector<glp::GenParams> table(count);
  std::vector<uint32_t> offsets(count + 1, 0);
  uint64_t total = 0, chain_cycles = 0;
  for (uint32_t i = 0; i < count; ++i) {
    glp_problem *pb = problems[i];
    if (!pb || pb->ctx != c)
      return fail(c, GLP_ERR_ARG, "problem %u does not belong to this context", i);
    if (((args[i].flags & GLP_GEN_VQ) != 0) != vq)
      return fail(c, GLP_ERR_ARG, "all chunks of a batch must use the same emission source");
    if (args[i].hap_idxs_in || (args[i].num_cycles && args[i].props))
      return fail(c, GLP_ERR_ARG, "prepared batches draw their surrogates on the device");
    if (args[i].trace_slot || args[i].trace_accept || args[i].trace_work)
      return fail(c, GLP_ERR_ARG, "prepared batches do not replay traces");
    if ((rc = make_params(c, pb, &args[i], &table[i])))
      return rc;
    total += args[i].num_samples;
    chain_cycles += (uint64_t)args[i].num_samples * args[i].num_cycles;
    if (total > 0xffffffffull)
      return fail(c, GLP_ERR_ARG, "a batch holds at most 2^32-1 samples");
    offsets[i + 1] = (uint32_t)total;
  }
  glp_batch *b = new glp_batch();
  b->c = c;
  b->count = count;
  b->total = total;
  b->chain_cycles = chain_cycles;
  cudaStream_t cs = nullptr;
  auto bail = [&](int code) {
    if (cs)
      cudaStreamDestroy(cs);
    glp_batch_destroy(b);
    return code;
  };
  if (cudaMalloc((void **)&b->d_table, sizeof(glp::GenParams) * count) != cudaSuccess ||
      cudaMalloc((void **)&b->d_offsets, sizeof(uint32_t) * (count + 1)) != cudaSuccess)
    return bail(fail(c, GLP_ERR_NOMEM, "batch descriptor allocation failed"));
  if (cudaMemcpy(b->d_table, table.data(), sizeof(glp::GenParams) * count,
                 cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->d_offsets, offsets.data(), sizeof(uint32_t) * (count + 1),
                 cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(fail(c, GLP_ERR_CUDA, "batch descriptor upload failed"));
  b->mp.chunks = b->d_table;
  b->mp.offsets = b->d_offsets;
  b->mp.nchunks = count;
  b->mp.counter = c->d_counter;
  b->mp.stats = c->d_stats;
  b->mp.error = c->d_error;
  const Shape sh = choose_shape(c, total, true, vq, table[0].pen);
  b->P = sh.P;
  b->fn = multi_kernel(sh, vq);
  b->grid = grid_for(c, b->fn, total, b->P, &rc);
  if (rc)
    return bail(rc);
  if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(c, GLP_ERR_CUDA, "capture stream creation failed"));
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess)
    return bail(fail(c, GLP_ERR_CUDA, "cudaStreamBeginCapture: %s", cudaGetErrorString(e)));
  rc = batch_enqueue(b, cs);
  e = cudaStreamEndCapture(cs, &b->graph);
  if (rc)
    return bail(rc);
  if (e != cudaSuccess)
    return bail(fail(c, GLP_ERR_CUDA, "cudaStreamEndCapture: %s", cudaGetErrorString(e)));
  e = cudaGraphInstantiate(&b->exec, b->graph, 0);
  if (e != cudaSuccess)
    return bail(fail(c, GLP_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e)));
  cudaStreamDestroy(cs);
  *out = b;
  return GLP_OK;
}

int glp_batch_run(glp_batch *b) {
  if (!b || !b->c)
    return GLP_ERR_ARG;
  glp_ctx *c = b->c;
  int rc = check_ctx(c);
  if (rc)
    return rc;
  GLP_CUDA(c, cudaGraphLaunch(b->exec, c->stream));
  c->lanes_used = b->P;
  c->last_chain_cycles = b->chain_cycles;
  return GLP_OK;
}

int glp_batch_launch(glp_batch *b) {
  if (!b || !b->c)
    return GLP_ERR_ARG;
  glp_ctx *c = b->c;
  int rc = check_ctx(c);
  if (rc || (rc = batch_enqueue(b, c->stream)))
    return rc;
  c->lanes_used = b->P;
  c->last_chain_cycles = b->chain_cycles;
  return GLP_OK;
}

int glp_finish(glp_ctx *c) {
  int rc = check_ctx(c);
  if (rc)
    return rc;
  GLP_CUDA(c, cudaStreamSynchronize(c->stream));
  GLP_CUDA(c, cudaGetLastError());
  int h_err = 0;
  GLP_CUDA(c, cudaMemcpy(&h_err, c->d_error, sizeof(int), cudaMemcpyDeviceToHost));
  GLP_CUDA(c, cudaMemcpy(c->last_stats, c->d_stats, sizeof(c->last_stats),
                         cudaMemcpyDeviceToHost));
  if (c->last_chain_cycles) {
    c->last_accept = (double)c->last_stats[2] / (double)c->last_chain_cycles;
    c->accept_pen = c->launch_pen;
  }
  if (c->block_sites == 0 && c->last_stats[0] && c->last_stats[3] * 1000ull > c->last_stats[0])
    c->short_blocks = true;
  if (h_err) {
    GLP_CUDA(c, cudaMemset(c->d_error, 0, sizeof(int)));
    if (h_err & ~1)
      return fail(c, GLP_ERR_INDEX, "device self-check failed: flag 0x%x", (unsigned)h_err);
    return fail(c, GLP_ERR_INDEX, "a haplotype index >= num_haps reached the device");
  }
  return GLP_OK;
}

int glp_run_generation_host(glp_ctx *c, const glp_generation_args *a) {
  int rc = check_ctx(c);
  if (rc)
    return rc;
  if (!a || !a->haps || !a->hap_idxs_out)
    return fail(c, GLP_ERR_ARG, "haps and hap_idxs_out are required");
  const uint32_t N = a->num_samples, S = a->num_sites, C = a->num_cycles, H = a->num_haps;
  const bool work = (a->flags & GLP_GEN_NO_WORK) == 0;
  if (work && !a->hnew)
    return fail(c, GLP_ERR_ARG, "hnew is required unless GLP_GEN_NO_WORK is set");
  const size_t wn = (S + 63) / 64;
  const size_t hw = (size_t)H * wn;
  if ((rc = ensure(c, c->d_haps, c->haps_cap, hw)))
    return rc;
  if (work && (rc = ensure(c, c->d_hnew, c->hnew_cap, hw)))
    return rc;
  if ((rc = ensure(c, c->d_quad, c->quad_cap, (size_t)4 * N)))
    return rc;
  if ((rc = ensure(c, c->d_quad_out, c->quad_out_cap, (size_t)4 * N)))
    return rc;
  if ((rc = ensure(c, c->d_props, c->props_cap, (size_t)C * N)))
    return rc;
  cudaStream_t st = c->stream;
  // hnew needs no upload: the kernel writes every word of rows 0..2N-1 and
  // only those rows are copied back.
  GLP_CUDA(c, cudaMemcpyAsync(c->d_haps, a->haps, hw * 8, cudaMemcpyHostToDevice, st));
  if (a->hap_idxs_in)
    GLP_CUDA(c, cudaMemcpyAsync(c->d_quad, a->hap_idxs_in, (size_t)16 * N,
                                cudaMemcpyHostToDevice, st));
  if (C && a->props)
    GLP_CUDA(c, cudaMemcpyAsync(c->d_props, a->props, (size_t)4 * C * N,
                                cudaMemcpyHostToDevice, st));
  glp_generation_args d = *a;
  d.haps = c->d_haps;
  d.hnew = work ? c->d_hnew : nullptr;
  d.hap_idxs_in = a->hap_idxs_in ? c->d_quad : nullptr;
  d.hap_idxs_out = c->d_quad_out;
  d.props = a->props ? c->d_props : nullptr;
  if (a->neighbors) {
    const size_t nk = (size_t)N * a->neighbors_per_sample;
    if ((rc = ensure(c, c->d_nbr, c->nbr_cap, nk)))
      return rc;
    GLP_CUDA(c, cudaMemcpyAsync(c->d_nbr, a->neighbors, nk * 4, cudaMemcpyHostToDevice, st));
    d.neighbors = c->d_nbr;
  }
  if (a->trace_slot || a->trace_accept || a->trace_work) {
    if (!(a->trace_slot && a->trace_accept && a->trace_work))
      return fail(c, GLP_ERR_ARG, "a replay trace needs slot, accept and work arrays");
    if ((rc = ensure(c, c->d_tr_slot, c->tr_slot_cap, (size_t)N * C)) ||
        (rc = ensure(c, c->d_tr_u, c->tr_u_cap, (size_t)N * C)) ||
        (rc = ensure(c, c->d_tr_work, c->tr_work_cap, (size_t)N * S)))
      return rc;
    GLP_CUDA(c, cudaMemcpyAsync(c->d_tr_slot, a->trace_slot, (size_t)N * C,
                                cudaMemcpyHostToDevice, st));
    GLP_CUDA(c, cudaMemcpyAsync(c->d_tr_u, a->trace_accept, (size_t)8 * N * C,
                                cudaMemcpyHostToDevice, st));
    GLP_CUDA(c, cudaMemcpyAsync(c->d_tr_work, a->trace_work, (size_t)4 * N * S,
                                cudaMemcpyHostToDevice, st));
    d.trace_slot = c->d_tr_slot;
    d.trace_accept = c->d_tr_u;
    d.trace_work = c->d_tr_work;
  }
  if (a->like_out) {
    if ((rc = ensure(c, c->d_like, c->like_cap, N)))
      return rc;
    d.like_out = c->d_like;
  }
  if (a->eval_trace) {
    if ((rc = ensure(c, c->d_evals, c->evals_cap, (size_t)N * (C + 1))))
      return rc;
    d.eval_trace = c->d_evals;
  }
  if (a->accept_trace) {
    if ((rc = ensure(c, c->d_acc, c->acc_cap, std::max<size_t>((size_t)N * C, 1))))
      return rc;
    d.accept_trace = c->d_acc;
  }
  if ((rc = launch_single(c, &c->def, &d)))
    return rc;
  GLP_CUDA(c, cudaMemcpyAsync(a->hap_idxs_out, c->d_quad_out, (size_t)16 * N,
                              cudaMemcpyDeviceToHost, st));
  if (work)
    GLP_CUDA(c, cudaMemcpyAsync(a->hnew, c->d_hnew, (size_t)2 * N * wn * 8,
                                cudaMemcpyDeviceToHost, st));
  if (a->like_out)
    GLP_CUDA(c, cudaMemcpyAsync(a->like_out, c->d_like, (size_t)8 * N, cudaMemcpyDeviceToHost,
                                st));
  if (a->eval_trace)
    GLP_CUDA(c, cudaMemcpyAsync(a->eval_trace, c->d_evals, (size_t)8 * N * (C + 1),
                                cudaMemcpyDeviceToHost, st));
  if (a->accept_trace && C)
    GLP_CUDA(c, cudaMemcpyAsync(a->accept_trace, c->d_acc, (size_t)N * C,
                                cudaMemcpyDeviceToHost, st));
  return glp_finish(c);
}

int glp_run_hmm_on_device(glp_ctx *c, const uint64_t *hap_panel, size_t panel_words,
                          const uint32_t *extra_prop_haps, uint32_t num_sites,
                          uint32_t num_samples, uint32_t num_cycles, uint32_t *hap_idxs,
                          uint64_t seed) {
  int rc = check_ctx(c);
  if (rc)
    return rc;
  if (!hap_panel || !hap_idxs || (num_cycles && !extra_prop_haps))
    return fail(c, GLP_ERR_ARG, "hap_panel, extra_prop_haps and hap_idxs are required");
  const size_t wn = ((size_t)num_sites + 63) / 64;
  if (wn == 0 || panel_words % wn)
    return fail(c, GLP_ERR_ARG, "panel of %zu words is not a whole number of %zu-word haps",
                panel_words, wn);
  const size_t H = panel_words / wn;
  if (H > 0xffffffffu || H < 2 * (size_t)num_samples)
    return fail(c, GLP_ERR_ARG, "panel holds %zu haplotypes for %u samples", H, num_samples);
  std::vector<uint32_t> out(4 * (size_t)num_samples);
  glp_generation_args a;
  std::memset(&a, 0, sizeof(a));
  a.num_samples = num_samples;
  a.num_sites = num_sites;
  a.num_cycles = num_cycles;
  a.num_haps = (uint32_t)H;
  a.haps = hap_panel;
  a.hap_idxs_in = hap_idxs;
  a.hap_idxs_out = out.data();
  a.props = extra_prop_haps;
  a.pen = 1.0f;  // findHapSet accepts with S = 1 (hmmLike.cu:159)
  a.seed = seed;
  a.flags = GLP_GEN_VQ | GLP_GEN_NO_WORK;
  rc = glp_run_generation_host(c, &a);
  if (rc)
    return rc;
  std::memcpy(hap_idxs, out.data(), out.size() * sizeof(uint32_t));
  return GLP_OK;
}

int glp_set_lanes_per_sample(glp_ctx *c, uint32_t lanes) {
  if (!c)
    return GLP_ERR_ARG;
  if (lanes && lanes != 1 && lanes != 2 && lanes != 4 && lanes != 8 && lanes != 16 &&
      lanes != 32)
    return fail(c, GLP_ERR_ARG, "lanes per sample must be 0, 1, 2, 4, 8, 16 or 32");
  c->lanes = lanes;
  return GLP_OK;
}

int glp_set_evals_per_lane(glp_ctx *c, uint32_t evals) {
  if (!c)
    return GLP_ERR_ARG;
  if (evals > 1)
    return fail(c, GLP_ERR_ARG, "each lane pair scores one evaluation a round: evals must be 0 or 1");
  c->evals = evals;
  return GLP_OK;
}

int glp_set_knn_metric(glp_ctx *c, int metric) {
  if (!c)
    return GLP_ERR_ARG;
  if (metric != GLP_KNN_HAMMING && metric != GLP_KNN_TRACT)
    return fail(c, GLP_ERR_ARG, "kNN metric must be GLP_KNN_HAMMING or GLP_KNN_TRACT");
  c->knn_metric = metric;
  return GLP_OK;
}

int glp_set_block_sites(glp_ctx *c, uint32_t sites) {
  if (!c)
    return GLP_ERR_ARG;
  if (sites != 0 && sites != 4 && sites != 8)
    return fail(c, GLP_ERR_ARG, "sites per normalisation block must be 0, 4 or 8");
  c->block_sites = sites;
  c->short_blocks = false;
  return GLP_OK;
}

int glp_get_block_sites(glp_ctx *c, uint32_t *sites) {
  if (!c || !sites)
    return GLP_ERR_ARG;
  *sites = (c->block_sites == 4 || (c->block_sites == 0 && c->short_blocks)) ? 4u : 8u;
  return GLP_OK;
}

int glp_get_stats(glp_ctx *c, uint64_t *evaluations, uint64_t *rounds, uint32_t *lanes_used) {
  if (!c)
    return GLP_ERR_ARG;
  if (evaluations)
    *evaluations = c->last_stats[0];
  if (rounds)
    *rounds = c->last_stats[1];
  if (lanes_used)
    *lanes_used = c->lanes_used;
  return GLP_OK;
}

// ---------------------------------------------------------------------------
// Request server: continuous batching behind the context.  The scheduling
// (queue, admission, per-request generation arguments, retirement) is
// glp::ServerCore (glp_server_core.h); here each tick's launches go to
// glp_run_batch and the tick waits for them.  Every draw is keyed by the
// request's seed and generation, so its result does not depend on the mix.

struct glp_server {
  glp_ctx *c = nullptr;
  glp::ServerCore core;
};

int glp_server_create(glp_ctx *c, uint64_t budget_bytes, int plain, glp_server **out) {
  int rc = check_ctx(c);
  if (rc)
    return rc;
  if (!out)
    return fail(c, GLP_ERR_ARG, "out must be non-null");
  glp_server *s = new glp_server();
  s->c = c;
  s->core.budget = budget_bytes;
  s->core.plain = plain != 0;
  *out = s;
  return GLP_OK;
}

int glp_server_submit(glp_server *s, glp_problem *pb, const glp_generation_args *args,
                      uint32_t generations, uint64_t *request_id) {
  if (!s)
    return GLP_ERR_ARG;
  glp_ctx *c = s->c;
  if (!pb || pb->ctx != c || !args || generations == 0)
    return fail(c, GLP_ERR_ARG, "a request needs a problem of this context, args and "
                                "at least one generation");
  if (!args->hnew || (args->flags & GLP_GEN_NO_WORK))
    return fail(c, GLP_ERR_ARG, "a served request runs hmm_work: hnew is required");
  glp::ServerCore::Req r = glp::ServerCore::make(pb, *args, generations);
  if (r.bytes > s->core.budget)
    return fail(c, GLP_ERR_ARG, "request needs %llu bytes, more than the budget %llu",
                (unsigned long long)r.bytes, (unsigned long long)s->core.budget);
  // validate the first generation now (sizes, model inputs, buffers), so a
  // bad request is refused here rather than failing every later tick
  int rc = check_ctx(c);
  if (rc)
    return rc;
  const glp_generation_args first = glp::ServerCore::args_of(r);
  glp::GenParams scratch;
  if ((rc = make_params(c, pb, &first, &scratch)))
    return rc;
  const uint64_t id = s->core.add(r);
  if (request_id)
    *request_id = id;
  return GLP_OK;
}

int glp_server_tick(glp_server *s, uint32_t *resident, uint32_t *finished) {
  if (!s)
    return GLP_ERR_ARG;
  glp_ctx *c = s->c;
  int rc = check_ctx(c);
  if (rc)
    return rc;
  auto run = [c](const std::vector<glp::ServerCore::Launch> &launches) {
    for (const auto &l : launches) {
      std::vector<glp_problem *> pbs;
      for (void *p : l.problems)
        pbs.push_back(static_cast<glp_problem *>(p));
      const int r = glp_run_batch(c, (uint32_t)pbs.size(), pbs.data(), l.args.data());
      if (r)
        return r;
    }
    return glp_finish(c);
  };
  return s->core.tick(run, resident, finished);
}

int glp_server_poll(glp_server *s, uint64_t request_id, int *state, uint32_t *generations_done,
                    const uint64_t **haps) {
  if (!s)
    return GLP_ERR_ARG;
  const glp::ServerCore::Req *r = s->core.find(request_id);
  if (!r)
    return fail(s->c, GLP_ERR_ARG, "no request %llu", (unsigned long long)request_id);
  if (state)
    *state = r->state;
  if (generations_done)
    *generations_done = r->gen;
  if (haps)
    *haps = glp::ServerCore::current_haps(*r);
  return GLP_OK;
}

int glp_server_release(glp_server *s, uint64_t request_id) {
  if (!s)
    return GLP_ERR_ARG;
  switch (s->core.release(request_id)) {
  case 0:
    return GLP_OK;
  case 1:
    return fail(s->c, GLP_ERR_ARG, "no request %llu", (unsigned long long)request_id);
  default:
    return fail(s->c, GLP_ERR_STATE, "request %llu has not finished",
                (unsigned long long)request_id);
  }
}

int glp_server_stats(glp_server *s, uint64_t *ticks, uint64_t *updates, uint64_t *used_bytes) {
  if (!s)
    return GLP_ERR_ARG;
  if (ticks)
    *ticks = s->core.ticks;
  if (updates)
    *updates = s->core.updates;
  if (used_bytes)
    *used_bytes = s->core.used;
  return GLP_OK;
}

void glp_server_destroy(glp_server *s) { delete s; }

int glp_kernel_times(glp_ctx *c, uint32_t n, float *gen_ms, float *work_ms) {
  if (!c)
    return GLP_ERR_ARG;
  if (n > glp_ctx::kTimed || n > c->ev_count)
    return fail(c, GLP_ERR_ARG, "at most %u of the %llu timed generations are kept",
                glp_ctx::kTimed, (unsigned long long)c->ev_count);
  for (uint32_t i = 0; i < n; ++i) {
    cudaEvent_t *ev = c->ev[(c->ev_count - n + i) % glp_ctx::kTimed];
    float g = 0.f, w = 0.f;
    GLP_CUDA(c, cudaEventSynchronize(ev[2]));
    GLP_CUDA(c, cudaEventElapsedTime(&g, ev[0], ev[1]));
    GLP_CUDA(c, cudaEventElapsedTime(&w, ev[1], ev[2]));
    if (gen_ms)
      gen_ms[i] = g;
    if (work_ms)
      work_ms[i] = w;
  }
  return GLP_OK;
}

int glp_get_counters(glp_ctx *c, uint64_t *counters, uint32_t n) {
  if (!c)
    return GLP_ERR_ARG;
  if (!counters && n)
    return fail(c, GLP_ERR_ARG, "counters must be non-null");
  for (uint32_t i = 0; i < n; ++i)
    counters[i] = i < (uint32_t)glp::kStats ? c->last_stats[i] : 0;
  return GLP_OK;
}

int glp_tally(glp_ctx *c, const uint64_t *haps, uint32_t N, uint32_t S, uint32_t *hsum) {
  int rc = check_ctx(c);
  if (rc)
    return rc;
  if (!haps || !hsum || N == 0 || S == 0)
    return fail(c, GLP_ERR_ARG, "haps, hsum, num_samples and num_sites are required");
  glp::replace_kernel<<<N, glp::kTallyThreads, 0, c->stream>>>(haps, N, S, (S + 63) / 64, hsum);
  GLP_CUDA(c, cudaGetLastError());
  return GLP_OK;
}

int glp_result(glp_ctx *c, const uint32_t *hsum, uint32_t N, uint32_t S, uint32_t sn,
               float *prob_out) {
  int rc = check_ctx(c);
  if (rc)
    return rc;
  if (!hsum || !prob_out || N == 0 || S == 0 || sn == 0)
    return fail(c, GLP_ERR_ARG, "hsum, prob_out, sizes and sampling_generations are required");
  const uint64_t total = (uint64_t)2 * N * S;
  const float norm = (float)(1.0 / sn);
  glp::result_kernel<<<(unsigned)((total + 255) / 256), 256, 0, c->stream>>>(hsum, N, S, norm,
                                                                          prob_out);
  GLP_CUDA(c, cudaGetLastError());
  return GLP_OK;
}

int glp_vq_train(glp_ctx *c, const float *gl, uint64_t P, uint32_t K, float *codebook,
                 uint64_t seed, uint32_t max_iter, uint32_t *iterations) {
  int rc = check_ctx(c);
  if (rc)
    return rc;
  if (!gl || !codebook || P == 0)
    return fail(c, GLP_ERR_ARG, "gl, codebook and num_gls are required");
  if (K < 4 || K > (uint32_t)glp::kVQMaxCodes)
    return fail(c, GLP_ERR_ARG, "codebook_size=%u must be in [4, %d]", K, glp::kVQMaxCodes);
  const uint64_t nb64 = (P + glp::kVQBlock - 1) / glp::kVQBlock;
  if (nb64 > 0x7fffffffu)
    return fail(c, GLP_ERR_ARG, "num_gls=%llu is too large", (unsigned long long)P);
  const uint32_t nb = (uint32_t)nb64;
  const size_t smem = glp::vq_assign_smem(K);
  GLP_CUDA(c, cudaFuncSetAttribute(glp::vq_assign_kernel,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  double *d_sums = nullptr, *d_var = nullptr;
  uint32_t *d_counts = nullptr;
  float2 *d_cb = nullptr;
  if (cudaMalloc((void **)&d_sums, (size_t)nb * (2 * K + 1) * sizeof(double)) != cudaSuccess ||
      cudaMalloc((void **)&d_counts, (size_t)nb * K * sizeof(uint32_t)) != cudaSuccess ||
      cudaMalloc((void **)&d_cb, K * sizeof(float2)) != cudaSuccess ||
      cudaMalloc((void **)&d_var, sizeof(double)) != cudaSuccess) {
    release(d_sums);
    release(d_counts);
    release(d_cb);
    release(d_var);
    return fail(c, GLP_ERR_NOMEM, "codebook training scratch");
  }
  cudaStream_t st = c->stream;
  auto assign = [&] {
    glp::vq_assign_kernel<<<nb, glp::kVQThreads, smem, st>>>(gl, P, d_cb, K, d_sums, d_counts);
  };
  // totals of the last assignment: its squared distance, and with `move` the
  // next entries (iteration `it`)
  auto totals = [&](uint32_t it, bool move, double *var) -> cudaError_t {
    glp::vq_update_kernel<<<1, 64, 0, st>>>(gl, P, nb, d_sums, d_counts, K, seed, it,
                                            move ? d_cb : nullptr, d_var);
    cudaError_t e = cudaMemcpyAsync(var, d_var, sizeof(double), cudaMemcpyDeviceToHost, st);
    return e == cudaSuccess ? cudaStreamSynchronize(st) : e;
  };
  cudaError_t e = cudaMemcpyAsync(d_cb, codebook, K * sizeof(float2), cudaMemcpyHostToDevice, st);
  double cur = 0.0, prev = std::numeric_limits<double>::max(), dummy = 0.0;
  uint32_t it = 0;
  if (e == cudaSuccess) {
    assign();
    e = totals(0, false, &cur);
  }
  // GLVQ::BuildCodeBook's loop (glVQ.cpp:78-89)
  while (e == cudaSuccess && std::fabs(cur - prev) > cur / 100) {
    if (++it > max_iter) {
      rc = fail(c, GLP_ERR_NO_CONVERGE,
                "[GLVQ] Clustering failed to converge within %u iterations", max_iter);
      break;
    }
    prev = cur;
    e = totals(it, true, &dummy);
    if (e != cudaSuccess)
      break;
    assign();
    e = totals(it, false, &cur);
  }
  if (e == cudaSuccess && rc == GLP_OK)
    e = cudaMemcpy(codebook, d_cb, K * sizeof(float2), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess)
    e = cudaGetLastError();
  release(d_sums);
  release(d_counts);
  release(d_cb);
  release(d_var);
  if (e != cudaSuccess)
    return fail(c, GLP_ERR_CUDA, "codebook training: %s", cudaGetErrorString(e));
  if (iterations)
    *iterations = std::min(it, max_iter);
  return rc;
}

int glp_vq_pack(glp_ctx *c, const float *gl, uint32_t N, uint32_t S, const float *codebook,
                uint32_t K, uint32_t bits, uint32_t *packed) {
  int rc = check_ctx(c);
  if (rc)
    return rc;
  if (!gl || !codebook || !packed || N == 0 || S == 0)
    return fail(c, GLP_ERR_ARG, "gl, codebook, packed_out and sizes are required");
  if (K < 4 || K > (uint32_t)glp::kVQMaxCodes)
    return fail(c, GLP_ERR_ARG, "codebook_size=%u must be in [4, %d]", K, glp::kVQMaxCodes);
  if ((bits != 2 && bits != 4 && bits != 8) || (1u << bits) < K)
    return fail(c, GLP_ERR_ARG, "bits=%u must be 2, 4 or 8 with 2^bits >= codebook_size=%u",
                bits, K);
  glp::VQBook book;
  for (uint32_t k = 0; k < K; ++k)
    book.e[k] = make_float2(codebook[2 * k], codebook[2 * k + 1]);
  const uint32_t per = 32u / bits;
  const uint64_t total = (uint64_t)((S + per - 1) / per) * N;
  glp::vq_pack_kernel<<<(unsigned)((total + 255) / 256), 256, 0, c->stream>>>(gl, N, S, book, K,
                                                                            bits, packed);
  GLP_CUDA(c, cudaGetLastError());
  return GLP_OK;
}

int glp_knn_neighbors(glp_ctx *c, const uint64_t *haps, uint32_t H, uint32_t S, uint32_t k,
                      double lb, double ub, int use_maf, uint32_t *neighbors) {
  int rc = check_ctx(c);
  if (rc)
    return rc;
  if (!haps || !neighbors || S == 0 || k == 0)
    return fail(c, GLP_ERR_ARG, "haps, neighbors, num_sites and k are required");
  const uint32_t half = (k + 1) / 2;
  if (H < 4 || (H & 1u) || H > glp::kKnnMaxHaps)
    return fail(c, GLP_ERR_ARG, "num_haps=%u must be even and in [4, %u]", H,
                glp::kKnnMaxHaps);
  if (2 * half > H - 2 || half > glp::kKnnMaxHalf)
    return fail(c, GLP_ERR_ARG, "k=%u needs 2*ceil(k/2) <= num_haps-2 and <= %u", k,
                2 * glp::kKnnMaxHalf);
  if (S >= 0xffffu)
    return fail(c, GLP_ERR_ARG, "num_sites must be below 65535 for kNN");
  const uint32_t wn = (S + 63) / 64;
  if ((rc = ensure(c, c->d_mask, c->mask_cap, wn)))
    return rc;
  glp::common_sites_kernel<<<wn, 64, 0, c->stream>>>(haps, H, wn, S, lb, ub, use_maf,
                                                     c->d_mask);
  GLP_CUDA(c, cudaGetLastError());
  const size_t smem = glp::knn_smem_bytes(H);
  // tiled distances of a chunk of samples (at most 256 MB of them) into
  // global memory, then the selection, chunk by chunk
  GLP_CUDA(c, cudaFuncSetAttribute(glp::knn_select_kernel,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const uint32_t NS = H / 2;
  const uint32_t chunk =
      (uint32_t)std::min<size_t>(NS, std::max<size_t>(64, ((size_t)256 << 20) / (4 * (size_t)H)));
  if ((rc = ensure(c, c->d_knn_dist, c->knn_dist_cap, (size_t)2 * chunk * H)))
    return rc;
  const bool tract = c->knn_metric == GLP_KNN_TRACT;
  for (uint32_t s0 = 0; s0 < NS; s0 += chunk) {
    const uint32_t n = std::min(chunk, NS - s0);
    if (tract) {
      const dim3 grid((H + glp::kTractH - 1) / glp::kTractH,
                      (2 * n + glp::kTractQ - 1) / glp::kTractQ);
      glp::knn_tract_dist_kernel<<<grid, glp::kDistThreads, 0, c->stream>>>(
          haps, H, wn, c->d_mask, 2 * s0, 2 * n, c->d_knn_dist);
    } else {
      const dim3 grid((H + glp::kDistH - 1) / glp::kDistH,
                      (2 * n + glp::kDistQ - 1) / glp::kDistQ);
      glp::knn_dist_kernel<<<grid, glp::kDistThreads, 0, c->stream>>>(haps, H, wn, c->d_mask,
                                                                      2 * s0, 2 * n,
                                                                      c->d_knn_dist);
    }
    glp::knn_select_kernel<<<n, glp::kKnnThreads, smem, c->stream>>>(c->d_knn_dist, H, s0, half,
                                                                    S, neighbors);
    GLP_CUDA(c, cudaGetLastError());
  }
  return GLP_OK;
}

}  // extern "C"

namespace {

// 8 independent FMA chains per thread; the result is stored so nothing is
// eliminated.
__global__ void __launch_bounds__(256) fp32_probe_kernel(float *out, int iters, float a,
                                                         float b) {
  float x0 = threadIdx.x * 1e-7f, x1 = x0 + 1e-7f, x2 = x0 + 2e-7f, x3 = x0 + 3e-7f;
  float x4 = x0 + 4e-7f, x5 = x0 + 5e-7f, x6 = x0 + 6e-7f, x7 = x0 + 7e-7f;
#pragma unroll 4
  for (int i = 0; i < iters; ++i) {
    x0 = fmaf(x0, a, b);
    x1 = fmaf(x1, a, b);
    x2 = fmaf(x2, a, b);
    x3 = fmaf(x3, a, b);
    x4 = fmaf(x4, a, b);
    x5 = fmaf(x5, a, b);
    x6 = fmaf(x6, a, b);
    x7 = fmaf(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
}

}  // namespace

extern "C" int glp_measure_fp32_peak(glp_ctx *c, float ms_target, double *tflops) {
  int rc = check_ctx(c);
  if (rc)
    return rc;
  if (!tflops || !(ms_target > 0))
    return fail(c, GLP_ERR_ARG, "tflops must be non-null and ms_target positive");
  const int threads = 256, blocks = c->sms * 8;
  float *out = nullptr;
  GLP_CUDA(c, cudaMalloc((void **)&out, sizeof(float) * threads * blocks));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int iters = 1 << 14;
  double best = 0;
  for (int rep = 0; rep < 6; ++rep) {
    cudaEventRecord(e0, c->stream);
    fp32_probe_kernel<<<blocks, threads, 0, c->stream>>>(out, iters, 0.999999f, 1e-7f);
    cudaEventRecord(e1, c->stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    const double flops = 2.0 * 8.0 * iters * (double)threads * blocks;
    if (rep >= 2)
      best = std::max(best, flops / (ms * 1e-3) / 1e12);
    if (ms > 0 && ms < ms_target)
      iters = (int)std::min<double>(iters * (ms_target / ms), 1 << 26);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  GLP_CUDA(c, cudaGetLastError());
  *tflops = best;
  return GLP_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free generation (glp_run_generation_noalloc).
//
// The scratch of one generation lives in a file-scope device array instead
// of memory from cudaMalloc.  Layout, in bytes from the start:
//   [0, 4)     work-queue counter          (cleared by every call)
//   [8, 56)    generation counters, 6 x uint64 (cleared by every call)
//   [64, 68)   device error flag           (cleared by every call)
//   [256, 256 + round_up(16 (S + 1), 256))  transition table, float4 [S + 1]
//   then       hmm_work rows, float4 [N][S] (written before they are read)
// Host code never dereferences g_noalloc_scratch: its name there is a host
// stand-in.  The array's device address belongs to a CUDA context, so it is
// looked up with cudaGetSymbolAddress once per context, with that context
// current (for the usual primary context: once per device), and cached under
// the context's unique id (cuCtxGetId), together with the launch set-up of
// the kernels (shared-memory attributes, resident threads per lane width).
// A context created later -- after cudaDeviceReset, or one a caller made with
// the driver API -- has another id and gets its own lookup.

namespace {

__device__ __align__(256) unsigned char g_noalloc_scratch[GLP_NOALLOC_SCRATCH_BYTES];

// Set-up of one CUDA context: the scratch array's device address there and
// the generation kernel's resident threads per lane width 1 .. 32.
struct NoallocSetup {
  unsigned long long ctx_id = 0;  // 0: slot unused
  unsigned char *base = nullptr;
  int sms = 0;
  double resident[6] = {};
};
constexpr int kNoallocContexts = 16;
std::mutex g_noalloc_mutex;
NoallocSetup g_noalloc_setup[kNoallocContexts];
unsigned g_noalloc_next = 0;

// Driver entry points (through the runtime, so the library needs no link to
// libcuda): the current context and its process-unique id.
using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_id = nullptr;
bool g_ctx_fns_loaded = false;

// Id of the calling thread's current context (0 if there is none or the
// driver cannot tell); call with g_noalloc_mutex held.
unsigned long long current_ctx_id() {
  if (!g_ctx_fns_loaded) {
    g_ctx_fns_loaded = true;
    void *f1 = nullptr, *f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault,
                                         &q1) == cudaSuccess &&
        q1 == cudaDriverEntryPointSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) ==
            cudaSuccess &&
        q2 == cudaDriverEntryPointSuccess) {
      g_ctx_current = reinterpret_cast<CtxGetCurrentFn>(f1);
      g_ctx_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!g_ctx_current || g_ctx_current(&ctx) != CUDA_SUCCESS || !ctx ||
      g_ctx_id(ctx, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

// The set-up of the caller's current context, made on first use; a copy is
// returned so no lock is held while the call launches.
int noalloc_setup(NoallocSetup *out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  unsigned long long id = current_ctx_id();
  if (id) {
    for (const NoallocSetup &e : g_noalloc_setup)
      if (e.ctx_id == id) {
        *out = e;
        return GLP_OK;
      }
  }
  NoallocSetup e;
  void *p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p)
    return GLP_ERR_CUDA;
  e.base = static_cast<unsigned char *>(p);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&e.sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      allow_chain_smem() != cudaSuccess)
    return GLP_ERR_CUDA;
  for (int i = 1; i < 6; ++i) {  // also sets each kernel's shared-memory attribute
    Shape sh;
    sh.P = 1u << i;
    e.resident[i] = resident_threads(single_kernel(sh, false), sh.P, e.sms);
    if (e.resident[i] <= 0)
      return GLP_ERR_CUDA;
  }
  // the lookup above made a context current if there was none
  e.ctx_id = id ? id : current_ctx_id();
  if (e.ctx_id) {
    g_noalloc_setup[g_noalloc_next] = e;
    g_noalloc_next = (g_noalloc_next + 1) % kNoallocContexts;
  }
  *out = e;
  return GLP_OK;
}

// Kernel layout of the reference's tran [S][3] (row 0 unused,
// hmmLike.cu:325): S + 1 rows, rows 0 and S the identity (the forward pass
// starts from row 0 so that the first step reproduces l = e / 4; the backward
// pass starts from row S); the fourth component is t0 - t2.  The same rows
// follow as (t1, t2, t0 - t2, t0 - t2) for the blocked recursion.
__global__ void tran4_kernel(const float *__restrict__ tran, uint32_t S,
                             float4 *__restrict__ out) {
  const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m <= S) {
    const float4 r = (m && m < S) ? make_float4(tran[3 * m], tran[3 * m + 1], tran[3 * m + 2],
                                                __fsub_rn(tran[3 * m], tran[3 * m + 2]))
                                  : make_float4(1.f, 0.f, 0.f, 1.f);
    out[m] = r;
    out[S + 1 + m] = make_float4(r.y, r.z, r.w, r.w);
  }
}

size_t round256(size_t x) { return (x + 255) & ~(size_t)255; }

static_assert(8 + glp::kStats * sizeof(unsigned long long) <= 64,
              "generation counters overlap the error flag in the scratch layout");

}  // namespace

extern "C" int glp_run_generation_noalloc(const glp_generation_args *a, const float *tran,
                                          const float *pc16, const float *emit,
                                          const float *prob, void *stream) {
  if (!a || !tran || !pc16 || !emit || !a->haps || !a->hap_idxs_out)
    return GLP_ERR_ARG;
  const uint32_t N = a->num_samples, S = a->num_sites, C = a->num_cycles, H = a->num_haps;
  const bool work = (a->flags & GLP_GEN_NO_WORK) == 0;
  if (N == 0 || S == 0 || H < 2 || (uint64_t)2 * N > H || (a->flags & GLP_GEN_VQ))
    return GLP_ERR_ARG;
  if ((work && (!a->hnew || !prob)) || ((uintptr_t)emit & 15u))
    return GLP_ERR_ARG;
  if (!(a->pen > 0.0f) || !std::isfinite(a->pen))
    return GLP_ERR_ARG;
  const bool tr = a->trace_slot || a->trace_accept || a->trace_work;
  if (tr && !(a->trace_slot && a->trace_accept && a->trace_work))
    return GLP_ERR_ARG;
  uint32_t lo = a->sample_lo, hi = a->sample_hi;
  if (lo == 0 && hi == 0)
    hi = H;
  if ((!a->hap_idxs_in || (C && !a->props)) && !a->neighbors &&
      (hi > H || lo >= hi || hi - lo < 3))
    return GLP_ERR_ARG;
  if (a->neighbors && a->neighbors_per_sample == 0)
    return GLP_ERR_ARG;
  const bool draws = !a->hap_idxs_in || (C && !a->props);
  const bool kick_first = (a->flags & GLP_GEN_KICK_FIRST) != 0;
  if (kick_first && draws && C && H < 2 * N + 1)  // as make_params
    return GLP_ERR_ARG;
  const size_t tran_off = 256, beta_off = tran_off + round256((size_t)32 * (S + 1));
  const size_t need = beta_off + (work ? (size_t)16 * N * S : 0);
  if (need > GLP_NOALLOC_SCRATCH_BYTES)
    return GLP_ERR_TOO_LARGE;

  NoallocSetup su;
  const int src = noalloc_setup(&su);
  if (src)
    return src;
  unsigned char *const base = su.base;
  const int sms = su.sms;
  cudaStream_t st = (cudaStream_t)stream;

  glp::GenParams p;
  std::memset(&p, 0, sizeof(p));
  p.N = N;
  p.S = S;
  p.C = C;
  p.H = H;
  p.wn = (S + 63) / 64;
  p.emit_mode = GLP_EMIT_FLOAT;
  p.haps = a->haps;
  p.hnew = a->hnew;
  p.emit = reinterpret_cast<const float4 *>(emit);
  p.prob = prob;
  p.tran4 = reinterpret_cast<const float4 *>(base + tran_off);
  p.tranp = p.tran4 + (S + 1);
  p.quad_in = a->hap_idxs_in;
  p.quad_out = a->hap_idxs_out;
  p.props = a->props;
  p.tr_slot = a->trace_slot;
  p.tr_u = a->trace_accept;
  p.tr_work = a->trace_work;
  p.like_out = a->like_out;
  p.eval_trace = a->eval_trace;
  p.accept_trace = a->accept_trace;
  p.beta = reinterpret_cast<float4 *>(base + beta_off);
  p.counter = reinterpret_cast<uint32_t *>(base);
  p.stats = reinterpret_cast<unsigned long long *>(base + 8);
  p.error = reinterpret_cast<int *>(base + 64);
  p.nbr = a->neighbors;
  p.klen = a->neighbors_per_sample;
  p.samp_lo = lo;
  p.samp_hi = hi;
  p.kick_first = kick_first ? 1u : 0u;
  std::memcpy(p.pc, pc16, sizeof(p.pc));
  p.pen = a->pen;
  p.seed = a->seed;
  p.generation = a->generation;
  p.do_work = work ? 1u : 0u;

  // speculation width for an acceptance rate of about 0.12 (the rule of
  // choose_lanes without a context's history), from the resident threads
  // measured at set-up
  bool known = true;
  const uint32_t P = pick_lanes(
      0.12, N, sms,
      [](uint32_t w) {
        Shape s1;
        s1.P = w;
        return (const void *)single_kernel(s1, false);
      },
      su.resident, &known);
  Shape sh;
  sh.P = P;
  SingleFn fn = single_kernel(sh, false);
  const size_t smem = glp::stage_bytes((int)P);
  const uint64_t resident_blocks =
      (uint64_t)(su.resident[__builtin_ctz(P)] / glp::kThreads + 0.5);
  const uint64_t groups = (uint64_t)glp::kThreads / P;
  const uint64_t want = ((uint64_t)N + groups - 1) / groups;
  const unsigned grid = (unsigned)std::max<uint64_t>(
      1, std::min<uint64_t>(want, std::max<uint64_t>(resident_blocks, (uint64_t)sms)));

  if (cudaMemsetAsync(base, 0, 256, st) != cudaSuccess)
    return GLP_ERR_CUDA;
  tran4_kernel<<<(S + 256) / 256, 256, 0, st>>>(tran, S, (float4 *)(base + tran_off));
  fn<<<grid, glp::kThreads, smem, st>>>(p);
  if (work)
    launch_work(p, N, st);
  if (cudaGetLastError() != cudaSuccess)
    return GLP_ERR_CUDA;
  int h_err = 0;
  if (cudaMemcpyAsync(&h_err, base + 64, sizeof(int), cudaMemcpyDeviceToHost, st) !=
          cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return GLP_ERR_CUDA;
  return h_err ? GLP_ERR_INDEX : GLP_OK;
}
