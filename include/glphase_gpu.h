/*
 * glphase_gpu.h -- C ABI of the GB300 (sm_103a) implementation of GLPhase's
 * per-sample MH/HMM hot path.  Plain pointers and sizes only; every entry
 * point returns a glp_status code and never exits or throws.
 *
 * The entry points replace the reference's device API, namespace HMMLikeCUDA
 * in src/hmmLike.h:23-38 (implemented in src/hmmLike.cu).  Each declaration
 * names the reference function it stands in for.  A header-only C++ shim with
 * the reference's exact signatures lives in include/hmmlike_cuda_shim.hpp,
 * so src/hmmLike.cpp and Insti::cudaSolve compile against this library
 * unchanged.
 *
 * Array layouts (row-major):
 *   haps          uint64 [H][wn], wn = ceil(S/64); site m -> word m>>6,
 *                 bit m&63; haplotypes 2i and 2i+1 belong to sample i,
 *                 panel haplotypes follow at 2N.. (src/impute.hpp:53-66,
 *                 src/insti.cpp:1395-1403)
 *   hap_idxs      uint32 [4][N] (father0, father1, mother0, mother1)
 *                 (src/hmmLike.cpp:81)
 *   props         uint32 [C][N] proposal haplotypes (src/hmmLike.cpp:86)
 *   tran          float  [S][3] (row 0 unused) (src/insti.cpp:1277-1300)
 *   pc            float  [4][4] row-major mutation matrix pc[i][j]
 *   emit          float  [N][S][4], prob float [N][S][3] (homRef, het,
 *                 homAlt) (src/insti.cpp:1345-1382)
 *   packed GLs    uint32 [ceil(S/8)][N], eight 4-bit codes per word, most
 *                 significant nibble first (src/glPack.cpp:112-165)
 *   codebook      float  [16][2] (homRef, het) (src/hmmLike.cu:369-383)
 */
#ifndef GLPHASE_GPU_H
#define GLPHASE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum glp_status {
  GLP_OK = 0,
  GLP_ERR_ARG = 1,      /* invalid argument or size mismatch */
  GLP_ERR_CUDA = 2,     /* a CUDA runtime call failed */
  GLP_ERR_NOMEM = 3,    /* device allocation failed */
  GLP_ERR_STATE = 4,    /* a required model input was not set */
  GLP_ERR_INDEX = 5,    /* a haplotype index >= num_haps reached the device */
  GLP_ERR_DEVICE = 6,   /* no usable device */
  GLP_ERR_TOO_LARGE = 7, /* problem exceeds the fixed scratch of glp_run_generation_noalloc */
  GLP_ERR_NO_CONVERGE = 8 /* codebook training did not converge within max_iter iterations */
} glp_status;

typedef struct glp_ctx glp_ctx;

/* Emission source of the MH likelihood. */
#define GLP_EMIT_FLOAT 0u /* float emit [N][S][4]: Impute::hmm_like semantics */
#define GLP_EMIT_VQ 1u    /* 4-bit VQ GL codes: HMMLikeCUDA::hmmLike semantics */

/* glp_generation_args.flags */
#define GLP_GEN_VQ 1u      /* score with the VQ codes (else float emit) */
#define GLP_GEN_NO_WORK 2u /* skip the fused hmm_work (hnew untouched) */
/* draw every chain's first proposal from the panel rows [2N, H) (the
 * reference's --kickstart, src/insti.cpp:1505-1511); in-kernel draws only */
#define GLP_GEN_KICK_FIRST 4u

/* One MH generation over all N samples. */
typedef struct glp_generation_args {
  uint32_t num_samples; /* N */
  uint32_t num_sites;   /* S: must equal the S of the model inputs */
  uint32_t num_cycles;  /* C */
  uint32_t num_haps;    /* H: rows of haps/hnew, all indices must be < H */
  const uint64_t *haps; /* [H][wn] current haplotypes (read only) */
  uint64_t *hnew;       /* [H][wn] rows 2i,2i+1 receive the new haplotypes */
  const uint32_t *hap_idxs_in; /* [4][N] initial quadruples */
  uint32_t *hap_idxs_out;      /* [4][N] final quadruples (may alias in) */
  const uint32_t *props;       /* [C][N] proposals */
  float pen;                   /* MH and hmm_work penalty (src/insti.cpp:1670) */
  uint64_t seed;               /* key of the counter-based random streams */
  uint32_t generation;         /* counter of the random streams */
  uint32_t flags;              /* GLP_GEN_* */
  /* optional replay trace (all three or none): */
  const uint8_t *trace_slot;   /* [N][C] replaced slot (0..3) */
  const double *trace_accept;  /* [N][C] accept uniforms */
  const float *trace_work;     /* [N][S] hmm_work uniforms */
  /* optional outputs: */
  double *like_out;            /* [N] final log-likelihood of each chain */
  double *eval_trace;          /* [N][C+1] every evaluated log-likelihood */
  uint8_t *accept_trace;       /* [N][C] accept decisions */
  /* Device-side surrogate draws, used for whichever of hap_idxs_in / props
   * is NULL: the 4 initial and C proposal haplotypes of each sample are drawn
   * in the kernel from the counter-based streams, from the neighbour table
   * when given (KNN::SampleHap, src/kNN.cpp:74-90), else uniformly over
   * [sample_lo, sample_hi) minus the sample's own pair
   * (UnifSampler::SampleHap, src/sampler.cpp:29-39); 0,0 means [0, H).
   * Replaces the host draws of RunHMMOnSamples (src/hmmLike.cpp:90-102). */
  const uint32_t *neighbors;     /* [N][neighbors_per_sample] device, or NULL */
  uint32_t neighbors_per_sample;
  uint32_t sample_lo, sample_hi;
  /* Used by prepared batches advancing on the device (glp_batch_run):
   * burnin > 0 recomputes pen = min((generation+1)/burnin, 1)^2 each
   * generation (src/insti.cpp:1670-1671); kick_start = 1 limits the
   * surrogates to [sample_lo, sample_hi) in the first generation only, then
   * [0, sample_hi) (README "kickstart" semantics). */
  uint32_t burnin;
  uint32_t kick_start;
} glp_generation_args;

/* Number of visible CUDA devices and whether device `device` is an sm_103
 * part.  Replaces HMMLikeCUDA::CheckDevice (src/hmmLike.cu:266-320). */
int glp_check_device(int device, int *device_count, int *cc_major, int *cc_minor,
                     int *sm_count);

/* Create a context on `device`.  Replaces HMMLikeCUDA::SetDevice and
 * InitializeConstants (src/hmmLike.cu:228-264). */
int glp_create(int device, glp_ctx **out);

/* Free every device buffer of the context; the device itself is not reset.
 * Replaces HMMLikeCUDA::Cleanup (src/hmmLike.cu:385-397). */
void glp_destroy(glp_ctx *ctx);

/* Message of the last failed call on this context (never NULL). */
const char *glp_last_error(const glp_ctx *ctx);

/* Bind the context to a CUDA stream (cudaStream_t; NULL = the context's own
 * stream).  Device-pointer calls are asynchronous on that stream.  The model
 * set-up calls (glp_set_tran, glp_set_mutation_mat, glp_set_codebook,
 * glp_set_packed_gls, glp_set_emission, glp_problem_set_model,
 * glp_problem_set_vq) copy synchronously and first wait for the work already
 * on that stream, so generations enqueued before them read the old data. */
int glp_set_stream(glp_ctx *ctx, void *stream);

/* Transition matrix tran [S][3].  Replaces HMMLikeCUDA::CopyTranToDevice
 * (src/hmmLike.cu:322-337); S is no longer capped at NUMSITES=1024. */
int glp_set_tran(glp_ctx *ctx, const float *tran, uint32_t num_sites);

/* Mutation matrix pc[4][4], row-major.  Replaces
 * HMMLikeCUDA::CopyMutationMatToDevice (src/hmmLike.cu:339-355). */
int glp_set_mutation_mat(glp_ctx *ctx, const float *pc16);

/* VQ codebook [entries][2], entries = 16.  Replaces
 * HMMLikeCUDA::CopyCodeBookToDevice (src/hmmLike.cu:368-383). */
int glp_set_codebook(glp_ctx *ctx, const float *codebook, uint32_t entries);

/* Packed VQ GLs [ceil(S/8)][N].  Replaces HMMLikeCUDA::CopyPackedGLsToDevice
 * (src/hmmLike.cu:357-366). */
int glp_set_packed_gls(glp_ctx *ctx, const uint32_t *packed, size_t num_words);

/* Float emission [N][S][4] and genotype probabilities [N][S][3] from the
 * host (Insti::initialize's emit and prob, src/insti.cpp:1345-1382): the
 * inputs of Impute::hmm_like and of the fused hmm_work.  prob may be NULL
 * when hmm_work is never run: a generation that runs it is then refused with
 * GLP_ERR_STATE until genotype probabilities are set with the emissions. */
int glp_set_emission(glp_ctx *ctx, const float *emit, const float *prob, uint32_t num_samples,
                     uint32_t num_sites);

/* The reference's device call, host buffers in and out: MH over numCycles
 * proposals per sample with VQ-decoded emissions and accept penalty 1,
 * no hmm_work; hap_idxs [4][N] in/out.  Replaces HMMLikeCUDA::RunHMMOnDevice
 * (src/hmmLike.cu:399-572).  The panel may hold fewer rows than the context
 * was sized for; all indices are checked against panel_words / wn. */
int glp_run_hmm_on_device(glp_ctx *ctx, const uint64_t *hap_panel, size_t panel_words,
                          const uint32_t *extra_prop_haps, uint32_t num_sites,
                          uint32_t num_samples, uint32_t num_cycles, uint32_t *hap_idxs,
                          uint64_t seed);

/* One generation with the fused hmm_work, all array pointers DEVICE
 * pointers, asynchronous on the context stream.  Call glp_finish() to wait
 * and collect device-side errors.  Replaces RunHMMOnDevice plus the OpenMP
 * hmm_work loop of Insti::cudaSolve (src/insti.cpp:1433-1463). */
int glp_run_generation(glp_ctx *ctx, const glp_generation_args *args);

/* The same generation with HOST pointers: copies inputs in, runs, copies
 * quadruples, hnew rows of the N samples and the optional outputs back,
 * synchronously. */
int glp_run_generation_host(glp_ctx *ctx, const glp_generation_args *args);

/* Wait for the context stream and report device-side errors. */
int glp_finish(glp_ctx *ctx);

/* Lanes that score one sample's chain speculatively: 2, 4, 8, 16 or 32, as
 * lane pairs that each score one chain position a round (one lane the
 * forward half of the sites, the other the backward half); 1 is taken as 2
 * (one position a round: the sequential chain); 0 = choose from the last
 * generation's acceptance rate. */
int glp_set_lanes_per_sample(glp_ctx *ctx, uint32_t lanes);

/* Evaluations each lane pair scores per speculative round: 1 (or 0, the
 * same); other values are refused with GLP_ERR_ARG.  No reference
 * counterpart (a tuning knob of the speculative scheme). */
int glp_set_evals_per_lane(glp_ctx *ctx, uint32_t evals);

/* Sites per normalisation block of the likelihood (no counterpart in the
 * reference, which rescales site by site): 8 or 4, or 0 = automatic (8 until
 * a generation finished by glp_finish recomputed more than 0.1 % of its
 * evaluations site by site, then 4 for the rest of the context's life).
 * Very confident GLs can shrink an 8-site block beyond the range one
 * normalisation covers; such evaluations are recomputed site by site
 * (counters[3] of glp_get_counters), which 4-site blocks almost never need,
 * at about 4 % more arithmetic.  Results are the same either way.
 * glp_get_block_sites reports the size the next launch uses. */
int glp_set_block_sites(glp_ctx *ctx, uint32_t sites);
int glp_get_block_sites(glp_ctx *ctx, uint32_t *sites);

/* Evaluations (scored quadruples, speculative ones included) and speculative
 * rounds of the most recent generation (after glp_finish). */
int glp_get_stats(glp_ctx *ctx, uint64_t *evaluations, uint64_t *rounds,
                  uint32_t *lanes_used);

/* Generation counters of the most recent generation (after glp_finish), the
 * first n of: [0] scored evaluations, [1] speculative rounds, [2] accepted
 * proposals, [3] evaluations recomputed site by site (a block left the
 * normalisation range), [4] warp rounds, [5] active lanes summed over warp
 * rounds.  Entries past the sixth are 0.  No reference counterpart
 * (diagnostics of the speculative kernel). */
int glp_get_counters(glp_ctx *ctx, uint64_t *counters, uint32_t n);

/* Device time of the last n generations launched by glp_run_generation or
 * glp_run_batch (n <= 64, oldest first): the generation kernel (gen_ms) and
 * the two hmm_work kernels (work_ms), from CUDA events on the launching
 * stream; waits for those generations to finish.  No reference counterpart
 * (measurement support). */
int glp_kernel_times(glp_ctx *ctx, uint32_t n, float *gen_ms, float *work_ms);

/* ---- Many phasing chunks per launch (no reference counterpart: the
 * reference runs one chunk per RunHMMOnDevice call, src/hmmLike.cu:399). ----
 * A problem holds one chunk's device-resident model inputs, the same ones
 * glp_set_tran / glp_set_mutation_mat / glp_set_emission / glp_set_codebook /
 * glp_set_packed_gls give the context's own chunk. */
typedef struct glp_problem glp_problem;

int glp_problem_create(glp_ctx *ctx, glp_problem **out);
void glp_problem_destroy(glp_problem *pb);

/* tran [S][3], pc [4][4], emit [N][S][4], prob [N][S][3] (prob may be NULL
 * when hmm_work is never run); host arrays, copied to the device. */
int glp_problem_set_model(glp_problem *pb, const float *tran, const float *pc16,
                          const float *emit, const float *prob, uint32_t num_samples,
                          uint32_t num_sites);

/* The same with emit and prob already in device memory: the problem borrows
 * the two DEVICE arrays (no copy); the caller keeps them alive until the
 * problem is destroyed or given new ones.  tran and pc are host arrays. */
int glp_problem_set_model_device(glp_problem *pb, const float *tran, const float *pc16,
                                 const float *emit_dev, const float *prob_dev,
                                 uint32_t num_samples, uint32_t num_sites);

/* VQ codes [ceil(S/8)][N] and codebook [16][2] (host arrays). */
int glp_problem_set_vq(glp_problem *pb, const uint32_t *packed, size_t num_words,
                       const float *codebook);

/* One generation of `count` chunks of any sizes in ONE persistent launch:
 * args[i] (device pointers, as for glp_run_generation) runs on problems[i].
 * The samples of all chunks share one work queue.  Asynchronous; finish with
 * glp_finish().  All chunks use the same emission source (GLP_GEN_VQ or
 * not).  Each chunk's results equal those of the same generation run alone
 * (glp_run_generation): every draw is keyed by the chunk's own seed. */
int glp_run_batch(glp_ctx *ctx, uint32_t count, glp_problem *const *problems,
                  const glp_generation_args *args);

/* A prepared batch: the chunk descriptors live on the device and each run
 * performs one generation of every chunk and then advances all chunks to
 * their next generation on the device (haps <-> hnew swap, generation + 1,
 * penalty schedule, kick-start end).  glp_batch_run replays a CUDA graph
 * captured at preparation (reset counters, the persistent generation kernel,
 * the advance kernel): no host work per generation.  glp_batch_launch issues
 * the same work as plain launches.  Both are asynchronous on the context
 * stream; glp_finish() waits and reports device errors.  The lanes per
 * sample are fixed at preparation. */
typedef struct glp_batch glp_batch;

int glp_batch_prepare(glp_ctx *ctx, uint32_t count, glp_problem *const *problems,
                      const glp_generation_args *args, glp_batch **out);
int glp_batch_run(glp_batch *batch);
int glp_batch_launch(glp_batch *batch);
void glp_batch_destroy(glp_batch *batch);

/* ---- Request server: continuous batching (no reference counterpart: the
 * reference phases one chunk per process, src/insti.cpp:1557-1728). ----
 * A request is a problem, a generation template and a generation count G.
 * Requests wait in arrival order; each glp_server_tick admits the waiting
 * requests whose device footprint, N*S*44 + 2*H*ceil(S/64)*8 bytes
 * (emission, genotype probabilities, hmm_work scratch, both haplotype
 * buffers), fits what is left of budget_bytes, runs one generation of every
 * resident request -- all in one glp_run_batch launch (one per emission
 * source, float or GLP_GEN_VQ, when both are resident), or one glp_run_batch
 * launch per request when `plain` -- waits for it, and retires the requests
 * that have run G generations.  Generation g of a request takes the
 * template with generation = g; pen = min((g+1)/burnin, 1)^2 in binary32
 * when burnin > 0 (src/insti.cpp:1670-1671), else the template's pen; haps
 * and hnew exchanged on odd g (generation g writes hnew on even g, haps on
 * odd g); the kick-start range in g = 0 only when kick_start = 1.  Every
 * draw is keyed by the template's seed and g, so a request's result does not
 * depend on the other requests it shared launches with.  The template's
 * device buffers stay owned by the caller and alive until the request is
 * done.  The ticks are synchronous on the context stream. */
typedef struct glp_server glp_server;

#define GLP_REQ_QUEUED 0   /* waiting for device memory */
#define GLP_REQ_RESIDENT 1 /* admitted, generations in progress */
#define GLP_REQ_DONE 2     /* all generations done */

int glp_server_create(glp_ctx *ctx, uint64_t budget_bytes, int plain, glp_server **out);
/* GLP_ERR_ARG when the footprint exceeds the whole budget, the problem
 * belongs to another context, hnew is NULL or GLP_GEN_NO_WORK is set; the
 * request's first generation is validated as glp_run_batch would (sizes,
 * buffers, the problem's model inputs), with the same status codes. */
int glp_server_submit(glp_server *server, glp_problem *problem,
                      const glp_generation_args *args, uint32_t generations,
                      uint64_t *request_id);
/* resident: requests run this tick; finished: requests that finished. */
int glp_server_tick(glp_server *server, uint32_t *resident, uint32_t *finished);
/* State, generations done and the buffer holding the current haplotypes:
 * the template's hnew after an odd number of generations, else its haps. */
int glp_server_poll(glp_server *server, uint64_t request_id, int *state,
                    uint32_t *generations_done, const uint64_t **haps);
/* Forget a finished request (its record; the caller owns its buffers):
 * GLP_ERR_ARG for an unknown id, GLP_ERR_STATE before it has finished. */
int glp_server_release(glp_server *server, uint64_t request_id);
/* Ticks run, site updates done (N*(C+1)*S per request generation), bytes
 * held by resident requests. */
int glp_server_stats(glp_server *server, uint64_t *ticks, uint64_t *updates,
                     uint64_t *used_bytes);
void glp_server_destroy(glp_server *server);

/* kNN surrogate restriction on the device: for each of the H/2 samples,
 * the ceil(K/2) haplotypes nearest (over the common sites, those whose
 * alt-allele frequency, or MAF when use_maf, lies in [freq_lb, freq_ub]) to
 * its first haplotype, then the ceil(K/2) nearest to its second that are not
 * yet chosen, interleaved; ties in index order.  The distance is the context's
 * kNN metric (glp_set_knn_metric): the Hamming distance by default, or the
 * number of common sites minus the longest run of common sites at which the
 * two haplotypes agree (Haplotype::MaxTractLen, src/haplotype.cpp:62-90;
 * insti -T, src/kNN.cpp:157-164).  haps and neighbors ([H/2][2*ceil(K/2)])
 * are DEVICE pointers; asynchronous, finish with glp_finish().  Replaces
 * KNN::KNN / KNN::ClusterHaps (src/kNN.cpp:7-206).  Needs H <= 50000 and
 * 2*ceil(K/2) <= H - 2. */
int glp_knn_neighbors(glp_ctx *ctx, const uint64_t *haps, uint32_t num_haps, uint32_t num_sites,
                      uint32_t k, double freq_lb, double freq_ub, int use_maf,
                      uint32_t *neighbors);
/* The distance glp_knn_neighbors uses from now on in this context:
 * GLP_KNN_HAMMING (the default) or GLP_KNN_TRACT (GLP_ERR_ARG otherwise). */
#define GLP_KNN_HAMMING 0
#define GLP_KNN_TRACT 1
int glp_set_knn_metric(glp_ctx *ctx, int metric);

/* Allele tallies of a sampling generation for all N samples: for each
 * sample, hsum rows 2i and 2i+1 ([2N][S] uint32) gain the sample's two
 * current haplotypes, in the orientation that agrees best with the tallies
 * so far.  Replaces the Impute::replace loop of Insti::estimate
 * (src/impute.cpp:564-595, src/insti.cpp:1710-1712).  DEVICE pointers,
 * asynchronous. */
int glp_tally(glp_ctx *ctx, const uint64_t *haps, uint32_t num_samples, uint32_t num_sites,
              uint32_t *hsum);

/* GL vector quantisation on the device (GLVQ::BuildCodeBook,
 * src/glVQ.cpp:26-146; GLPack::GetPackedGLs, src/glPack.cpp:112-165).
 *
 * glp_vq_train: Lloyd training of a codebook of K (4 <= K <= 16) (homRef,
 * het) entries over the num_gls GL triples gl ([num_gls][3] float32, DEVICE
 * pointer), each normalised by its sum.  codebook ([K][2] float32, HOST) holds
 * the initial entries on entry (the reference seeds (0,1), (0,0), (1,0),
 * (1/3,1/3) and random ones) and the trained ones on return.  Iterates until
 * the total squared distance changes by at most 1 %, as the reference does;
 * GLP_ERR_NO_CONVERGE after max_iter updates (the reference's limit is
 * 1000).  A point's entry is the nearest by the reference's comparator
 * (differences in binary32, squared distance in binary64, first smallest
 * root); an entry's new value is the binary64 mean of its points in a fixed
 * summation order, rounded to binary32; an entry without points moves onto
 * the point SplitMix64 picks from (seed, iteration, entry).  *iterations
 * (optional) receives the number of updates.  Synchronous. */
int glp_vq_train(glp_ctx *ctx, const float *gl, uint64_t num_gls, uint32_t codebook_size,
                 float *codebook, uint64_t seed, uint32_t max_iter, uint32_t *iterations);

/* Codes of gl ([N][S][3] float32, DEVICE) packed 32/bits to a word, first
 * site in the most significant bits, packed_out [ceil(S/(32/bits))][N]
 * uint32 (DEVICE); sites past S take the code of the array's first GL
 * (glPack.cpp:147-149).  bits in {2, 4} with 2^bits >= codebook_size;
 * codebook [K][2] float32 HOST.  Asynchronous. */
int glp_vq_pack(glp_ctx *ctx, const float *gl, uint32_t num_samples, uint32_t num_sites,
                const float *codebook, uint32_t codebook_size, uint32_t bits,
                uint32_t *packed_out);

/* Allele probabilities from the tallies: prob_out [S][2N] = hsum / sn in
 * binary32.  Replaces Impute::result (src/impute.cpp:599-613).  DEVICE
 * pointers, asynchronous. */
int glp_result(glp_ctx *ctx, const uint32_t *hsum, uint32_t num_samples, uint32_t num_sites,
               uint32_t sampling_generations, float *prob_out);

/* Allocation-free generation (no counterpart in the reference).
 *
 * For callers that must not allocate device memory: code whose device memory
 * is owned by another allocator (a framework's caching allocator or an arena
 * reserved at start-up) and code that must not stall other streams, since
 * cudaMalloc/cudaFree can synchronize the whole device.  Every other entry
 * point of this library allocates its buffers (context, staging, scratch) on
 * first use; this one allocates nothing.
 *
 * It runs one generation like glp_run_generation (fused hmm_work, float
 * emission, surrogates from args or drawn on the device) with all of its
 * scratch -- work counter, statistics, error flag, the transition table in
 * kernel layout and the hmm_work rows -- in one fixed array of
 * GLP_NOALLOC_SCRATCH_BYTES (32 MiB) of device memory that every GPU loading
 * this library holds until the process exits.  It needs
 * 256 + 32*ceil((S+1)/8)*8 + 16*N*S bytes of it and returns GLP_ERR_TOO_LARGE
 * beyond that (about N*S <= 2.0e6 site-samples).
 *
 * All array arguments are DEVICE pointers except pc16 (host, row-major
 * pc[4][4]): tran [S][3], emit [N][S][4] (16-byte aligned), prob [N][S][3],
 * and those of args (GLP_GEN_VQ is not accepted).  Work is issued on
 * `stream` (cudaStream_t, NULL = legacy default stream) and the call returns
 * when it has finished, reporting GLP_ERR_INDEX for an out-of-range
 * haplotype index.
 *
 * The array's device address belongs to a CUDA context.  The first call in
 * each context -- with the usual primary context, the first call on each
 * device -- looks it up (cudaGetSymbolAddress, with that context current) and
 * sets the kernels' launch attributes; later calls in the same context reuse
 * that set-up.  Any context is supported: the set-up is kept per context id,
 * so a context made after cudaDeviceReset or with the driver API gets its
 * own.  Every call copies the device error flag back into host memory and
 * synchronizes `stream` before it returns, so no call may be made while a
 * stream is capturing (a CUDA graph cannot hold it).  Calls share the one array, which keeps what the last
 * call left there (each call clears the counters and flag it reads): calls
 * that overlap on the GPU (other host threads, other streams) race and must
 * be serialized by the caller. */
#define GLP_NOALLOC_SCRATCH_BYTES ((size_t)32 << 20)
int glp_run_generation_noalloc(const glp_generation_args *args, const float *tran,
                               const float *pc16, const float *emit, const float *prob,
                               void *stream);

/* Calibration (no reference counterpart): runs a dependent-free FMA stream on
 * every SM for about `ms_target` milliseconds and reports the achieved FP32
 * rate in TFLOP/s (2 flops per FMA): the roofline denominator of the
 * FP32-bound likelihood recursion. */
int glp_measure_fp32_peak(glp_ctx *ctx, float ms_target, double *tflops);

#ifdef __cplusplus
}
#endif
#endif /* GLPHASE_GPU_H */
