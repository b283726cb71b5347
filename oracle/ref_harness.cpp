/*
 * ref_harness.cpp -- C entry points into the reference's own Impute class
 * (impute.hpp / impute.cpp, compiled unmodified from the reference tree by
 * oracle/Makefile).  TEST INFRASTRUCTURE ONLY: the resulting
 * oracle/_ref/libglp_ref.so pins the C restatement in glp_oracle.c; it never
 * runs on the product path.
 *
 * Impute keeps its state in protected members; RefImpute below only fills
 * them for one sample and forwards to the reference's member functions:
 *   glpr_hmm_like   -> Impute::hmm_like   (impute.cpp:327-376)
 *   glpr_hmm_work   -> Impute::hmm_work   (impute.cpp:380-485)
 *   glpr_initialize -> Impute::initialize (impute.cpp:182-322), model part
 *   glpr_replace    -> Impute::replace    (impute.cpp:564-595)
 *   glpr_result     -> Impute::result     (impute.cpp:599-613)
 *   glpr_mh_chain   -> MHSampler<unsigned>::SampleHap (MHSampler.hpp:81-96),
 *                      plain MH, over a sequence of proposals
 */
#include <cstring>
#include <vector>

#include "MHSampler.hpp"
#include "impute.hpp"

namespace {

struct RefImpute : public Impute {
  void load_one(const float *emit_row, const float *tran_in,
                const uint64_t *haps_in, uint32_t H, uint32_t wn_in,
                uint32_t S) {
    mn = S;
    wn = wn_in;
    en = 4 * S;
    pn = 3 * S;
    in = 1;
    hn = 2;
    haps.assign(haps_in, haps_in + (size_t)H * wn_in);
    emit.assign(emit_row, emit_row + (size_t)S * 4);
    tran.assign(tran_in, tran_in + (size_t)S * 3);
  }
  float like(const uint32_t P[4]) {
    unsigned p[4] = {P[0], P[1], P[2], P[3]};
    return hmm_like(0, p);
  }
  void work(const float *prob_row, const float pc_in[16], const uint32_t P[4],
            float pen, const float *u, uint64_t *ha, uint64_t *hb) {
    prob.assign(prob_row, prob_row + (size_t)mn * 3);
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j)
        pc[i][j] = pc_in[i * 4 + j];
    hnew.assign((size_t)2 * wn, 0);
    std::vector<double> ud(u, u + mn);
    rng->u = ud.data();
    rng->nu = ud.size();
    rng->pu = 0;
    unsigned p[4] = {P[0], P[1], P[2], P[3]};
    hmm_work(0, p, pen);
    rng->u = 0;
    rng->nu = 0;
    std::memcpy(ha, hnew.data(), sizeof(uint64_t) * wn);
    std::memcpy(hb, hnew.data() + wn, sizeof(uint64_t) * wn);
  }
  void init_model(const float *prob_site_major, const double *pos, uint32_t N,
                  uint32_t S, double dens, float *tran_out, float *pc_out,
                  float *emit_out, float *t_out) {
    in = N;
    mn = S;
    density = dens;
    is_x = false;
    prob.assign(prob_site_major, prob_site_major + (size_t)S * N * 2);
    posi.assign(pos, pos + S);
    name.assign(N, std::string("s"));
    initialize();
    std::memcpy(tran_out, tran.data(), sizeof(float) * 3 * S);
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j)
        pc_out[i * 4 + j] = pc[i][j];
    std::memcpy(emit_out, emit.data(), sizeof(float) * 4 * (size_t)N * S);
    std::memcpy(t_out, prob.data(), sizeof(float) * 3 * (size_t)N * S);
  }
  void tally(const uint64_t *haps_in, uint32_t N, uint32_t S, uint32_t wn_in,
             uint32_t sample, uint32_t *hsum_io) {
    in = N;
    mn = S;
    wn = wn_in;
    haps.assign(haps_in, haps_in + (size_t)2 * N * wn_in);
    hsum.assign(hsum_io, hsum_io + (size_t)2 * N * S);
    replace(sample);
    std::memcpy(hsum_io, hsum.data(), sizeof(uint32_t) * 2 * (size_t)N * S);
  }
  void probabilities(const uint32_t *hsum_in, uint32_t N, uint32_t S, uint32_t sampling,
                     float *prob_out) {
    in = N;
    hn = 2 * N;
    mn = S;
    sn = sampling;
    hsum.assign(hsum_in, hsum_in + (size_t)2 * N * S);
    result();
    std::memcpy(prob_out, prob.data(), sizeof(float) * 2 * (size_t)N * S);
  }
};

} // namespace

extern "C" {

float glpr_hmm_like(const float *emit_row, const float *tran,
                    const uint64_t *haps, uint32_t H, uint32_t wn, uint32_t S,
                    const uint32_t P[4]) {
  RefImpute r;
  r.load_one(emit_row, tran, haps, H, wn, S);
  return r.like(P);
}

void glpr_hmm_work(const float *emit_row, const float *prob_row,
                   const float *tran, const float pc[16], const uint64_t *haps,
                   uint32_t H, uint32_t wn, uint32_t S, const uint32_t P[4],
                   float pen, const float *u, uint64_t *ha, uint64_t *hb) {
  RefImpute r;
  r.load_one(emit_row, tran, haps, H, wn, S);
  r.work(prob_row, pc, P, pen, u, ha, hb);
}

void glpr_initialize(const float *prob_site_major, const double *pos,
                     uint32_t N, uint32_t S, double density, float *tran,
                     float *pc, float *emit, float *t) {
  RefImpute r;
  r.init_model(prob_site_major, pos, N, S, density, tran, pc, emit, t);
}

void glpr_replace(const uint64_t *haps, uint32_t N, uint32_t S, uint32_t wn,
                  uint32_t sample, uint32_t *hsum) {
  RefImpute r;
  r.tally(haps, N, S, wn, sample, hsum);
}

void glpr_result(const uint32_t *hsum, uint32_t N, uint32_t S, uint32_t sn,
                 float *prob_out) {
  RefImpute r;
  r.probabilities(hsum, N, S, sn, prob_out);
}

// A chain as Insti::solve runs it (insti.cpp:1497-1531): the sampler starts
// at log-likelihood like[0]; proposal c (1 .. n) changes the state from
// c - 1 to c with log-likelihood like[c] and is accepted or reverted.  The
// sampler draws its uniforms from u in order (one per proposal that scores
// below the current likelihood).  accept[c - 1] and state[c - 1] receive the
// decision and the state after it.
void glpr_mh_chain(const double *like, uint32_t n, double pen, const double *u,
                   uint32_t nu, uint8_t *accept, uint32_t *state) {
  gsl_rng *rng = gsl_rng_alloc(gsl_rng_default);
  rng->u = u;
  rng->nu = nu;
  rng->pu = 0;
  MHSampler<unsigned> mh(rng, like[0], pen);
  unsigned object = 0;
  for (uint32_t c = 1; c <= n; ++c) {
    const unsigned prev = object;
    object = c;
    accept[c - 1] = mh.SampleHap(object, prev, like[c]) ? 1 : 0;
    state[c - 1] = object;
  }
  gsl_rng_free(rng);
}
}
