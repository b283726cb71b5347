/*
 * Stand-in for GSL's <gsl/gsl_rng.h>, used only to compile the reference's
 * impute.cpp in place (oracle/Makefile -> oracle/_ref).  GSL is not installed
 * here and its only role on the hot path is to supply random draws
 * (impute.cpp:292-294, 470, 498-517), which the oracle replays from a trace
 * instead.  This file is test infrastructure; it implements no GSL algorithm.
 *
 * gsl_rng_uniform() serves the next value of a caller-provided trace
 * (glpr_set_uniforms in ref_harness.cpp); gsl_rng_get() serves the next value
 * of an integer trace, or a fixed counter when none is set.
 */
#ifndef GLP_REF_SHIM_GSL_RNG_H
#define GLP_REF_SHIM_GSL_RNG_H

#include <stddef.h>
#include <stdint.h>

typedef struct gsl_rng_type {
  int unused;
} gsl_rng_type;

typedef struct gsl_rng {
  const double *u;
  size_t nu, pu;
  const unsigned long *g;
  size_t ng, pg;
  unsigned long counter;
} gsl_rng;

static const gsl_rng_type glp_shim_rng_type = {0};
#define gsl_rng_default (&glp_shim_rng_type)

static inline gsl_rng *gsl_rng_alloc(const gsl_rng_type *) {
  gsl_rng *r = new gsl_rng;
  r->u = 0;
  r->nu = r->pu = 0;
  r->g = 0;
  r->ng = r->pg = 0;
  r->counter = 0;
  return r;
}
static inline void gsl_rng_free(gsl_rng *r) { delete r; }
static inline void gsl_rng_set(gsl_rng *, unsigned long) {}
static inline double gsl_rng_uniform(gsl_rng *r) {
  return (r->pu < r->nu) ? r->u[r->pu++] : 0.5;
}
static inline unsigned long gsl_rng_get(gsl_rng *r) {
  return (r->pg < r->ng) ? r->g[r->pg++] : r->counter++;
}
static inline unsigned long gsl_rng_uniform_int(gsl_rng *r, unsigned long n) {
  return gsl_rng_get(r) % n;
}

#endif
