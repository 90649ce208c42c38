/* Test-only stand-in for the GSL RNG API (declarations follow GSL's public
 * documentation).  The McLiCS reference includes this header; only the few
 * entry points it calls are provided.  The generator is NOT GSL's ranlxs0 or
 * taus: streams differ, and a test can feed an explicit list of uniforms. */
#ifndef MCX_GSL_SHIM_RNG_H_
#define MCX_GSL_SHIM_RNG_H_
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct gsl_rng_type { const char *name; } gsl_rng_type;
typedef struct gsl_rng { const gsl_rng_type *type; unsigned long long state; } gsl_rng;
extern const gsl_rng_type *gsl_rng_ranlxs0;
extern const gsl_rng_type *gsl_rng_taus;
const gsl_rng_type *gsl_rng_env_setup(void);
gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_set(const gsl_rng *r, unsigned long int s);
double gsl_rng_uniform(const gsl_rng *r);
void gsl_rng_free(gsl_rng *r);
/* Shim-only hook: when set, gsl_rng_uniform returns feed[0..n-1] in order. */
void mcx_shim_feed(const double *feed, long n);
long mcx_shim_feed_used(void);
#ifdef __cplusplus
}
#endif
#endif
