/* Test-only stand-in for GSL's random distributions (declaration only). */
#ifndef MCX_GSL_SHIM_RANDIST_H_
#define MCX_GSL_SHIM_RANDIST_H_
#include <gsl/gsl_rng.h>
#ifdef __cplusplus
extern "C" {
#endif
void gsl_ran_dir_3d(const gsl_rng *r, double *x, double *y, double *z);
#ifdef __cplusplus
}
#endif
#endif
