/* Minimal stand-in (see gsl_rng.h): gamma variates abort when called. */
#ifndef SMC_GSL_SHIM_RANDIST_H
#define SMC_GSL_SHIM_RANDIST_H
#include "gsl_rng.h"
#ifdef __cplusplus
extern "C" {
#endif
double gsl_ran_gamma(const gsl_rng *r, double a, double b);
#ifdef __cplusplus
}
#endif
#endif
