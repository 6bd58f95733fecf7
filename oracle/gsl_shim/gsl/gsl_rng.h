/* Minimal stand-in for the GNU Scientific Library RNG header, written for
 * building the reference superMC sources as a parity checker.  Only the
 * multiplicity-fluctuation path (cc_fluctuation_model > 5) calls into it,
 * and that path is not exercised by the checker; every function aborts. */
#ifndef SMC_GSL_SHIM_RNG_H
#define SMC_GSL_SHIM_RNG_H
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { int unused; } gsl_rng_type;
typedef struct { unsigned long state; } gsl_rng;
extern const gsl_rng_type *gsl_rng_default;
void gsl_rng_env_setup(void);
gsl_rng *gsl_rng_alloc(const gsl_rng_type *t);
void gsl_rng_set(const gsl_rng *r, unsigned long seed);
void gsl_rng_free(gsl_rng *r);
#ifdef __cplusplus
}
#endif
#endif
