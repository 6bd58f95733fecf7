/* Definitions for the minimal GSL stand-in headers.  Every entry point that
 * would produce a number aborts: the parity checker only drives code paths
 * of the reference that do not use GSL. */
#include <stdio.h>
#include <stdlib.h>
#include "gsl/gsl_rng.h"
#include "gsl/gsl_randist.h"
#include "gsl/gsl_spline.h"

static void shim_abort(const char *what) {
  fprintf(stderr, "gsl shim: %s is not available in the parity checker\n", what);
  abort();
}
static const gsl_rng_type shim_rng_type = {0};
const gsl_rng_type *gsl_rng_default = &shim_rng_type;
static const gsl_interp_type shim_cspline = {0};
const gsl_interp_type *gsl_interp_cspline = &shim_cspline;

void gsl_rng_env_setup(void) {}
gsl_rng *gsl_rng_alloc(const gsl_rng_type *t) { (void)t; return (gsl_rng *)calloc(1, sizeof(gsl_rng)); }
void gsl_rng_set(const gsl_rng *r, unsigned long seed) { (void)r; (void)seed; }
void gsl_rng_free(gsl_rng *r) { free(r); }
double gsl_ran_gamma(const gsl_rng *r, double a, double b) { (void)r; (void)a; (void)b; shim_abort("gsl_ran_gamma"); return 0; }
gsl_interp_accel *gsl_interp_accel_alloc(void) { shim_abort("gsl_interp_accel_alloc"); return NULL; }
void gsl_interp_accel_free(gsl_interp_accel *a) { (void)a; }
gsl_spline *gsl_spline_alloc(const gsl_interp_type *t, size_t n) { (void)t; (void)n; shim_abort("gsl_spline_alloc"); return NULL; }
int gsl_spline_init(gsl_spline *s, const double xa[], const double ya[], size_t n) { (void)s; (void)xa; (void)ya; (void)n; shim_abort("gsl_spline_init"); return 0; }
double gsl_spline_eval(const gsl_spline *s, double x, gsl_interp_accel *a) { (void)s; (void)x; (void)a; shim_abort("gsl_spline_eval"); return 0; }
void gsl_spline_free(gsl_spline *s) { (void)s; }
