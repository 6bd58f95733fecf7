/* Minimal stand-in (see gsl_rng.h): splines are only used by the rcBK and
 * large-x models, which the checker never constructs; every function aborts. */
#ifndef SMC_GSL_SHIM_SPLINE_H
#define SMC_GSL_SHIM_SPLINE_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { int unused; } gsl_interp_type;
typedef struct { int unused; } gsl_interp_accel;
typedef struct { int unused; } gsl_spline;
extern const gsl_interp_type *gsl_interp_cspline;
gsl_interp_accel *gsl_interp_accel_alloc(void);
void gsl_interp_accel_free(gsl_interp_accel *a);
gsl_spline *gsl_spline_alloc(const gsl_interp_type *t, size_t n);
int gsl_spline_init(gsl_spline *s, const double xa[], const double ya[], size_t n);
double gsl_spline_eval(const gsl_spline *s, double x, gsl_interp_accel *a);
void gsl_spline_free(gsl_spline *s);
#ifdef __cplusplus
}
#endif
#endif
