/* Minimal stand-in: the reference only needs <math.h> through this header. */
#ifndef SMC_GSL_SHIM_MATH_H
#define SMC_GSL_SHIM_MATH_H
#include <math.h>
#endif
