/* Minimal stand-in: no error-handler calls are made by the checked path. */
#ifndef SMC_GSL_SHIM_ERRNO_H
#define SMC_GSL_SHIM_ERRNO_H
#endif
