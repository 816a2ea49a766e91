/* gsl/gsl_errno.h -- the GSL status codes the reference sources name (TEST INFRASTRUCTURE). */
#ifndef GSREF_SHIM_GSL_ERRNO_H
#define GSREF_SHIM_GSL_ERRNO_H
#define GSL_SUCCESS 0
#define GSL_FAILURE (-1)
#define GSL_CONTINUE (-2)
#endif
