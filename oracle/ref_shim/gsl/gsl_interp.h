/* gsl/gsl_interp.h -- included by the reference's input processing, whose interpolation
 * calls are commented out; nothing is declared (TEST INFRASTRUCTURE). */
#ifndef GSREF_SHIM_GSL_INTERP_H
#define GSREF_SHIM_GSL_INTERP_H
#endif
