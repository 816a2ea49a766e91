/* gsl/gsl_sf_gamma.h -- stand-in for gsl_sf_gamma (TEST INFRASTRUCTURE): the C library's tgamma. */
#ifndef GSREF_SHIM_GSL_SF_GAMMA_H
#define GSREF_SHIM_GSL_SF_GAMMA_H
#ifdef __cplusplus
extern "C" {
#endif
double gsl_sf_gamma(double x);
#ifdef __cplusplus
}
#endif
#endif
