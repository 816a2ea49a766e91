/* gsl/gsl_sf_bessel.h -- stand-in for the GSL Bessel functions of the reference build (TEST
 * INFRASTRUCTURE).  J0 and J1 come from the C library (POSIX j0 / j1); the s-th positive zero
 * of J0 is McMahon's asymptotic expansion refined by Newton's method on j0 / j1. */
#ifndef GSREF_SHIM_GSL_SF_BESSEL_H
#define GSREF_SHIM_GSL_SF_BESSEL_H
#ifdef __cplusplus
extern "C" {
#endif
double gsl_sf_bessel_J0(double x);
double gsl_sf_bessel_J1(double x);
double gsl_sf_bessel_zero_J0(unsigned int s);
#ifdef __cplusplus
}
#endif
#endif
