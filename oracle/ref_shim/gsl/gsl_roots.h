/* gsl/gsl_roots.h -- a secant root finder with GSL's fdfsolver interface (TEST
 * INFRASTRUCTURE).  The reference uses it only to pick the FHATHA transform's log spacing,
 * which the QDHT builds never construct. */
#ifndef GSREF_SHIM_GSL_ROOTS_H
#define GSREF_SHIM_GSL_ROOTS_H
#include "gsl_math.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { const char* name; } gsl_root_fdfsolver_type;
typedef struct {
    const gsl_root_fdfsolver_type* type;
    gsl_function_fdf* fdf;
    double root, f, df;
} gsl_root_fdfsolver;
extern const gsl_root_fdfsolver_type* gsl_root_fdfsolver_secant;
gsl_root_fdfsolver* gsl_root_fdfsolver_alloc(const gsl_root_fdfsolver_type* T);
int gsl_root_fdfsolver_set(gsl_root_fdfsolver* s, gsl_function_fdf* fdf, double root);
int gsl_root_fdfsolver_iterate(gsl_root_fdfsolver* s);
double gsl_root_fdfsolver_root(const gsl_root_fdfsolver* s);
void gsl_root_fdfsolver_free(gsl_root_fdfsolver* s);
int gsl_root_test_delta(double x1, double x0, double epsabs, double epsrel);
#ifdef __cplusplus
}
#endif
#endif
