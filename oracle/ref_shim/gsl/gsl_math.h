/* gsl/gsl_math.h -- the function-with-derivative record of GSL's root finders (TEST
 * INFRASTRUCTURE). */
#ifndef GSREF_SHIM_GSL_MATH_H
#define GSREF_SHIM_GSL_MATH_H
typedef struct {
    double (*f)(double x, void* params);
    double (*df)(double x, void* params);
    void (*fdf)(double x, void* params, double* f, double* df);
    void* params;
} gsl_function_fdf;
#endif
