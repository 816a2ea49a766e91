/* fftw3.h -- stand-in for the FFTW3 double-precision calls of the reference build (TEST
 * INFRASTRUCTURE: only oracle/_ref is compiled against it).
 *
 * Same conventions as FFTW3: unnormalised DFT, sign FFTW_FORWARD = -1 for exp(-2 pi i jk/n)
 * and FFTW_BACKWARD = +1, "many" plans over howmany transforms of rank 1 with strides and
 * distances, execute_dft on new arrays of the plan's layout, in place allowed.  The transform
 * itself is this project's own radix-2 FFT (power-of-two n; a direct DFT for any other n), not
 * FFTW's codelets, so results agree with FFTW to rounding only. */
#ifndef GSREF_SHIM_FFTW3_H
#define GSREF_SHIM_FFTW3_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct gsref_fftw_plan_s* fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_PATIENT (1U << 5)

fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out, int sign, unsigned flags);
fftw_plan fftw_plan_many_dft(int rank, const int* n, int howmany, fftw_complex* in, const int* inembed, int istride,
                             int idist, fftw_complex* out, const int* onembed, int ostride, int odist, int sign,
                             unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out);
void fftw_destroy_plan(fftw_plan p);
void* fftw_malloc(size_t n);
void fftw_free(void* p);

#ifdef __cplusplus
}
#endif
#endif
