/* fftw3-mpi.h -- declarations of the FFTW3 MPI calls the reference sources name (TEST
 * INFRASTRUCTURE).  They belong to its two-dimensional transverse build, which oracle/_ref
 * does not build (TRANSVERSE_DIMENSIONS = 1); fftw_mpi_init does nothing and the others
 * abort if they are ever reached. */
#ifndef GSREF_SHIM_FFTW3_MPI_H
#define GSREF_SHIM_FFTW3_MPI_H

#include <stddef.h>
#include "fftw3.h"
#include "mpi.h"

#ifdef __cplusplus
extern "C" {
#endif

#define FFTW_MPI_DEFAULT_BLOCK (0)
#define FFTW_MPI_TRANSPOSED_IN (1U << 29)
#define FFTW_MPI_TRANSPOSED_OUT (1U << 30)

void fftw_mpi_init(void);
ptrdiff_t fftw_mpi_local_size_many_transposed(int rnk, const ptrdiff_t* n, ptrdiff_t howmany, ptrdiff_t block0,
                                              ptrdiff_t block1, MPI_Comm comm, ptrdiff_t* local_n0,
                                              ptrdiff_t* local_0_start, ptrdiff_t* local_n1, ptrdiff_t* local_1_start);
fftw_plan fftw_mpi_plan_many_dft(int rnk, const ptrdiff_t* n, ptrdiff_t howmany, ptrdiff_t iblock, ptrdiff_t oblock,
                                 fftw_complex* in, fftw_complex* out, MPI_Comm comm, int sign, unsigned flags);
void fftw_mpi_execute_dft(fftw_plan p, fftw_complex* in, fftw_complex* out);

#ifdef __cplusplus
}
#endif
#endif
