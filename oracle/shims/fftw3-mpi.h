/* Stand-in for the FFTW3-MPI API subset the reference uses (test infrastructure only). */
#ifndef CAPOW_SHIM_FFTW3_MPI_H
#define CAPOW_SHIM_FFTW3_MPI_H
#include <stddef.h>
#include "fftw3.h"
#include "mpi.h"
void fftw_mpi_init(void);
ptrdiff_t fftw_mpi_local_size_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, MPI_Comm comm, ptrdiff_t *local_n0,
                                 ptrdiff_t *local_0_start);
fftw_plan fftw_mpi_plan_dft_r2c_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, double *in, fftw_complex *out,
                                   MPI_Comm comm, unsigned flags);
#endif
