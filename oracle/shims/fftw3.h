/* Stand-in for the FFTW3 API subset the reference uses (test infrastructure only).
 * Plans are in-place 3-D r2c transforms executed by the oracle FFT (oracle/orc_fft.c):
 * sign -1, unnormalised, padded last dimension, as FFTW documents. */
#ifndef CAPOW_SHIM_FFTW3_H
#define CAPOW_SHIM_FFTW3_H
#include <stddef.h>
typedef double fftw_complex[2];
typedef struct capow_shim_plan *fftw_plan;
#define FFTW_ESTIMATE (1U << 6)
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
#endif
