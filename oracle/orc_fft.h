/* Oracle FFT: double-precision mixed-radix FFT used by the CPU oracle and by the
 * single-rank FFTW shim that lets the reference sources build without FFTW.
 *
 * TEST INFRASTRUCTURE ONLY. Nothing in the product (capow_gb300/) links this.
 *
 * Convention follows FFTW's forward r2c transform as the reference calls it
 * (main.c:1200-1201 plans, main.c:266-271 executes): sign -1, unnormalised,
 * in place on a row-major [n0][n1][2*(n2/2+1)] real array, output
 * [n0][n1][n2/2+1] complex, not transposed.
 */
#ifndef ORC_FFT_H
#define ORC_FFT_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* out-of-place complex DFT of length n (interleaved re,im), sign -1 */
void orc_fft_c2c_1d(int n, const double *in, double *out);

/* in-place 3-D r2c on the padded layout described above */
void orc_fft_r2c_3d_inplace(int n0, int n1, int n2, double *data);

/* in-place 3-D c2c (interleaved, [n0][n1][n2]); sign -1 forward, +1 backward, unnormalised */
void orc_fft_c2c_3d_inplace(int n0, int n1, int n2, double *data, int sign);

/* in-place 3-D c2r (inverse of r2c without 1/N), [n0][n1][n2/2+1] complex in,
 * padded real out. Hermitian symmetry of the input is assumed as FFTW does. */
void orc_fft_c2r_3d_inplace(int n0, int n1, int n2, double *data);

#ifdef __cplusplus
}
#endif
#endif
