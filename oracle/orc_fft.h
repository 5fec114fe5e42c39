/*
 * orc_fft.h -- double-precision 2-D real FFTs for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY: this file belongs to the CPU oracle.  Only the
 * tests, the smoke check and bench.py's CPU-baseline leg may use it.
 *
 * Conventions are those of FFTW3's r2c/c2r 2-D transforms, which the
 * reference calls in collisionless/double/src/fourier.cc:36-41,81:
 *   forward  X[k0][k1] = sum_{j0,j1} x[j0][j1] exp(-2 pi i (j0 k0/n0 + j1 k1/n1))
 *   backward x[j0][j1] = sum_{k0,k1} X[k0][k1] exp(+2 pi i (...))   (no 1/N)
 * Real data is row-major n0 x n1; the half spectrum is n0 x (n1/2+1).
 * The c2r treats its input as the half of a Hermitian array (only the real
 * part of the reconstructed signal is kept), as FFTW does; the input array
 * is not modified.
 *
 * The algorithm is an iterative radix-2 Cooley-Tukey FFT for power-of-two
 * lengths and a direct O(n^2) DFT otherwise.
 */
#ifndef ORC_FFT_H
#define ORC_FFT_H

#ifdef __cplusplus
extern "C" {
#endif

/* in: n0*n1 doubles; out: n0*(n1/2+1) complex as interleaved (re, im). */
void orc_fft2d_r2c(int n0, int n1, const double *in, double *out);
/* in: n0*(n1/2+1) complex (not modified); out: n0*n1 doubles, unnormalised. */
void orc_fft2d_c2r(int n0, int n1, const double *in, double *out);
/* In-place complex 1-D transform of n points (interleaved re/im).
 * sign = -1 forward, +1 backward, unnormalised. */
void orc_fft1d(int n, double *data, int sign);

#ifdef __cplusplus
}
#endif
#endif
