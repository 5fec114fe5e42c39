/*
 * fftw3.h -- FFTW3-API shim used ONLY to compile the reference's CPU sources
 * (collisionless/double/src/fourier.cc) into the test oracle under
 * oracle/_ref/.  FFTW3 itself is not installed in this image.
 *
 * TEST INFRASTRUCTURE ONLY.  Only the seven names that fourier.cc uses are
 * provided, with FFTW's documented signatures; the transforms are the
 * oracle's own FFT (orc_fft.c).  Semantics follow the FFTW3 manual:
 * unnormalised r2c (exp(-i)) and c2r (exp(+i)) 2-D transforms, row-major,
 * half spectrum n0 x (n1/2+1).  One documented FFTW behaviour is NOT
 * reproduced: FFTW_MEASURE planning without wisdom overwrites the arrays
 * the first time a size is planned; this shim never touches them, which is
 * what FFTW does for every later plan of the same size in one process.
 */
#ifndef ORACLE_FFTW3_SHIM_H
#define ORACLE_FFTW3_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct oracle_fftw_plan_s *fftw_plan;

#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

void *fftw_malloc(size_t n);
void fftw_free(void *p);
fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex *in, double *out, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

#ifdef __cplusplus
}
#endif
#endif
