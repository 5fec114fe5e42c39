/*
 * fftw_shim.c -- implementation of the FFTW3-API shim (see fftw3.h).
 * TEST INFRASTRUCTURE ONLY: linked into oracle/_ref with the reference's
 * CPU sources.  Memory from fftw_malloc must be releasable with free(),
 * because the reference frees its FFT input with free()
 * (collisionless/double/src/fourier.cc:123).
 */
#include "fftw3.h"
#include "../orc_fft.h"

#include <stdlib.h>

struct oracle_fftw_plan_s {
    int kind; /* 0 = r2c, 1 = c2r */
    int n0, n1;
    void *in, *out;
};

void *fftw_malloc(size_t n) { return malloc(n ? n : 1); }
void fftw_free(void *p) { free(p); }

static fftw_plan make_plan(int kind, int n0, int n1, void *in, void *out)
{
    fftw_plan p = (fftw_plan)malloc(sizeof(*p));
    p->kind = kind;
    p->n0 = n0;
    p->n1 = n1;
    p->in = in;
    p->out = out;
    return p;
}

fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out, unsigned flags)
{
    (void)flags;
    return make_plan(0, n0, n1, in, out);
}

fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex *in, double *out, unsigned flags)
{
    (void)flags;
    return make_plan(1, n0, n1, in, out);
}

void fftw_execute(const fftw_plan p)
{
    if (p->kind == 0)
        orc_fft2d_r2c(p->n0, p->n1, (const double *)p->in, (double *)p->out);
    else
        orc_fft2d_c2r(p->n0, p->n1, (const double *)p->in, (double *)p->out);
}

void fftw_destroy_plan(fftw_plan p) { free(p); }
