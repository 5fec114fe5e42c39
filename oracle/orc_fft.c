/*
 * orc_fft.c -- CPU FFT for the oracle (test infrastructure only).
 *
 * Iterative radix-2 Cooley-Tukey (decimation in time, bit-reversed input
 * order) for power-of-two lengths; a direct DFT for any other length.
 * Twiddles are computed with cos/sin of the exact angle for every stage so
 * that accuracy does not degrade through recurrences.
 */
#include "orc_fft.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

static void fft_pow2(int n, double *a, int sign)
{
    /* bit-reversal permutation */
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            double tr = a[2 * i], ti = a[2 * i + 1];
            a[2 * i] = a[2 * j];
            a[2 * i + 1] = a[2 * j + 1];
            a[2 * j] = tr;
            a[2 * j + 1] = ti;
        }
    }
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1;
        double ang = sign * 2.0 * M_PI / (double)len;
        for (int k = 0; k < half; ++k) {
            double wr = cos(ang * k), wi = sin(ang * k);
            for (int s = 0; s < n; s += len) {
                int u = s + k, v = s + k + half;
                double xr = a[2 * v] * wr - a[2 * v + 1] * wi;
                double xi = a[2 * v] * wi + a[2 * v + 1] * wr;
                a[2 * v] = a[2 * u] - xr;
                a[2 * v + 1] = a[2 * u + 1] - xi;
                a[2 * u] += xr;
                a[2 * u + 1] += xi;
            }
        }
    }
}

static void dft_direct(int n, double *a, int sign)
{
    double *t = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    for (int k = 0; k < n; ++k) {
        double sr = 0.0, si = 0.0;
        for (int j = 0; j < n; ++j) {
            /* reduce the phase index exactly before forming the angle */
            long m = ((long)j * (long)k) % n;
            double ang = sign * 2.0 * M_PI * (double)m / (double)n;
            double c = cos(ang), s = sin(ang);
            sr += a[2 * j] * c - a[2 * j + 1] * s;
            si += a[2 * j] * s + a[2 * j + 1] * c;
        }
        t[2 * k] = sr;
        t[2 * k + 1] = si;
    }
    memcpy(a, t, sizeof(double) * 2 * (size_t)n);
    free(t);
}

void orc_fft1d(int n, double *data, int sign)
{
    if (n <= 1) return;
    if (is_pow2(n))
        fft_pow2(n, data, sign);
    else
        dft_direct(n, data, sign);
}

void orc_fft2d_r2c(int n0, int n1, const double *in, double *out)
{
    const int nh = n1 / 2 + 1;
    double *row = (double *)malloc(sizeof(double) * 2 * (size_t)n1);
    double *col = (double *)malloc(sizeof(double) * 2 * (size_t)n0);
    /* rows: full complex transform of each real row, keep the first half */
    for (int i = 0; i < n0; ++i) {
        for (int j = 0; j < n1; ++j) {
            row[2 * j] = in[(size_t)i * n1 + j];
            row[2 * j + 1] = 0.0;
        }
        orc_fft1d(n1, row, -1);
        memcpy(out + (size_t)2 * i * nh, row, sizeof(double) * 2 * (size_t)nh);
    }
    /* columns */
    for (int j = 0; j < nh; ++j) {
        for (int i = 0; i < n0; ++i) {
            col[2 * i] = out[((size_t)i * nh + j) * 2];
            col[2 * i + 1] = out[((size_t)i * nh + j) * 2 + 1];
        }
        orc_fft1d(n0, col, -1);
        for (int i = 0; i < n0; ++i) {
            out[((size_t)i * nh + j) * 2] = col[2 * i];
            out[((size_t)i * nh + j) * 2 + 1] = col[2 * i + 1];
        }
    }
    free(row);
    free(col);
}

void orc_fft2d_c2r(int n0, int n1, const double *in, double *out)
{
    const int nh = n1 / 2 + 1;
    double *half = (double *)malloc(sizeof(double) * 2 * (size_t)n0 * nh);
    double *col = (double *)malloc(sizeof(double) * 2 * (size_t)n0);
    double *row = (double *)malloc(sizeof(double) * 2 * (size_t)n1);
    memcpy(half, in, sizeof(double) * 2 * (size_t)n0 * nh);
    /* columns: backward complex transform */
    for (int j = 0; j < nh; ++j) {
        for (int i = 0; i < n0; ++i) {
            col[2 * i] = half[((size_t)i * nh + j) * 2];
            col[2 * i + 1] = half[((size_t)i * nh + j) * 2 + 1];
        }
        orc_fft1d(n0, col, +1);
        for (int i = 0; i < n0; ++i) {
            half[((size_t)i * nh + j) * 2] = col[2 * i];
            half[((size_t)i * nh + j) * 2 + 1] = col[2 * i + 1];
        }
    }
    /* rows: rebuild the Hermitian full row and keep the real part */
    for (int i = 0; i < n0; ++i) {
        const double *h = half + (size_t)2 * i * nh;
        for (int j = 0; j < nh; ++j) {
            row[2 * j] = h[2 * j];
            row[2 * j + 1] = h[2 * j + 1];
        }
        for (int j = nh; j < n1; ++j) {
            row[2 * j] = h[2 * (n1 - j)];
            row[2 * j + 1] = -h[2 * (n1 - j) + 1];
        }
        orc_fft1d(n1, row, +1);
        for (int j = 0; j < n1; ++j) out[(size_t)i * n1 + j] = row[2 * j];
    }
    free(half);
    free(col);
    free(row);
}
