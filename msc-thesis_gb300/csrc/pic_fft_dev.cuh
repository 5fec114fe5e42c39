// pic_fft_dev.cuh -- shared-memory complex FFTs of power-of-two lengths
// 16..4096 for the spectral Poisson solve (pic_spectral.cu).
//
// Stockham auto-sort passes as published by Govindaraju et al., "High
// performance discrete Fourier transforms on graphics processors" (SC'08):
// pass p with radix R over sub-transforms of length Ns takes butterfly j's
// inputs at j + r N/R, multiplies input r by W_N^(r (j mod Ns) N/(Ns R)),
// transforms the R values and writes output r to
// (j / Ns) Ns R + (j mod Ns) + r Ns; after the last pass the sequence is in
// natural order.  Passes are of radix 16, plus one of radix 8, 4 or 2 for the
// remaining factor.  Every thread of a transform holds 16 elements in
// registers (its butterflies of the pass: j = t + b N/16 for b < 16/R); the
// passes exchange through one shared-memory buffer per transform, indexed
// with one pad slot per 16 elements against bank conflicts.  The length is a
// template parameter, so that all but a per-thread base of every
// shared-memory and twiddle address is a compile-time offset.  Twiddles come
// from per-pass tables computed in double on the host (twiddle_len entries
// per length; a warp reads consecutive entries).
#pragma once
#include <cuda_runtime.h>

namespace pic {
namespace fft {

constexpr int E = 16;  // elements per thread

// shared-memory float2 slots of one transform's buffer; `extra` spreads
// interleaved buffers over the banks
__host__ __device__ constexpr int buf_stride(int n, int extra) { return n + (n >> 4) + extra; }
__device__ __forceinline__ int pad(int i) { return i + (i >> 4); }

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

// a * exp(-+2 pi i k / 16) for k in [0, 8) (- forward, + inverse); k is a
// compile-time constant after unrolling, so the switch folds away
template <bool INV>
__device__ __forceinline__ float2 w16(float2 a, int k)
{
    const float C = 0.92387953251128675613f;  // cos(pi / 8)
    const float S = 0.38268343236508977173f;  // sin(pi / 8)
    const float H = 0.70710678118654752440f;  // sqrt(1 / 2)
    float c, s;
    switch (k) {
    case 0: return a;
    case 4: return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
    case 1: c = C; s = S; break;
    case 2: c = H; s = H; break;
    case 3: c = S; s = C; break;
    case 5: c = -S; s = C; break;
    case 6: c = -H; s = H; break;
    default: c = -C; s = S; break;
    }
    if (!INV) s = -s;
    return make_float2(fmaf(a.x, c, -a.y * s), fmaf(a.x, s, a.y * c));
}

template <int R>
__host__ __device__ constexpr int bit_reverse(int i)
{
    int r = 0;
    for (int m = 1, b = R >> 1; m < R; m <<= 1, b >>= 1)
        if (i & m) r |= b;
    return r;
}

// in-register DFT of v[0, R), natural order in and out: radix-2 decimation
// in frequency (butterfly twiddle W_2h^j = W_16^(16 j / 2h)), then the
// bit-reversal permutation (register renaming)
template <int R, bool INV>
__device__ __forceinline__ void dft(float2 *v)
{
#pragma unroll
    for (int h = R / 2; h >= 1; h >>= 1) {
#pragma unroll
        for (int s = 0; s < R; s += 2 * h) {
#pragma unroll
            for (int j = 0; j < h; ++j) {
                const float2 a = v[s + j], b = v[s + j + h];
                v[s + j] = cadd(a, b);
                v[s + j + h] = w16<INV>(csub(a, b), j * (16 / (2 * h)));
            }
        }
    }
#pragma unroll
    for (int i = 0; i < R; ++i) {
        const int r = bit_reverse<R>(i);
        if (r > i) {
            const float2 t = v[i];
            v[i] = v[r];
            v[r] = t;
        }
    }
}

// Pass of a length-2^LGN transform over sub-transforms of length 2^LGNS:
// radix 2^LGR, LGR = 4 while four or more bits remain (LGNS is 0, 4 or 8).
template <int LGN, int LGNS>
struct Pass {
    static constexpr int LGR = (LGN - LGNS) >= 4 ? 4 : (LGN - LGNS);
    static constexpr int R = 1 << LGR, NS = 1 << LGNS, TP = 1 << (LGN - 4), NB = E / R;
    static constexpr bool LAST = LGNS + LGR == LGN;
    static constexpr int TWLEN = LGNS > 0 ? R * NS : 0;  // its twiddle table
};

__host__ __device__ constexpr int pass_lgr(int lgn, int lgns) { return (lgn - lgns) >= 4 ? 4 : (lgn - lgns); }
__host__ __device__ inline int twiddle_len(int lgn)
{
    int len = 0;
    for (int lgns = 0; lgns < lgn; lgns += pass_lgr(lgn, lgns))
        if (lgns > 0) len += 1 << (lgns + pass_lgr(lgn, lgns));
    return len;
}

// twiddles and butterflies of one pass; tw is the pass's table, entry
// r Ns + m = W_(Ns R)^(r m): consecutive lanes (consecutive m = j mod Ns) read
// consecutive entries
template <int LGN, int LGNS, bool INV>
__device__ __forceinline__ void pass_compute(float2 (&v)[E], int t, const float2 *__restrict__ tw)
{
    using P = Pass<LGN, LGNS>;
#pragma unroll
    for (int b = 0; b < P::NB; ++b) {
        if (LGNS > 0) {
            const float2 *tb = tw + ((t + b * P::TP) & (P::NS - 1));
#pragma unroll
            for (int r = 1; r < P::R; ++r) {
                float2 w = __ldg(tb + r * P::NS);
                if (INV) w.y = -w.y;
                v[b * P::R + r] = cmul(v[b * P::R + r], w);
            }
        }
        dft<P::R, INV>(v + b * P::R);
    }
}

// Registers of pass (LGN, LGNS): k = b R + r holds input r of butterfly
// j = t + b TP, element j + r N/R.  Where an offset is a multiple of 16,
// pad(x + c) = pad(x) + c + c/16 keeps it a compile-time offset.
template <int LGN, int LGNS, int NA>
__device__ __forceinline__ void load_pass(float2 (&v)[NA][E], float2 *const (&buf)[NA], int t)
{
    using P = Pass<LGN, LGNS>;
    constexpr int STRIDE = (1 << LGN) / P::R;
#pragma unroll
    for (int b = 0; b < P::NB; ++b) {
        const int x = t + b * P::TP, px = pad(x);
#pragma unroll
        for (int r = 0; r < P::R; ++r) {
            const int c = r * STRIDE;
            const int s = (STRIDE % 16 == 0) ? px + c + c / 16 : pad(x + c);
#pragma unroll
            for (int a = 0; a < NA; ++a) v[a][b * P::R + r] = buf[a][s];
        }
    }
}

// outputs of pass (LGN, LGNS): output r of butterfly j to
// (j / Ns) Ns R + (j mod Ns) + r Ns
template <int LGN, int LGNS, int NA>
__device__ __forceinline__ void store_pass(float2 (&v)[NA][E], float2 *const (&buf)[NA], int t)
{
    using P = Pass<LGN, LGNS>;
    static_assert(LGNS != 0 || P::R == 16, "the first pass is of radix 16");
#pragma unroll
    for (int b = 0; b < P::NB; ++b) {
        const int j = t + b * P::TP;
        if constexpr (LGNS == 0) {
            // slot pad(16 j + r) = 17 j + r
#pragma unroll
            for (int r = 0; r < P::R; ++r)
#pragma unroll
                for (int a = 0; a < NA; ++a) buf[a][17 * j + r] = v[a][b * P::R + r];
        } else {
            const int pd = pad(((j >> LGNS) << (LGNS + P::LGR)) + (j & (P::NS - 1)));
#pragma unroll
            for (int r = 0; r < P::R; ++r) {
                const int c = r * P::NS;  // Ns >= 16
#pragma unroll
                for (int a = 0; a < NA; ++a) buf[a][pd + c + c / 16] = v[a][b * P::R + r];
            }
        }
    }
}

// Transforms of length 2^LGN (16 <= n <= 4096), NA of them per thread (one
// buffer each).  On entry v[a][k] holds element t + k n/16 of transform a;
// on exit v[a][k] holds output element result_index<LGN>(k, t).  The buffers
// are free on entry and hold intermediate passes on exit.  Every thread of
// the block must call this (block-wide barriers).
template <int LGN, bool INV, int NA, int LGNS = 0>
__device__ __forceinline__ void transform(float2 (&v)[NA][E], float2 *const (&buf)[NA], int t,
                                          const float2 *__restrict__ tw)
{
    using P = Pass<LGN, LGNS>;
#pragma unroll
    for (int a = 0; a < NA; ++a) pass_compute<LGN, LGNS, INV>(v[a], t, tw);
    if constexpr (!P::LAST) {
        __syncthreads();  // every thread has read the previous contents
        store_pass<LGN, LGNS, NA>(v, buf, t);
        __syncthreads();
        load_pass<LGN, LGNS + P::LGR, NA>(v, buf, t);
        transform<LGN, INV, NA, LGNS + P::LGR>(v, buf, t, tw + P::TWLEN);
    }
}

// radix (log2) of the last pass of a length-2^lgn transform
__host__ __device__ constexpr int last_lgr(int lgn) { return (lgn & 3) ? (lgn & 3) : 4; }

// element index of register k after transform<LGN>: t + (k / R) n/16 +
// (k mod R) n/R, R the last pass's radix
template <int LGN>
__device__ __forceinline__ int result_index(int k, int t)
{
    constexpr int LGR = last_lgr(LGN);
    return t + (k >> LGR) * (1 << (LGN - 4)) + (k & ((1 << LGR) - 1)) * (1 << (LGN - LGR));
}

}  // namespace fft
}  // namespace pic
