// pic_field_dev.cuh -- device functions of the grid side of the step
// (fixed-point conversion, the k-space Poisson operator per mode, the
// diagnostics fold), shared by the single-run kernels (pic_field.cu) and the
// ensemble kernels (pic_ensemble.cu).
#pragma once
#include <cuda_runtime.h>

#include "pic_internal.cuh"

namespace pic {

__device__ __forceinline__ double warp_sum_d(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float fixed_to_float(unsigned long long v, long long mean_fix, float scale)
{
    // int64 -> float as hi * 2^32 + lo: two 32-bit conversions and one fma
    // (at most one extra rounding)
    const long long d = (long long)v - mean_fix;
    return fmaf((float)(int)(d >> 32), 4294967296.0f, (float)(unsigned)(d & 0xFFFFFFFFll)) * scale;
}

// One mode of the Poisson solve: phi^ = rho^ inv_eps0_n / k^2 (zero mode
// removed), E^ = -i k phi^ with the Nyquist component of each derivative
// set to zero, and the mode's weighted |E^|^2 for the Parseval sum (the
// half spectrum counts interior columns twice).
struct KMode {
    float2 ph, ex, ey;
    float fe;
};

__device__ __forceinline__ KMode kspace_mode(float2 r, int mx, int my, int nx, int ny, float kx1,
                                             float ky1, float inv_eps0_n, bool zero_mode)
{
    const bool nx_even = (nx & 1) == 0, ny_even = (ny & 1) == 0;
    const int sy = (2 * my <= ny) ? my : my - ny;
    const float kx = kx1 * (float)mx, ky = ky1 * (float)sy;
    const float k2 = kx * kx + ky * ky;
    const float inv = zero_mode ? 0.f : inv_eps0_n / k2;
    KMode K;
    K.ph = make_float2(r.x * inv, r.y * inv);
    const float kxe = (nx_even && 2 * mx == nx) ? 0.f : kx;
    const float kye = (ny_even && 2 * my == ny) ? 0.f : ky;
    K.ex = make_float2(kxe * K.ph.y, -kxe * K.ph.x);
    K.ey = make_float2(kye * K.ph.y, -kye * K.ph.x);
    const float w = (mx == 0 || (nx_even && 2 * mx == nx)) ? 1.f : 2.f;
    K.fe = w * (K.ex.x * K.ex.x + K.ex.y * K.ex.y + K.ey.x * K.ey.x + K.ey.y * K.ey.y);
    return K;
}

// Moves the accumulators of the finished stage into the history ring and
// clears them; one warp, lane l folds slot l.  ADV_PUSH closes the particle
// pass of step s (kinetic energy and momentum belong to step s) and advances
// the step counter; ADV_FIELD records the field of the current step (after
// the push fold when both bits are set).
__device__ __forceinline__ void advance_state(DevState *d, double *hist, int cap, int kind,
                                              double fe_scale)
{
    const int l = threadIdx.x;  // 32 threads = ACC_SLOTS
    long long s = d->step;
    int k = (int)(s % cap);
    if (kind & ADV_PUSH) {
        const double ke = warp_sum_d(d->ke[l]), px = warp_sum_d(d->px[l]), py = warp_sum_d(d->py[l]);
        d->ke[l] = d->px[l] = d->py[l] = 0.0;
        if (l == 0) {
            hist[1 * (size_t)cap + k] = ke;
            hist[2 * (size_t)cap + k] = px;
            hist[3 * (size_t)cap + k] = py;
            d->step = s + 1;
        }
        k = (int)(++s % cap);
    }
    if (kind & ADV_FIELD) {
        const double fe = warp_sum_d(d->fe[l]);
        const unsigned long long q = warp_sum_u64(d->q[l]);
        d->fe[l] = 0.0;
        d->q[l] = 0ull;
        if (l == 0) {
            hist[0 * (size_t)cap + k] = fe * fe_scale;
            hist[4 * (size_t)cap + k] = (double)(long long)q;
            hist[5 * (size_t)cap + k] = d->mode_amp;
            d->mode_amp = 0.0;
        }
    }
}

}  // namespace pic
