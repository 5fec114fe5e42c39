// pic_field.cu -- the grid side of the step: fixed-point density to float,
// the k-space Poisson kernel, and per-step diagnostics bookkeeping.
//
// Replaces (reference paths inside taylorj5/msc-thesis,
// thesisCode/collisionless/double/src/):
//   fourier.cc:15-126 fftPoissonSolver   -> convert + cuFFT R2C + kspace + cuFFT C2R
//   grid.cc:85-96     computeElectricField (the field comes from E^ = -i k phi^
//                                           in the same k-space kernel)
// with physical conventions: k = 2 pi m / L, phi^ = rho^ / (eps0 k^2), the
// zero mode removed (immobile neutralising background) and one 1/N.
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

// rho = (rho_fix - mean) * scale, sum(rho_fix) -> dev->q; rho_fix is cleared
// by a memset after this kernel.  The background is removed in exact integer
// arithmetic before the single rounding to float, so small perturbations of a
// large mean keep their relative precision.  Two cells per thread per
// iteration (16-byte loads, 8-byte stores; n is even).
__global__ void __launch_bounds__(256)
convert_kernel(const unsigned long long *__restrict__ rho_fix, float *__restrict__ rho, long long n,
               long long mean_fix, float scale, DevState *dev)
{
    __shared__ unsigned long long s_part[8];
    unsigned long long qs = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long n2 = n >> 1;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += stride) {
        const ulonglong2 v = reinterpret_cast<const ulonglong2 *>(rho_fix)[i];
        qs += v.x + v.y;
        reinterpret_cast<float2 *>(rho)[i] =
            make_float2(fixed_to_float(v.x, mean_fix, scale), fixed_to_float(v.y, mean_fix, scale));
    }
    if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        const unsigned long long v = rho_fix[n - 1];
        qs += v;
        rho[n - 1] = fixed_to_float(v, mean_fix, scale);
    }
    qs = warp_sum_u64(qs);
    if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = qs;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_part[w];
        atomicAdd(&dev->q[acc_slot()], t);
    }
}

struct KspaceArgs {
    const float2 *rhohat;
    float2 *ehat;    // [2][ny][nh] (E mode) or phi^ (phi mode)
    int nx, ny, nh;
    float kx1, ky1;  // 2 pi / Lx, 2 pi / Ly
    float inv_eps0_n;  // 1 / (eps0 nx ny): folds the C2R normalisation in
    int phi_mode;
    int tmx, tmy;      // tracked mode (tmx < 0: none)
    DevState *dev;
};

__global__ void __launch_bounds__(256) kspace_kernel(KspaceArgs A)
{
    __shared__ double s_part[8];
    const long long total = (long long)A.ny * A.nh;
    const bool nx_even = (A.nx & 1) == 0, ny_even = (A.ny & 1) == 0;
    float fe = 0.f;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += stride) {
        const int my = (int)(idx / A.nh);
        const int mx = (int)(idx - (long long)my * A.nh);
        const int sy = (2 * my <= A.ny) ? my : my - A.ny;
        const float kx = A.kx1 * (float)mx, ky = A.ky1 * (float)sy;
        const float k2 = kx * kx + ky * ky;
        const float2 r = A.rhohat[idx];
        const float inv = (idx == 0) ? 0.f : A.inv_eps0_n / k2;
        const float2 ph = make_float2(r.x * inv, r.y * inv);
        if (mx == A.tmx && my == A.tmy)
            A.dev->mode_amp = sqrt((double)r.x * r.x + (double)r.y * r.y) / ((double)A.nx * A.ny);
        if (A.phi_mode) {
            A.ehat[idx] = ph;
            continue;
        }
        // E^ = -i k phi^; the Nyquist component of a derivative is set to zero
        const float kxe = (nx_even && 2 * mx == A.nx) ? 0.f : kx;
        const float kye = (ny_even && 2 * my == A.ny) ? 0.f : ky;
        const float2 ex = make_float2(kxe * ph.y, -kxe * ph.x);
        const float2 ey = make_float2(kye * ph.y, -kye * ph.x);
        A.ehat[idx] = ex;
        A.ehat[total + idx] = ey;
        const float w = (mx == 0 || (nx_even && 2 * mx == A.nx)) ? 1.f : 2.f;
        fe += w * (ex.x * ex.x + ex.y * ex.y + ey.x * ey.x + ey.y * ey.y);
    }
    if (A.phi_mode) return;
    double d = warp_sum_d((double)fe);
    if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = d;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_part[w];
        atomicAdd(&A.dev->fe[acc_slot()], t);
    }
}

// Moves the accumulators of the finished stage into the history ring and
// clears them; one warp, lane l folds slot l.  ADV_PUSH closes the particle
// pass of step s (kinetic energy and momentum belong to step s) and advances
// the step counter; ADV_FIELD records the field of the current step.
__global__ void advance_kernel(DevState *d, double *hist, int cap, int kind, double fe_scale)
{
    const int l = threadIdx.x;  // 32 threads = ACC_SLOTS
    const long long s = d->step;
    const int k = (int)(s % cap);
    if (kind == ADV_PUSH) {
        const double ke = warp_sum_d(d->ke[l]), px = warp_sum_d(d->px[l]), py = warp_sum_d(d->py[l]);
        d->ke[l] = d->px[l] = d->py[l] = 0.0;
        if (l == 0) {
            hist[1 * (size_t)cap + k] = ke;
            hist[2 * (size_t)cap + k] = px;
            hist[3 * (size_t)cap + k] = py;
            d->step = s + 1;
        }
    } else {
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

pic_status launch_convert(pic_handle *h)
{
    const Geometry &g = h->g;
    const long long n = (long long)g.nx * g.ny;
    const float scale = (float)(h->q_unit / (4294967296.0 * g.dx * g.dy));
    convert_kernel<<<grid_for((n + 1) / 2, 256), 256, 0, h->stream>>>(h->rho_fix, h->rho, n,
                                                                    h->mean_fix, scale, h->dev);
    PIC_CUDA(cudaGetLastError());
    PIC_CUDA(cudaMemsetAsync(h->rho_fix, 0, sizeof(unsigned long long) * (size_t)n, h->stream));
    return PIC_OK;
}

pic_status launch_kspace(pic_handle *h, bool phi_only, float2 *phihat)
{
    const Geometry &g = h->g;
    KspaceArgs A;
    A.rhohat = h->rhohat;
    A.ehat = phi_only ? phihat : h->ehat;
    A.nx = g.nx;
    A.ny = g.ny;
    A.nh = g.nh;
    A.kx1 = (float)(2.0 * 3.14159265358979323846 / g.Lx);
    A.ky1 = (float)(2.0 * 3.14159265358979323846 / g.Ly);
    A.inv_eps0_n = (float)(1.0 / (h->cfg.eps0 * (double)g.nx * (double)g.ny));
    A.phi_mode = phi_only ? 1 : 0;
    A.tmx = phi_only ? -1 : h->track_mx;
    A.tmy = phi_only ? -1 : h->track_my;
    A.dev = h->dev;
    const long long total = (long long)g.ny * g.nh;
    kspace_kernel<<<grid_for(total, 256), 256, 0, h->stream>>>(A);
    PIC_CUDA(cudaGetLastError());
    return PIC_OK;
}

pic_status launch_advance(pic_handle *h, int kind)
{
    const Geometry &g = h->g;
    // sum_n |E_n|^2 = N sum_k |E'^_k|^2 with E' the 1/N-scaled spectrum
    const double fe_scale = 0.5 * h->cfg.eps0 * g.dx * g.dy * (double)g.nx * (double)g.ny;
    advance_kernel<<<1, ACC_SLOTS, 0, h->stream>>>(h->dev, h->hist, h->hist_cap, kind, fe_scale);
    PIC_CUDA(cudaGetLastError());
    return PIC_OK;
}

}  // namespace pic
