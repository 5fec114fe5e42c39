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

#include "pic_field_dev.cuh"

namespace pic {

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

// blocks walk rows of the half spectrum, threads the modes of a row
__global__ void __launch_bounds__(256) kspace_kernel(KspaceArgs A)
{
    __shared__ double s_part[8];
    const long long total = (long long)A.ny * A.nh;
    float fe = 0.f;
    for (int my = blockIdx.x; my < A.ny; my += gridDim.x)
    for (int mx = threadIdx.x; mx < A.nh; mx += blockDim.x) {
        const long long idx = (long long)my * A.nh + mx;
        const float2 r = A.rhohat[idx];
        const KMode K = kspace_mode(r, mx, my, A.nx, A.ny, A.kx1, A.ky1, A.inv_eps0_n, idx == 0);
        if (mx == A.tmx && my == A.tmy)
            A.dev->mode_amp = sqrt((double)r.x * r.x + (double)r.y * r.y) / ((double)A.nx * A.ny);
        if (A.phi_mode) {
            A.ehat[idx] = K.ph;
            continue;
        }
        A.ehat[idx] = K.ex;
        A.ehat[total + idx] = K.ey;
        fe += K.fe;
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

// diagnostics fold of one handle (one warp)
__global__ void advance_kernel(DevState *d, double *hist, int cap, int kind, double fe_scale)
{
    advance_state(d, hist, cap, kind, fe_scale);
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
    kspace_kernel<<<grid_for((long long)g.ny * 256, 256), 256, 0, h->stream>>>(A);
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
