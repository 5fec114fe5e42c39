// pic_adjoint_dev.cuh -- device functions of the adjoint of the step (CIC
// weights and their gradients, the transposed spectral solve per mode),
// shared by the single-run adjoint (pic_adjoint.cu) and the ensemble adjoint
// (pic_ensemble_adjoint.cu).
#pragma once
#include <cuda_runtime.h>

#include "pic_internal.cuh"

namespace pic {

struct Cic {
    int i00, i10, i01, i11;
    float fx, fy;
    bool ok;
};

__device__ __forceinline__ Cic cic_of(int c, float ox, float oy, int nx, int ny)
{
    Cic w;
    const int cx = c & 0xFFFF, cy = c >> 16;
    w.ok = c >= 0 && cx < nx && cy < ny;
    const int cx1 = (cx + 1 == nx) ? 0 : cx + 1, cy1 = (cy + 1 == ny) ? 0 : cy + 1;
    w.i00 = cy * nx + cx;
    w.i10 = cy * nx + cx1;
    w.i01 = cy1 * nx + cx;
    w.i11 = cy1 * nx + cx1;
    w.fx = ox;
    w.fy = oy;
    return w;
}

// sum_k grad w_k s_k, physical units
__device__ __forceinline__ float2 grad_dot(const Cic &w, float s00, float s10, float s01,
                                           float s11, float inv_dx, float inv_dy)
{
    const float fx = w.fx, fy = w.fy;
    return make_float2(((1.f - fy) * (s10 - s00) + fy * (s11 - s01)) * inv_dx,
                       ((1.f - fx) * (s01 - s00) + fx * (s11 - s10)) * inv_dy);
}

// One mode of psi = S^T g, the transpose of the field solve E = S rho:
// psi^ = i (kx g^x + ky g^y) / (eps0 N k^2) with the Nyquist derivative
// zeroed as in the forward solve and the zero mode removed (N folded in).
__device__ __forceinline__ float2 adj_mode(float2 a, float2 b, int mx, int my, int nx, int ny,
                                           float kx1, float ky1, float inv_eps0_n, bool zero_mode)
{
    const bool nx_even = (nx & 1) == 0, ny_even = (ny & 1) == 0;
    const int sy = (2 * my <= ny) ? my : my - ny;
    const float kx = kx1 * (float)mx, ky = ky1 * (float)sy;
    const float kxe = (nx_even && 2 * mx == nx) ? 0.f : kx;
    const float kye = (ny_even && 2 * my == ny) ? 0.f : ky;
    const float hr = kxe * a.x + kye * b.x, hi = kxe * a.y + kye * b.y;
    const float inv = zero_mode ? 0.f : inv_eps0_n / (kx * kx + ky * ky);
    return make_float2(-hi * inv, hr * inv);  // i (hr + i hi)
}

}  // namespace pic
