// pic_push.cu -- the particle pass of the step: CIC field gather, leapfrog
// push and fixed-point CIC deposit of the new positions, fused in one kernel.
//
// Replaces, in one pass over the particle arrays (reference paths inside
// taylorj5/msc-thesis, thesisCode/collisionless/double/src/):
//   particle.cc:37-60  Particle::forceCalculation   (gather)
//   particle.cc:69-106 Particle::positionUpdate     (push)
//   grid.cc:46-76      Grid::chargeAssignment       (deposit, for the next step)
//
// Work decomposition: the particle arrays are kept sorted by cell tile (see
// pic_sort.cu), and block b processes particles [b*chunk, (b+1)*chunk).
// The sort records for every chunk the tile of its first particle; the block
// stages a window of two tiles plus a halo of E in shared memory, gathers
// from it, and accumulates its deposit in a shared-memory fixed-point tile
// that is flushed to the global density with 64-bit atomics at the end.
// Particles that have drifted outside the window since the last sort take
// the global path (direct loads and atomics), so the result never depends
// on how stale the sort is.
//
// Deposit arithmetic is exact: with fx = rint(ox 2^16), fy = rint(oy 2^16)
// the four node weights (2^16-fx)(2^16-fy), fx(2^16-fy), (2^16-fx)fy, fx fy
// are integers that sum to 2^32 for every particle, so the density in
// 2^-32 charge units is an integer sum, independent of summation order, and
// the total charge is exact.  Each thread owns four consecutive particles of
// the sorted array (one 128-bit load per field); those that land in the same
// cell are combined in registers (the four weights of a group follow from the
// group's count and sums of fx, fy and fx*fy) before one set of atomics.  In
// shared memory every node keeps two 32-bit accumulators, the low 16 bits and
// the rest of its unsigned weight, so the hot atomics are native 32-bit adds;
// the charge sign is applied once per node when the window is flushed with a
// 64-bit atomic to the global density.
#include <cuda_runtime.h>

#include "pic_internal.cuh"

namespace pic {

struct Cic4 {
    unsigned long long w00, w10, w01, w11;
};

// Node weights of `cnt` particles in one cell from their sums of fx, fy, fx*fy.
__device__ __forceinline__ Cic4 cic_weights(unsigned cnt, unsigned sfx, unsigned sfy,
                                            unsigned long long sxy)
{
    Cic4 W;
    W.w11 = sxy;
    W.w10 = ((unsigned long long)sfx << 16) - sxy;
    W.w01 = ((unsigned long long)sfy << 16) - sxy;
    W.w00 = ((unsigned long long)cnt << 32) - ((unsigned long long)(sfx + sfy) << 16) + sxy;
    return W;
}

__device__ __forceinline__ void deposit_global(unsigned long long *rho, int nx, int ny, int cx,
                                               int cy, const Cic4 &W, unsigned long long q)
{
    const int cx1 = (cx + 1 == nx) ? 0 : cx + 1;
    const int cy1 = (cy + 1 == ny) ? 0 : cy + 1;
    atomicAdd(rho + (size_t)cy * nx + cx, W.w00 * q);
    atomicAdd(rho + (size_t)cy * nx + cx1, W.w10 * q);
    atomicAdd(rho + (size_t)cy1 * nx + cx, W.w01 * q);
    atomicAdd(rho + (size_t)cy1 * nx + cx1, W.w11 * q);
}

__device__ __forceinline__ void smem_add(unsigned *lo, unsigned *hi, int i, unsigned long long w)
{
    atomicAdd(lo + i, (unsigned)(w & 0xFFFFull));
    atomicAdd(hi + i, (unsigned)(w >> 16));
}

struct PushArgs {
    const int32_t *cin;
    const float *oxin, *oyin, *vxin, *vyin;
    int32_t *cout;
    float *oxout, *oyout, *vxout, *vyout;
    const uint32_t *pidin;  // copied to pidout when non-null (out-of-place pass)
    uint32_t *pidout;
    const float *vzin;      // copied to vzout when non-null
    float *vzout;
    const int32_t *anchor;
    const long long *d_n;
    const float *ex, *ey;
    unsigned long long *rho;
    DevState *dev;
    int nx, ny, tw, th, halo, wcx, wcy, chunk;
    float qm_dt, dtdx, dtdy;
    unsigned long long qmul;  // q_int as two's complement
    double ke_scale, p_scale; // m/4, m/2 (0 disables the diagnostics)
};

template <bool GATHER, bool DEPOSIT>
__global__ void __launch_bounds__(256) push_kernel(PushArgs A)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const long long n = *A.d_n;
    const long long base = (long long)blockIdx.x * A.chunk;
    if (base >= n) return;  // block-uniform
    const long long n4 = (n + 3) & ~3ll;
    const long long end = min(base + (long long)A.chunk, n4);
    const int nx = A.nx, ny = A.ny;

    const int nwx = A.wcx + 1, nwy = A.wcy + 1, nw = nwx * nwy;
    float2 *sE = reinterpret_cast<float2 *>(smem);
    unsigned *sLo = reinterpret_cast<unsigned *>(smem + (size_t)nw * sizeof(float2));
    unsigned *sHi = sLo + nw;
    double *sAcc = reinterpret_cast<double *>(smem + (size_t)nw * 16);

    const int anc = A.anchor[blockIdx.x];
    const bool win = anc >= 0;
    int wx0 = 0, wy0 = 0;
    if (win) {
        wx0 = (anc & 0xFFFF) * A.tw - A.halo;
        wy0 = (anc >> 16) * A.th - A.halo;
        wx0 %= nx;
        if (wx0 < 0) wx0 += nx;
        wy0 %= ny;
        if (wy0 < 0) wy0 += ny;
        for (int i = threadIdx.x; i < nw; i += blockDim.x) {
            const int a = i % nwx, b = i / nwx;
            const int gx = (wx0 + a) % nx, gy = (wy0 + b) % ny;
            if (GATHER) sE[i] = make_float2(A.ex[(size_t)gy * nx + gx], A.ey[(size_t)gy * nx + gx]);
            if (DEPOSIT) {
                sLo[i] = 0u;
                sHi[i] = 0u;
            }
        }
    }
    if (threadIdx.x < 3) sAcc[threadIdx.x] = 0.0;
    __syncthreads();

    // deposit of one group of particles in one cell: window or global
    auto deposit = [&](int cx, int cy, const Cic4 &W) {
        int dxl = cx - wx0, dyl = cy - wy0;
        if (dxl < 0) dxl += nx;
        if (dyl < 0) dyl += ny;
        if (win && dxl < A.wcx && dyl < A.wcy) {
            const int i = dyl * nwx + dxl;
            smem_add(sLo, sHi, i, W.w00);
            smem_add(sLo, sHi, i + 1, W.w10);
            smem_add(sLo, sHi, i + nwx, W.w01);
            smem_add(sLo, sHi, i + nwx + 1, W.w11);
        } else {
            deposit_global(A.rho, nx, ny, cx, cy, W, A.qmul);
        }
    };

    float ke = 0.f, px = 0.f, py = 0.f;
    bool bad = false;
    for (long long q = base + 4ll * threadIdx.x; q < end; q += 4ll * blockDim.x) {
        // plain (coherent) loads: with an in-place pass the same addresses are stored below
        const int4 c4 = *reinterpret_cast<const int4 *>(A.cin + q);
        const float4 a4 = *reinterpret_cast<const float4 *>(A.oxin + q);
        const float4 b4 = *reinterpret_cast<const float4 *>(A.oyin + q);
        const float4 u4 = *reinterpret_cast<const float4 *>(A.vxin + q);
        const float4 v4 = *reinterpret_cast<const float4 *>(A.vyin + q);
        int cc[4] = {c4.x, c4.y, c4.z, c4.w};
        float xo[4] = {a4.x, a4.y, a4.z, a4.w}, yo[4] = {b4.x, b4.y, b4.z, b4.w};
        float xv[4] = {u4.x, u4.y, u4.z, u4.w}, yv[4] = {v4.x, v4.y, v4.z, v4.w};
        // register aggregate of the particles that share the first one's new cell
        unsigned gcnt = 0u, gfx = 0u, gfy = 0u;
        unsigned long long gxy = 0ull;
        int gkey = -1, gcx = 0, gcy = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = cc[j];
            if (c < 0) continue;  // empty slot
            int cx = c & 0xFFFF, cy = c >> 16;
            if (cx >= nx || cy >= ny) {  // corrupt cell: flag, leave untouched
                bad = true;
                atomicOr(&A.dev->err, (unsigned)PIC_DEVERR_CELL);
                continue;
            }
            float ox = xo[j], oy = yo[j], vx = xv[j], vy = yv[j];
            if (GATHER) {
                const float gx = 1.f - ox, gy = 1.f - oy;
                float2 e00, e10, e01, e11;
                int dxl = cx - wx0, dyl = cy - wy0;
                if (dxl < 0) dxl += nx;
                if (dyl < 0) dyl += ny;
                if (win && dxl < A.wcx && dyl < A.wcy) {
                    const int i = dyl * nwx + dxl;
                    e00 = sE[i];
                    e10 = sE[i + 1];
                    e01 = sE[i + nwx];
                    e11 = sE[i + nwx + 1];
                } else {
                    const int cx1 = (cx + 1 == nx) ? 0 : cx + 1;
                    const int cy1 = (cy + 1 == ny) ? 0 : cy + 1;
                    const size_t i00 = (size_t)cy * nx + cx, i10 = (size_t)cy * nx + cx1;
                    const size_t i01 = (size_t)cy1 * nx + cx, i11 = (size_t)cy1 * nx + cx1;
                    e00 = make_float2(A.ex[i00], A.ey[i00]);
                    e10 = make_float2(A.ex[i10], A.ey[i10]);
                    e01 = make_float2(A.ex[i01], A.ey[i01]);
                    e11 = make_float2(A.ex[i11], A.ey[i11]);
                }
                const float Ex = gy * fmaf(gx, e00.x, ox * e10.x) + oy * fmaf(gx, e01.x, ox * e11.x);
                const float Ey = gy * fmaf(gx, e00.y, ox * e10.y) + oy * fmaf(gx, e01.y, ox * e11.y);
                const float vx0 = vx, vy0 = vy;
                vx = fmaf(A.qm_dt, Ex, vx);
                vy = fmaf(A.qm_dt, Ey, vy);
                ke = fmaf(vx0, vx0, fmaf(vy0, vy0, fmaf(vx, vx, fmaf(vy, vy, ke))));
                px += vx0 + vx;
                py += vy0 + vy;
            } else {
                ke = fmaf(2.f * vx, vx, fmaf(2.f * vy, vy, ke));
                px = fmaf(2.f, vx, px);
                py = fmaf(2.f, vy, py);
            }
            bad |= !(fabsf(vx) <= 3.0e38f) || !(fabsf(vy) <= 3.0e38f);
            // drift in cell units; carry whole cells into the index
            ox = fmaf(vx, A.dtdx, ox);
            oy = fmaf(vy, A.dtdy, oy);
            float sx = floorf(ox), sy = floorf(oy);
            ox -= sx;
            oy -= sy;
            if (ox >= 1.f) { ox -= 1.f; sx += 1.f; }
            if (oy >= 1.f) { oy -= 1.f; sy += 1.f; }
            cx += (int)sx;
            cy += (int)sy;
            if ((unsigned)cx >= (unsigned)nx) { cx %= nx; if (cx < 0) cx += nx; }
            if ((unsigned)cy >= (unsigned)ny) { cy %= ny; if (cy < 0) cy += ny; }
            const int cn = cx | (cy << 16);
            cc[j] = cn;
            xo[j] = ox;
            yo[j] = oy;
            xv[j] = vx;
            yv[j] = vy;
            if (DEPOSIT) {
                const unsigned fx = __float2uint_rn(ox * 65536.0f);
                const unsigned fy = __float2uint_rn(oy * 65536.0f);
                const unsigned long long fxy = (unsigned long long)fx * fy;
                if (gkey < 0) {
                    gkey = cn;
                    gcx = cx;
                    gcy = cy;
                }
                if (cn == gkey) {
                    ++gcnt;
                    gfx += fx;
                    gfy += fy;
                    gxy += fxy;
                } else {
                    deposit(cx, cy, cic_weights(1u, fx, fy, fxy));
                }
            }
        }
        if (DEPOSIT && gcnt) deposit(gcx, gcy, cic_weights(gcnt, gfx, gfy, gxy));
        *reinterpret_cast<int4 *>(A.cout + q) = make_int4(cc[0], cc[1], cc[2], cc[3]);
        *reinterpret_cast<float4 *>(A.oxout + q) = make_float4(xo[0], xo[1], xo[2], xo[3]);
        *reinterpret_cast<float4 *>(A.oyout + q) = make_float4(yo[0], yo[1], yo[2], yo[3]);
        *reinterpret_cast<float4 *>(A.vxout + q) = make_float4(xv[0], xv[1], xv[2], xv[3]);
        *reinterpret_cast<float4 *>(A.vyout + q) = make_float4(yv[0], yv[1], yv[2], yv[3]);
        if (A.pidin)
            *reinterpret_cast<uint4 *>(A.pidout + q) = *reinterpret_cast<const uint4 *>(A.pidin + q);
        if (A.vzin)
            *reinterpret_cast<float4 *>(A.vzout + q) = *reinterpret_cast<const float4 *>(A.vzin + q);
    }

    // diagnostics: FP32 per thread and per warp, FP64 across warps and blocks
    if (A.ke_scale != 0.0) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            ke += __shfl_xor_sync(0xffffffffu, ke, o);
            px += __shfl_xor_sync(0xffffffffu, px, o);
            py += __shfl_xor_sync(0xffffffffu, py, o);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(sAcc + 0, (double)ke);
            atomicAdd(sAcc + 1, (double)px);
            atomicAdd(sAcc + 2, (double)py);
        }
    }
    const int any_bad = __syncthreads_or(bad ? 1 : 0);
    if (threadIdx.x == 0) {
        if (A.ke_scale != 0.0) {
            atomicAdd(&A.dev->ke, sAcc[0] * A.ke_scale);
            atomicAdd(&A.dev->px, sAcc[1] * A.p_scale);
            atomicAdd(&A.dev->py, sAcc[2] * A.p_scale);
        }
        if (any_bad) atomicOr(&A.dev->err, (unsigned)PIC_DEVERR_NAN);
    }
    if (DEPOSIT && win) {
        for (int i = threadIdx.x; i < nw; i += blockDim.x) {
            const unsigned long long v = ((unsigned long long)sHi[i] << 16) + sLo[i];
            if (v) {
                const int a = i % nwx, b = i / nwx;
                const int gx = (wx0 + a) % nx, gy = (wy0 + b) % ny;
                atomicAdd(A.rho + (size_t)gy * nx + gx, v * A.qmul);
            }
        }
    }
}

// Deposit-only pass (after a sort or an import, before the first step):
// fixed-point CIC straight to the global density, one particle per thread.
__global__ void __launch_bounds__(256)
deposit_flat_kernel(const int32_t *__restrict__ cell, const float *__restrict__ ox,
                    const float *__restrict__ oy, const long long *d_n, long long n_host,
                    int nx, int ny, unsigned long long qmul, unsigned long long *rho,
                    unsigned int *err)
{
    const long long n = d_n ? *d_n : n_host;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int c = cell[i];
        if (c < 0) continue;
        const int cx = c & 0xFFFF, cy = c >> 16;
        if (cx >= nx || cy >= ny) {
            if (err) atomicOr(err, (unsigned)PIC_DEVERR_CELL);
            continue;
        }
        const unsigned fx = __float2uint_rn(ox[i] * 65536.0f);
        const unsigned fy = __float2uint_rn(oy[i] * 65536.0f);
        deposit_global(rho, nx, ny, cx, cy, cic_weights(1u, fx, fy, (unsigned long long)fx * fy),
                       qmul);
    }
}

__global__ void fixed_to_double_kernel(const unsigned long long *__restrict__ src, long long n,
                                       double scale, double *__restrict__ dst)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        dst[i] = (double)(long long)src[i] * scale;
}

static size_t push_smem(const Geometry &g)
{
    return (size_t)(g.wcx + 1) * (g.wcy + 1) * 16 + 32;
}

pic_status launch_push(pic_handle *h, int s, int src, bool deposit, float dt_scale)
{
    SpeciesBuf &B = h->sp[s];
    const pic_species_desc &D = h->cfg.species[s];
    const Geometry &g = h->g;
    if (B.nchunks == 0) return PIC_OK;
    PushArgs A;
    A.cin = B.cell[src];
    A.oxin = B.ox[src];
    A.oyin = B.oy[src];
    A.vxin = B.vx[src];
    A.vyin = B.vy[src];
    A.cout = B.cell[0];
    A.oxout = B.ox[0];
    A.oyout = B.oy[0];
    A.vxout = B.vx[0];
    A.vyout = B.vy[0];
    A.pidin = src ? B.pid[1] : nullptr;
    A.pidout = B.pid[0];
    A.vzin = (src && B.vz[1]) ? B.vz[1] : nullptr;
    A.vzout = B.vz[0];
    A.anchor = B.anchor;
    A.d_n = &h->dev->n[s];
    A.ex = h->e;
    A.ey = h->e + (size_t)g.nx * g.ny;
    A.rho = h->rho_fix;
    A.dev = h->dev;
    A.nx = g.nx;
    A.ny = g.ny;
    A.tw = g.tw;
    A.th = g.th;
    A.halo = g.halo;
    A.wcx = g.wcx;
    A.wcy = g.wcy;
    A.chunk = g.chunk;
    const double dt = h->cfg.dt * dt_scale;
    const bool move = dt_scale > 0.0f;
    A.qm_dt = (float)(D.q / D.m * dt);
    A.dtdx = move ? (float)(h->cfg.dt / g.dx) : 0.f;
    A.dtdy = move ? (float)(h->cfg.dt / g.dy) : 0.f;
    A.qmul = (unsigned long long)(long long)D.q_int;
    A.ke_scale = move ? 0.25 * D.m : 0.0;
    A.p_scale = 0.5 * D.m;
    const bool charged = D.q != 0.0;
    const bool dep = deposit && D.q_int != 0;
    const size_t sm = push_smem(g);
    dim3 grid((unsigned)B.nchunks), block(256);
    if (charged && dep)
        push_kernel<true, true><<<grid, block, sm, h->stream>>>(A);
    else if (charged)
        push_kernel<true, false><<<grid, block, sm, h->stream>>>(A);
    else if (dep)
        push_kernel<false, true><<<grid, block, sm, h->stream>>>(A);
    else
        push_kernel<false, false><<<grid, block, sm, h->stream>>>(A);
    PIC_CUDA(cudaGetLastError());
    return PIC_OK;
}

pic_status launch_deposit(pic_handle *h, int s)
{
    SpeciesBuf &B = h->sp[s];
    const pic_species_desc &D = h->cfg.species[s];
    if (D.q_int == 0 || B.cap == 0) return PIC_OK;
    deposit_flat_kernel<<<grid_for(B.cap, 256), 256, 0, h->stream>>>(
        B.cell[0], B.ox[0], B.oy[0], &h->dev->n[s], 0, h->g.nx, h->g.ny,
        (unsigned long long)(long long)D.q_int, h->rho_fix, &h->dev->err);
    PIC_CUDA(cudaGetLastError());
    return PIC_OK;
}

}  // namespace pic

// ---------------------------------------------------------------- C ABI
extern "C" pic_status pic_deposit_grid(int nx, int ny, long long n, const int32_t *cell_dev,
                                       const float *ox_dev, const float *oy_dev, int q_int,
                                       double scale, double *rho_dev, void *stream)
{
    using namespace pic;
    if (nx < 1 || ny < 1 || nx > 32768 || ny > 32768 || n < 0 || !rho_dev ||
        (n > 0 && (!cell_dev || !ox_dev || !oy_dev))) {
        set_error("pic_deposit_grid: bad grid size, count or pointer");
        return PIC_ERR_INVALID_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    const long long ng = (long long)nx * ny;
    unsigned long long *acc = nullptr;
    PIC_CUDA(cudaMalloc(&acc, (size_t)ng * sizeof(unsigned long long)));
    pic_status rc = PIC_OK;
    cudaError_t e = cudaMemsetAsync(acc, 0, (size_t)ng * sizeof(unsigned long long), st);
    if (e == cudaSuccess && n > 0) {
        deposit_flat_kernel<<<grid_for(n, 256), 256, 0, st>>>(cell_dev, ox_dev, oy_dev, nullptr, n,
                                                             nx, ny, 1ull, acc, nullptr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        fixed_to_double_kernel<<<grid_for(ng, 256), 256, 0, st>>>(
            acc, ng, (double)q_int * scale / 4294967296.0, rho_dev);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_fail(e, "pic_deposit_grid");
    cudaFree(acc);
    return rc;
}
