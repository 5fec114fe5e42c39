// pic_compat.cu -- the reference's step, with its CPU conventions, in FP64 on
// the GPU: the drop-in for picFloatGpu.
//
// Follows, operation for operation where the GPU allows (reference paths in
// taylorj5/msc-thesis, thesisCode/collisionless/double/):
//   src/grid.cc:46-76      chargeAssignment: CIC weights to the opposite corner
//                          nodes, written at ghost-padded index (1+cx, 1+cy),
//                          q*w per node, then the periodic ghost copy
//   src/fourier.cc:15-126  fftPoissonSolver: k = 2 pi m, the second index
//                          mapped with `2*j < nyh` (so j >= nyh/2 maps to j-ny),
//                          phi^ = -rho^/k^2, normalised twice by 1/(nx ny)
//   src/grid.cc:85-96      computeElectricField: central differences, Ex along
//                          the second index, Ey along the first, interior only
//   src/particle.cc:37-106 forceCalculation (E read at (cx, cy) without the
//                          ghost offset) and the lagged kick-drift-kick
//                          positionUpdate with forceOld, wrap with `>` and `< 0`
// The deposit uses FP64 atomics (the reference's GPU kernel races,
// src/pic.cu:124-127); the density is zeroed every step and forceOld starts at
// zero for every particle (the reference GPU path copies it with a grid-sized
// launch, src/pic.cu:574-575).  This file is compiled with --fmad=false so no
// multiply-add is contracted, as in the reference's x86 build.
#include <cuda_runtime.h>
#include <cufft.h>

#include <chrono>
#include <vector>

#include "pic_internal.cuh"

namespace pic {

struct CompatDev {
    int nx, ny, X, Y, nyh;
    int xDim, yDim;
    double dx, dy, area, q, qm, dt;
    long long np;
    double *px, *py, *cx, *cy, *vx, *vy, *fox, *foy;
    double *rho, *phi, *ex, *ey, *fin;
    cufftDoubleComplex *fout;
};

__global__ void compat_deposit_kernel(CompatDev D)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    const int Y = D.Y;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < D.np; k += stride) {
        const double X_ = D.px[k], Y_ = D.py[k], cx = D.cx[k], cy = D.cy[k];
        // cells run 0..nx (a particle exactly at x = xDim has cell nx); anything
        // else would index outside the padded grid, so it is skipped
        if (!(cx >= 0 && cx <= D.nx && cy >= 0 && cy <= D.ny)) continue;
        const double dx = D.dx, dy = D.dy, A = D.area;
        const double a1 = __ddiv_rn(__dmul_rn(X_ - cx * dx, Y_ - cy * dy), A);
        const double a2 = __ddiv_rn(__dmul_rn((cx * dx + dx) - X_, Y_ - cy * dy), A);
        const double a3 = __ddiv_rn(__dmul_rn(X_ - cx * dx, (cy * dy + dy) - Y_), A);
        const double a4 = __ddiv_rn(__dmul_rn((cx * dx + dx) - X_, (cy * dy + dy) - Y_), A);
        const int icx = (int)cx, icy = (int)cy;
        const int ix1 = (int)(cx + 1) % D.nx, iy1 = (int)(cy + 1) % D.ny;
        atomicAdd(D.rho + (size_t)((1 + cx) * Y + (1 + cy)), a1 * D.q);
        atomicAdd(D.rho + (size_t)((1 + ix1) * Y + (1 + icy)), a2 * D.q);
        atomicAdd(D.rho + (size_t)((1 + icx) * Y + (1 + iy1)), a3 * D.q);
        atomicAdd(D.rho + (size_t)((1 + ix1) * Y + (1 + iy1)), a4 * D.q);
    }
}

// Periodic ghost copy of a padded grid, two loops as the reference runs them
// (grid.cc:66-75 for rho with first = 0, fourier.cc:108-115 for phi with
// first = 1).  One block; the loops have no intra-loop dependencies.
__global__ void compat_ghost_kernel(double *g, int nx, int ny, int first)
{
    const int Y = ny + 2, nxe = nx + 2, nye = ny + 2;
    const int last = first ? nye - 1 : nye;
    for (int i = first + threadIdx.x; i < last; i += blockDim.x) {
        g[i] = g[nx * Y + i];
        g[(nxe - 1) * Y + i] = g[Y + i];
    }
    __syncthreads();
    for (int i = 1 + threadIdx.x; i < nxe - 1; i += blockDim.x) {
        g[i * Y] = g[i * Y + ny];
        g[i * Y + (nye - 1)] = g[i * Y + 1];
    }
}

__global__ void compat_pack_kernel(CompatDev D)
{
    const long long n = (long long)D.nx * D.ny;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t / D.ny), j = (int)(t % D.ny);
        D.fin[t] = D.rho[(i + 1) * D.Y + (j + 1)];
    }
}

__global__ void compat_kspace_kernel(CompatDev D)
{
    const double pi = 3.14159265358979323846;
    const long long n = (long long)D.nx * D.nyh;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t / D.nyh), j = (int)(t % D.nyh);
        const int II = (2 * i < D.nx) ? i : i - D.nx;
        const int JJ = (2 * j < D.nyh) ? j : j - D.ny;
        const double k1 = 2 * pi * II, k2 = 2 * pi * JJ;
        const double fact = __dadd_rn(__dmul_rn(k1, k1), __dmul_rn(k2, k2));
        cufftDoubleComplex o = D.fout[t];
        if (fabs(fact) < 1e-14) {
            o.x = 0.0;
            o.y = 0.0;
        } else {
            o.x = __ddiv_rn(o.x, -fact);
            o.y = __ddiv_rn(o.y, -fact);
        }
        D.fout[t] = o;
    }
}

__global__ void compat_unpack_phi_kernel(CompatDev D, double norm)
{
    const long long n = (long long)D.nx * D.ny;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t / D.ny), j = (int)(t % D.ny);
        D.phi[(i + 1) * D.Y + (j + 1)] = __dmul_rn(__dmul_rn(D.fin[t], norm), norm);
    }
}

__global__ void compat_efield_kernel(CompatDev D)
{
    const long long n = (long long)D.nx * D.ny;
    const int Y = D.Y;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = 1 + (int)(t / D.ny), j = 1 + (int)(t % D.ny);
        D.ex[i * Y + j] = __ddiv_rn(D.phi[i * Y + (j - 1)] - D.phi[i * Y + (j + 1)], 2 * D.dx);
        D.ey[i * Y + j] = __ddiv_rn(D.phi[(i - 1) * Y + j] - D.phi[(i + 1) * Y + j], 2 * D.dy);
    }
}

__global__ void compat_push_kernel(CompatDev D)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    const int Y = D.Y;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < D.np; k += stride) {
        double X = D.px[k], Yp = D.py[k];
        const double cx = D.cx[k], cy = D.cy[k];
        if (!(cx >= 0 && cx <= D.nx && cy >= 0 && cy <= D.ny)) continue;
        const double dx = D.dx, dy = D.dy, A = D.area;
        const double a1 = __ddiv_rn(__dmul_rn(X - cx * dx, Yp - cy * dy), A);
        const double a2 = __ddiv_rn(__dmul_rn((cx * dx + dx) - X, Yp - cy * dy), A);
        const double a3 = __ddiv_rn(__dmul_rn(X - cx * dx, (cy * dy + dy) - Yp), A);
        const double a4 = __ddiv_rn(__dmul_rn((cx * dx + dx) - X, (cy * dy + dy) - Yp), A);
        const int ix1 = (int)(cx + 1) % D.nx, iy1 = (int)(cy + 1) % D.ny;
        const size_t i1 = (size_t)(cx * Y + cy);
        const size_t i2 = (size_t)(ix1 * Y + cy);
        const size_t i3 = (size_t)(cx * Y + iy1);
        const size_t i4 = (size_t)(ix1 * Y + iy1);
        double fx = 0.0;
        fx = __dadd_rn(fx, __dmul_rn(a1, D.ex[i1]));
        fx = __dadd_rn(fx, __dmul_rn(a2, D.ex[i2]));
        fx = __dadd_rn(fx, __dmul_rn(a3, D.ex[i3]));
        fx = __dadd_rn(fx, __dmul_rn(a4, D.ex[i4]));
        fx = __dmul_rn(fx, D.qm);
        double fy = 0.0;
        fy = __dadd_rn(fy, __dmul_rn(a1, D.ey[i1]));
        fy = __dadd_rn(fy, __dmul_rn(a2, D.ey[i2]));
        fy = __dadd_rn(fy, __dmul_rn(a3, D.ey[i3]));
        fy = __dadd_rn(fy, __dmul_rn(a4, D.ey[i4]));
        fy = __dmul_rn(fy, D.qm);
        const double dt = D.dt;
        const double vxh = __dadd_rn(D.vx[k], __dmul_rn(__dmul_rn(0.5, dt), D.fox[k]));
        const double vyh = __dadd_rn(D.vy[k], __dmul_rn(__dmul_rn(0.5, dt), D.foy[k]));
        X = __dadd_rn(X, __dmul_rn(vxh, dt));
        Yp = __dadd_rn(Yp, __dmul_rn(vyh, dt));
        if (X > D.xDim)
            X -= D.xDim;
        else if (X < 0)
            X += D.xDim;
        if (Yp > D.yDim)
            Yp -= D.yDim;
        else if (Yp < 0)
            Yp += D.yDim;
        D.vx[k] = __dadd_rn(vxh, __dmul_rn(__dmul_rn(0.5, dt), fx));
        D.vy[k] = __dadd_rn(vyh, __dmul_rn(__dmul_rn(0.5, dt), fy));
        D.fox[k] = fx;
        D.foy[k] = fy;
        D.px[k] = X;
        D.py[k] = Yp;
        D.cx[k] = (int)__ddiv_rn(X, dx);
        D.cy[k] = (int)__ddiv_rn(Yp, dy);
    }
}

// Particle::Particle (particle.cc:21-29): cell from position, forces zero.
__global__ void compat_setup_kernel(CompatDev D)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < D.np; k += stride) {
        D.cx[k] = (int)__ddiv_rn(D.px[k], D.dx);
        D.cy[k] = (int)__ddiv_rn(D.py[k], D.dy);
        D.fox[k] = 0.0;
        D.foy[k] = 0.0;
    }
}

static long long count_steps(double dt, double tmax)
{
    long long n = 0;
    double t = 0.0;
    while (t < tmax) {
        t += dt;
        ++n;
    }
    return n;
}

static pic_status compat_validate(const pic_ref_params *p)
{
    // main.cc:82 argument checks, plus the limits of this implementation
    if (!p || p->npx < 1 || p->npy < 1 || p->xDim <= 0 || p->yDim <= 0 || p->nx < 2 ||
        p->ny < 2 || !(p->dt > 0.0) || p->tmax < 0.0 || !(p->mass != 0.0) ||
        (long long)p->nx * p->ny > (1ll << 26)) {
        set_error("pic_compat_run: invalid reference parameters");
        return PIC_ERR_INVALID_ARG;
    }
    return PIC_OK;
}

namespace {
struct CompatRun {
    CompatDev D{};
    cufftHandle fwd = 0, inv = 0;
    cudaStream_t st = nullptr;
    std::vector<void *> allocs;
    ~CompatRun()
    {
        if (fwd) cufftDestroy(fwd);
        if (inv) cufftDestroy(inv);
        for (void *a : allocs) cudaFree(a);
        if (st) cudaStreamDestroy(st);
    }
    template <class T> pic_status alloc(T **p, size_t n)
    {
        void *q = nullptr;
        PIC_CUDA(cudaMalloc(&q, n * sizeof(T)));
        allocs.push_back(q);
        *p = (T *)q;
        return PIC_OK;
    }
};
}  // namespace

static pic_status compat_core(const pic_ref_params *p, const double *x0, const double *y0,
                              const double *vx0, const double *vy0, long long nsteps, double *x,
                              double *y, double *vx, double *vy, double *rho, double *phi,
                              double *ex, double *ey)
{
    PIC_TRY(compat_validate(p));
    if (!x0 || !y0 || !vx0 || !vy0 || nsteps < 0) {
        set_error("pic_compat_run: null input array or negative step count");
        return PIC_ERR_INVALID_ARG;
    }
    CompatRun R;
    CompatDev &D = R.D;
    D.nx = p->nx;
    D.ny = p->ny;
    D.X = p->nx + 2;
    D.Y = p->ny + 2;
    D.nyh = p->ny / 2 + 1;
    D.xDim = p->xDim;
    D.yDim = p->yDim;
    D.dx = (double)p->xDim / p->nx;  // main.cc:75-77
    D.dy = (double)p->yDim / p->ny;
    D.area = D.dx * D.dy;
    D.q = p->charge;
    D.qm = p->charge / p->mass;
    D.dt = p->dt;
    D.np = (long long)p->npx * p->npy;
    const size_t np = (size_t)D.np, ng = (size_t)D.X * D.Y;
    PIC_CUDA(cudaStreamCreateWithFlags(&R.st, cudaStreamNonBlocking));
    double *pool = nullptr;
    PIC_TRY(R.alloc(&pool, 8 * np + 4 * ng + (size_t)p->nx * p->ny));
    D.px = pool;
    D.py = D.px + np;
    D.cx = D.py + np;
    D.cy = D.cx + np;
    D.vx = D.cy + np;
    D.vy = D.vx + np;
    D.fox = D.vy + np;
    D.foy = D.fox + np;
    D.rho = D.foy + np;
    D.phi = D.rho + ng;
    D.ex = D.phi + ng;
    D.ey = D.ex + ng;
    D.fin = D.ey + ng;
    PIC_TRY(R.alloc(&D.fout, (size_t)p->nx * D.nyh));
    PIC_CUDA(cudaMemsetAsync(D.phi, 0, sizeof(double) * 3 * ng, R.st));  // phi, Ex, Ey
    PIC_CUDA(cudaMemcpyAsync(D.px, x0, sizeof(double) * np, cudaMemcpyHostToDevice, R.st));
    PIC_CUDA(cudaMemcpyAsync(D.py, y0, sizeof(double) * np, cudaMemcpyHostToDevice, R.st));
    PIC_CUDA(cudaMemcpyAsync(D.vx, vx0, sizeof(double) * np, cudaMemcpyHostToDevice, R.st));
    PIC_CUDA(cudaMemcpyAsync(D.vy, vy0, sizeof(double) * np, cudaMemcpyHostToDevice, R.st));
    PIC_CUFFT(cufftPlan2d(&R.fwd, p->nx, p->ny, CUFFT_D2Z));
    PIC_CUFFT(cufftPlan2d(&R.inv, p->nx, p->ny, CUFFT_Z2D));
    PIC_CUFFT(cufftSetStream(R.fwd, R.st));
    PIC_CUFFT(cufftSetStream(R.inv, R.st));
    const int gp = grid_for(D.np, 256), gg = grid_for((long long)p->nx * p->ny, 256);
    compat_setup_kernel<<<gp, 256, 0, R.st>>>(D);
    PIC_CUDA(cudaGetLastError());
    const double norm = 1.0 / (p->nx * p->ny);
    for (long long s = 0; s < nsteps; ++s) {
        PIC_CUDA(cudaMemsetAsync(D.rho, 0, sizeof(double) * ng, R.st));
        compat_deposit_kernel<<<gp, 256, 0, R.st>>>(D);
        compat_ghost_kernel<<<1, 1024, 0, R.st>>>(D.rho, D.nx, D.ny, 0);
        compat_pack_kernel<<<gg, 256, 0, R.st>>>(D);
        PIC_CUFFT(cufftExecD2Z(R.fwd, D.fin, D.fout));
        compat_kspace_kernel<<<gg, 256, 0, R.st>>>(D);
        PIC_CUFFT(cufftExecZ2D(R.inv, D.fout, D.fin));
        compat_unpack_phi_kernel<<<gg, 256, 0, R.st>>>(D, norm);
        compat_ghost_kernel<<<1, 1024, 0, R.st>>>(D.phi, D.nx, D.ny, 1);
        compat_efield_kernel<<<gg, 256, 0, R.st>>>(D);
        compat_push_kernel<<<gp, 256, 0, R.st>>>(D);
        PIC_CUDA(cudaGetLastError());
    }
    if (x) PIC_CUDA(cudaMemcpyAsync(x, D.px, sizeof(double) * np, cudaMemcpyDeviceToHost, R.st));
    if (y) PIC_CUDA(cudaMemcpyAsync(y, D.py, sizeof(double) * np, cudaMemcpyDeviceToHost, R.st));
    if (vx) PIC_CUDA(cudaMemcpyAsync(vx, D.vx, sizeof(double) * np, cudaMemcpyDeviceToHost, R.st));
    if (vy) PIC_CUDA(cudaMemcpyAsync(vy, D.vy, sizeof(double) * np, cudaMemcpyDeviceToHost, R.st));
    if (rho) PIC_CUDA(cudaMemcpyAsync(rho, D.rho, sizeof(double) * ng, cudaMemcpyDeviceToHost, R.st));
    if (phi) PIC_CUDA(cudaMemcpyAsync(phi, D.phi, sizeof(double) * ng, cudaMemcpyDeviceToHost, R.st));
    if (ex) PIC_CUDA(cudaMemcpyAsync(ex, D.ex, sizeof(double) * ng, cudaMemcpyDeviceToHost, R.st));
    if (ey) PIC_CUDA(cudaMemcpyAsync(ey, D.ey, sizeof(double) * ng, cudaMemcpyDeviceToHost, R.st));
    PIC_CUDA(cudaStreamSynchronize(R.st));
    return PIC_OK;
}

}  // namespace pic

extern "C" pic_status pic_compat_run_steps(const pic_ref_params *p, const double *x0,
                                           const double *y0, const double *vx0,
                                           const double *vy0, long long nsteps, double *x,
                                           double *y, double *vx, double *vy, double *rho,
                                           double *phi, double *ex, double *ey)
{
    return pic::compat_core(p, x0, y0, vx0, vy0, nsteps, x, y, vx, vy, rho, phi, ex, ey);
}

extern "C" pic_status pic_compat_run(const pic_ref_params *p, const double *posX,
                                     const double *posY, const double *velX, const double *velY,
                                     double *xOut, double *yOut, double *seconds)
{
    PIC_TRY(pic::compat_validate(p));
    const auto t0 = std::chrono::steady_clock::now();
    const long long nsteps = pic::count_steps(p->dt, p->tmax);
    pic_status s = pic::compat_core(p, posX, posY, velX, velY, nsteps, xOut, yOut, nullptr,
                                    nullptr, nullptr, nullptr, nullptr, nullptr);
    const auto t1 = std::chrono::steady_clock::now();
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    return s;
}
