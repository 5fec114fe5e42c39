// pic_adjoint.cu -- discrete adjoint of the collisionless GPU step.
//
// Forward map (one charged species): v(-1/2) = v0 + c0 (q/m) F(x0) with
// c0 = -dt/2, then for n = 0..N-1: v(n+1/2) = v(n-1/2) + dt (q/m) F(x_n),
// x_(n+1) = x_n + dt v(n+1/2), where F(x)_i = sum_k w_k(x_i) E_k and
// E = S rho(x) (CIC deposit, spectral Poisson, E = -i k phi).  Objective
// J = 1/2 eps0 dA sum_k |E_k(x_N)|^2.
//
// Backward (a_x = dJ/dx, a_v = dJ/dv): a_x = grad J(x_N); for n = N-1..0:
// a_v += dt a_x (drift), then the kick transpose with mu = dt (q/m) a_v:
//   local     a_x,i += sum_k grad w_k(x_i) (E_k . mu_i)
//   scatter   g_k = sum_i w_k(x_i) mu_i                (adjoint of the gather)
//   solve     psi = S^T g, psi^ = i k.g^ / (eps0 k^2)  (S^T of the field solve)
//   gather    a_x,j += (q / dA) sum_m psi_m grad w_m(x_j) (adjoint of the deposit)
// and finally the priming kick with coefficient c0.  grad J(x_N) is the
// solve + gather with g = eps0 dA E(x_N).  The deposit's 2^-16 weight
// quantisation is not differentiated (continuous CIC weights are used).
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <vector>

#include "pic_adjoint_dev.cuh"

namespace pic {

struct AdjArgs {
    const int32_t *cell;
    const float *ox, *oy;      // positions of the step (ring slot)
    const float *ex, *ey;      // field of the step
    float *ax, *ay, *avx, *avy;  // adjoint state (storage order)
    float *gx, *gy;            // scatter target planes
    const float *psi;          // S^T g
    long long n;
    int nx, ny;
    float inv_dx, inv_dy;
    float C;                   // kick coefficient times q/m
    float drift_dt;            // dt for the drift adjoint (0: none)
    float q_over_dA;
};

// drift adjoint, kick local term and scatter of mu
__global__ void __launch_bounds__(256) adj_kick_scatter_kernel(AdjArgs A)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += stride) {
        const Cic w = cic_of(A.cell[i], A.ox[i], A.oy[i], A.nx, A.ny);
        if (!w.ok) continue;
        float ax = A.ax[i], ay = A.ay[i];
        float avx = A.avx[i], avy = A.avy[i];
        avx = fmaf(A.drift_dt, ax, avx);
        avy = fmaf(A.drift_dt, ay, avy);
        const float mx = A.C * avx, my = A.C * avy;
        const float gx = 1.f - w.fx, gy = 1.f - w.fy;
        const float w00 = gx * gy, w10 = w.fx * gy, w01 = gx * w.fy, w11 = w.fx * w.fy;
        atomicAdd(A.gx + w.i00, w00 * mx);
        atomicAdd(A.gy + w.i00, w00 * my);
        atomicAdd(A.gx + w.i10, w10 * mx);
        atomicAdd(A.gy + w.i10, w10 * my);
        atomicAdd(A.gx + w.i01, w01 * mx);
        atomicAdd(A.gy + w.i01, w01 * my);
        atomicAdd(A.gx + w.i11, w11 * mx);
        atomicAdd(A.gy + w.i11, w11 * my);
        const float s00 = A.ex[w.i00] * mx + A.ey[w.i00] * my;
        const float s10 = A.ex[w.i10] * mx + A.ey[w.i10] * my;
        const float s01 = A.ex[w.i01] * mx + A.ey[w.i01] * my;
        const float s11 = A.ex[w.i11] * mx + A.ey[w.i11] * my;
        const float2 l = grad_dot(w, s00, s10, s01, s11, A.inv_dx, A.inv_dy);
        A.ax[i] = ax + l.x;
        A.ay[i] = ay + l.y;
        A.avx[i] = avx;
        A.avy[i] = avy;
    }
}

// adjoint of the deposit: a_x += (q/dA) sum_m psi_m grad w_m
__global__ void __launch_bounds__(256) adj_gather_kernel(AdjArgs A)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += stride) {
        const Cic w = cic_of(A.cell[i], A.ox[i], A.oy[i], A.nx, A.ny);
        if (!w.ok) continue;
        const float2 g = grad_dot(w, A.psi[w.i00], A.psi[w.i10], A.psi[w.i01], A.psi[w.i11],
                                  A.inv_dx, A.inv_dy);
        A.ax[i] = fmaf(A.q_over_dA, g.x, A.ax[i]);
        A.ay[i] = fmaf(A.q_over_dA, g.y, A.ay[i]);
    }
}

// psi^ = i (kx g^x + ky g^y) / (eps0 N k^2), Nyquist derivative zeroed as in
// the forward solve, zero mode removed
__global__ void __launch_bounds__(256) adj_kspace_kernel(const float2 *gh, float2 *ph, int nx, int ny,
                                                         int nh, float kx1, float ky1, float inv_eps0_n)
{
    const long long total = (long long)ny * nh;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int my = (int)idx / nh, mx = (int)idx - my * nh;  // ny nh < 2^31
        ph[idx] = adj_mode(gh[idx], gh[total + idx], mx, my, nx, ny, kx1, ky1, inv_eps0_n, idx == 0);
    }
}

__global__ void scale_planes_kernel(const float *ex, const float *ey, float s, float *gx, float *gy,
                                    long long n)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        gx[i] = s * ex[i];
        gy[i] = s * ey[i];
    }
}

// storage order -> id order (double) for two arrays
__global__ void to_id_order_kernel(const float *a, const float *b, const uint32_t *pid, long long n,
                                   double *oa, double *ob)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const uint32_t p = pid[i];
        if ((long long)p >= n) continue;
        oa[p] = a[i];
        ob[p] = b[i];
    }
}

// ---------------------------------------------------------------- driver
namespace {

struct AdjWork {
    pic_handle *h;
    std::vector<void *> allocs;
    cufftHandle r2c2 = 0;
    ~AdjWork()
    {
        for (void *p : allocs) cudaFree(p);
        if (r2c2) cufftDestroy(r2c2);
    }
    template <class T> pic_status alloc(T **p, size_t n)
    {
        void *q = nullptr;
        PIC_CUDA(cudaMalloc(&q, (n ? n : 1) * sizeof(T)));
        allocs.push_back(q);
        *p = (T *)q;
        return PIC_OK;
    }
};

struct Snap {  // particle state of species 0 (storage order)
    int32_t *cell;
    float *ox, *oy, *vx, *vy;
};

pic_status snap_alloc(AdjWork &W, Snap &S, size_t n)
{
    PIC_TRY(W.alloc(&S.cell, n));
    PIC_TRY(W.alloc(&S.ox, n));
    PIC_TRY(W.alloc(&S.oy, n));
    PIC_TRY(W.alloc(&S.vx, n));
    PIC_TRY(W.alloc(&S.vy, n));
    return PIC_OK;
}

pic_status snap_copy(pic_handle *h, Snap &S, bool save, size_t n)
{
    SpeciesBuf &B = h->sp[0];
    const cudaMemcpyKind k = cudaMemcpyDeviceToDevice;
    cudaStream_t st = h->stream;
    if (save) {
        PIC_CUDA(cudaMemcpyAsync(S.cell, B.cell[0], n * 4, k, st));
        PIC_CUDA(cudaMemcpyAsync(S.ox, B.ox[0], n * 4, k, st));
        PIC_CUDA(cudaMemcpyAsync(S.oy, B.oy[0], n * 4, k, st));
        PIC_CUDA(cudaMemcpyAsync(S.vx, B.vx[0], n * 4, k, st));
        PIC_CUDA(cudaMemcpyAsync(S.vy, B.vy[0], n * 4, k, st));
    } else {
        PIC_CUDA(cudaMemcpyAsync(B.cell[0], S.cell, n * 4, k, st));
        PIC_CUDA(cudaMemcpyAsync(B.ox[0], S.ox, n * 4, k, st));
        PIC_CUDA(cudaMemcpyAsync(B.oy[0], S.oy, n * 4, k, st));
        PIC_CUDA(cudaMemcpyAsync(B.vx[0], S.vx, n * 4, k, st));
        PIC_CUDA(cudaMemcpyAsync(B.vy[0], S.vy, n * 4, k, st));
    }
    return PIC_OK;
}

}  // namespace

pic_status adjoint_run(pic_handle *h, const pic_init_spec *spec, long long nsteps, int every,
                       double *gx0, double *gy0, double *gvx0, double *gvy0,
                       pic_adjoint_result *out)
{
    const pic_config &c = h->cfg;
    if (c.nspecies != 1 || c.species[0].q == 0.0 || h->mcc.on || h->dsmc.on || nsteps < 1 ||
        every < 1) {
        set_error("pic_adjoint_run: needs one charged species, no collisions, nsteps >= 1, every >= 1");
        return PIC_ERR_INVALID_ARG;
    }
    if (spec) PIC_TRY(pic_init_particles(h, 0, spec));
    if (!h->fields_valid) {
        set_error("pic_adjoint_run: no particles loaded");
        return PIC_ERR_STATE;
    }
    const Geometry &g = h->g;
    const size_t np = (size_t)h->sp[0].cap;
    const long long n = h->sp[0].n;
    const size_t ncell = (size_t)g.nx * g.ny, nk = (size_t)g.ny * g.nh;
    const double qm = c.species[0].q / c.species[0].m, dt = c.dt;
    const int K = (int)std::min<long long>(every, nsteps);
    const int nseg = (int)((nsteps + K - 1) / K);
    AdjWork W;
    W.h = h;
    std::vector<Snap> ck(nseg);
    for (auto &S : ck) PIC_TRY(snap_alloc(W, S, np));
    Snap fin;
    PIC_TRY(snap_alloc(W, fin, np));
    // ring of one segment: positions and fields per step
    int32_t *rc = nullptr;
    float *rox = nullptr, *roy = nullptr, *re = nullptr;
    PIC_TRY(W.alloc(&rc, np * K));
    PIC_TRY(W.alloc(&rox, np * K));
    PIC_TRY(W.alloc(&roy, np * K));
    PIC_TRY(W.alloc(&re, 2 * ncell * K));
    float *ax = nullptr, *ay = nullptr, *avx = nullptr, *avy = nullptr, *gpl = nullptr, *psi = nullptr;
    float2 *gh = nullptr, *ph = nullptr;
    PIC_TRY(W.alloc(&ax, np));
    PIC_TRY(W.alloc(&ay, np));
    PIC_TRY(W.alloc(&avx, np));
    PIC_TRY(W.alloc(&avy, np));
    PIC_TRY(W.alloc(&gpl, 2 * ncell));
    PIC_TRY(W.alloc(&psi, ncell));
    PIC_TRY(W.alloc(&gh, 2 * nk));
    PIC_TRY(W.alloc(&ph, nk));
    int dims[2] = {g.ny, g.nx};
    PIC_CUFFT(cufftPlanMany(&W.r2c2, 2, dims, nullptr, 1, (int)ncell, nullptr, 1, (int)nk,
                            CUFFT_R2C, 2));
    PIC_CUFFT(cufftSetStream(W.r2c2, h->stream));
    cudaStream_t st = h->stream;
    SpeciesBuf &B = h->sp[0];

    // ---- forward: prime, checkpoints every K steps, no re-sorting
    PIC_TRY(pic_prime_leapfrog(h));
    for (int m = 0; m < nseg; ++m) {
        PIC_TRY(snap_copy(h, ck[m], true, np));
        const long long s0 = (long long)m * K, s1 = std::min<long long>(nsteps, s0 + K);
        for (long long s = s0; s < s1; ++s) {
            PIC_CUDA(cudaMemsetAsync(h->rho_fix, 0, ncell * 8, st));
            PIC_TRY(record_push_all(h, 0, true));
            PIC_TRY(record_poisson(h));
        }
    }
    PIC_TRY(snap_copy(h, fin, true, np));
    PIC_CUDA(cudaStreamSynchronize(st));
    h->steps_host += nsteps;
    h->since_sort += (int)std::min<long long>(nsteps, 1 << 30);
    pic_diag d;
    PIC_TRY(pic_diagnostics(h, &d));
    const double J = d.field_energy;
    // the recompute passes below advance the step counter and the history;
    // the device state of step nsteps is put back at the end
    DevState saved;
    PIC_CUDA(cudaMemcpy(&saved, h->dev, sizeof(DevState), cudaMemcpyDeviceToHost));
    const size_t hist_bytes = 6 * (size_t)h->hist_cap * sizeof(double);
    double *hist_saved;
    PIC_TRY(W.alloc(&hist_saved, 6 * (size_t)h->hist_cap));
    PIC_CUDA(cudaMemcpyAsync(hist_saved, h->hist, hist_bytes, cudaMemcpyDeviceToDevice, st));

    AdjArgs A;
    A.n = n;
    A.nx = g.nx;
    A.ny = g.ny;
    A.inv_dx = (float)(1.0 / g.dx);
    A.inv_dy = (float)(1.0 / g.dy);
    A.q_over_dA = (float)(c.species[0].q / (g.dx * g.dy));
    A.ax = ax;
    A.ay = ay;
    A.avx = avx;
    A.avy = avy;
    A.gx = gpl;
    A.gy = gpl + ncell;
    A.psi = psi;
    const int gp = grid_for(n, 256), gg = grid_for((long long)nk, 256);
    const float kx1 = (float)(2.0 * 3.14159265358979323846 / g.Lx);
    const float ky1 = (float)(2.0 * 3.14159265358979323846 / g.Ly);
    const float inv_eps0_n = (float)(1.0 / (c.eps0 * (double)ncell));
    // psi = S^T g and a_x += (q/dA) sum psi grad w at the positions in A
    auto solve_and_gather = [&]() -> pic_status {
        if (h->spectral) {
            PIC_TRY(launch_spectral_adjoint(h, gpl, gpl + ncell, gh, ph, psi));
        } else {
            PIC_CUFFT(cufftExecR2C(W.r2c2, gpl, (cufftComplex *)gh));
            adj_kspace_kernel<<<gg, 256, 0, st>>>(gh, ph, g.nx, g.ny, g.nh, kx1, ky1, inv_eps0_n);
            PIC_CUDA(cudaGetLastError());
            PIC_CUFFT(cufftExecC2R(h->plan_c2r1, (cufftComplex *)ph, psi));
        }
        adj_gather_kernel<<<gp, 256, 0, st>>>(A);
        PIC_CUDA(cudaGetLastError());
        return PIC_OK;
    };
    auto kick = [&](float C, float drift) -> pic_status {
        A.C = (float)(C * qm);
        A.drift_dt = drift;
        PIC_CUDA(cudaMemsetAsync(gpl, 0, 2 * ncell * 4, st));
        adj_kick_scatter_kernel<<<gp, 256, 0, st>>>(A);
        PIC_CUDA(cudaGetLastError());
        return solve_and_gather();
    };

    // ---- terminal condition: a_x = grad J(x_N)
    PIC_CUDA(cudaMemsetAsync(ax, 0, np * 4, st));
    PIC_CUDA(cudaMemsetAsync(ay, 0, np * 4, st));
    PIC_CUDA(cudaMemsetAsync(avx, 0, np * 4, st));
    PIC_CUDA(cudaMemsetAsync(avy, 0, np * 4, st));
    scale_planes_kernel<<<grid_for((long long)ncell, 256), 256, 0, st>>>(
        h->e, h->e + ncell, (float)(c.eps0 * g.dx * g.dy), gpl, gpl + ncell, (long long)ncell);
    PIC_CUDA(cudaGetLastError());
    A.cell = B.cell[0];
    A.ox = B.ox[0];
    A.oy = B.oy[0];
    PIC_TRY(solve_and_gather());

    // ---- backward over the segments, recomputing each into the ring
    for (int m = nseg - 1; m >= 0; --m) {
        const long long s0 = (long long)m * K, s1 = std::min<long long>(nsteps, s0 + K);
        PIC_TRY(snap_copy(h, ck[m], false, np));
        PIC_TRY(deposit_now(h));
        PIC_TRY(record_poisson(h));
        for (long long s = s0; s < s1; ++s) {
            const size_t r = (size_t)(s - s0);
            PIC_CUDA(cudaMemcpyAsync(rc + r * np, B.cell[0], np * 4, cudaMemcpyDeviceToDevice, st));
            PIC_CUDA(cudaMemcpyAsync(rox + r * np, B.ox[0], np * 4, cudaMemcpyDeviceToDevice, st));
            PIC_CUDA(cudaMemcpyAsync(roy + r * np, B.oy[0], np * 4, cudaMemcpyDeviceToDevice, st));
            PIC_CUDA(cudaMemcpyAsync(re + r * 2 * ncell, h->e, 2 * ncell * 4, cudaMemcpyDeviceToDevice, st));
            if (s + 1 < s1) {
                PIC_CUDA(cudaMemsetAsync(h->rho_fix, 0, ncell * 8, st));
                PIC_TRY(record_push_all(h, 0, true));
                PIC_TRY(record_poisson(h));
            }
        }
        for (long long s = s1 - 1; s >= s0; --s) {
            const size_t r = (size_t)(s - s0);
            A.cell = rc + r * np;
            A.ox = rox + r * np;
            A.oy = roy + r * np;
            A.ex = re + r * 2 * ncell;
            A.ey = A.ex + ncell;
            PIC_TRY(kick((float)dt, (float)dt));
        }
    }
    // ---- the priming kick v(-1/2) = v0 - (q/m) F(x0) dt/2 (ring slot 0 of segment 0)
    A.cell = rc;
    A.ox = rox;
    A.oy = roy;
    A.ex = re;
    A.ey = re + ncell;
    PIC_TRY(kick((float)(-0.5 * dt), 0.f));

    // ---- outputs in id order
    double *buf;
    PIC_TRY(W.alloc(&buf, 4 * (size_t)n));
    to_id_order_kernel<<<gp, 256, 0, st>>>(ax, ay, B.pid[0], n, buf, buf + n);
    to_id_order_kernel<<<gp, 256, 0, st>>>(avx, avy, B.pid[0], n, buf + 2 * n, buf + 3 * n);
    PIC_CUDA(cudaGetLastError());
    std::vector<double> hb(4 * (size_t)n);
    PIC_CUDA(cudaMemcpyAsync(hb.data(), buf, hb.size() * 8, cudaMemcpyDeviceToHost, st));
    PIC_CUDA(cudaStreamSynchronize(st));
    if (gx0) std::copy(hb.begin(), hb.begin() + n, gx0);
    if (gy0) std::copy(hb.begin() + n, hb.begin() + 2 * n, gy0);
    if (gvx0) std::copy(hb.begin() + 2 * n, hb.begin() + 3 * n, gvx0);
    if (gvy0) std::copy(hb.begin() + 3 * n, hb.begin() + 4 * n, gvy0);
    if (out) {
        out->J = J;
        out->dJ_dbeam_v = 0.0;
        out->dJ_damp = 0.0;
        if (spec) {
            double sb = 0.0;
            for (long long i = 0; i < n; ++i) sb += (i & 1) ? -hb[2 * n + i] : hb[2 * n + i];
            out->dJ_dbeam_v = sb;  // vx carries +-beam_v by id parity
            std::vector<double> dA(2 * (size_t)n);
            double *dAd;
            PIC_TRY(W.alloc(&dAd, 2 * (size_t)n));
            int lx = 0, ly = 0;
            if (spec->layout == PIC_LOAD_LATTICE) PIC_TRY(lattice_dims(h, n, &lx, &ly));
            PIC_TRY(launch_init_dA(h, spec, lx, ly, dAd, dAd + n));
            PIC_CUDA(cudaMemcpyAsync(dA.data(), dAd, dA.size() * 8, cudaMemcpyDeviceToHost, st));
            PIC_CUDA(cudaStreamSynchronize(st));
            double sa = 0.0;
            for (long long i = 0; i < n; ++i) sa += hb[i] * dA[i] + hb[n + i] * dA[n + i];
            out->dJ_damp = sa;
        }
    }
    // ---- leave the handle at step nsteps
    PIC_TRY(snap_copy(h, fin, false, np));
    PIC_TRY(deposit_now(h));
    PIC_TRY(record_poisson(h));
    PIC_CUDA(cudaMemcpyAsync(h->dev, &saved, sizeof(DevState), cudaMemcpyHostToDevice, st));
    PIC_CUDA(cudaMemcpyAsync(h->hist, hist_saved, hist_bytes, cudaMemcpyDeviceToDevice, st));
    PIC_CUDA(cudaStreamSynchronize(st));
    return PIC_OK;
}

}  // namespace pic

extern "C" pic_status pic_adjoint_run(pic_handle *h, const pic_init_spec *spec, long long nsteps,
                                      int every, double *dJ_dx0, double *dJ_dy0, double *dJ_dvx0,
                                      double *dJ_dvy0, pic_adjoint_result *out)
{
    if (!h) {
        pic::set_error("pic_adjoint_run: null handle");
        return PIC_ERR_INVALID_ARG;
    }
    PIC_CUDA(cudaSetDevice(h->device));
    return pic::adjoint_run(h, spec, nsteps, every, dJ_dx0, dJ_dy0, dJ_dvx0, dJ_dvy0, out);
}
