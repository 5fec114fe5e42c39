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
// group's count and sums of fx, fy and fx*fy) before one set of atomics.
// Because the weights are linear in those moments, the shared-memory window
// keeps per cell five 32-bit sums (count, sum fx, sum fy, and the low 16 and
// the high bits of sum fx*fy): five native 32-bit atomics per group instead
// of two per node (eight), on the shared-memory pipe that limits this
// kernel.  At the end of the block each window node forms its weight from
// the moments of its four cells and the charge sign is applied once per
// node in a 64-bit atomic to the global density.  Per block and cell the
// sums stay at most 2^31 for chunks of at most 32768 particles.
#include <cuda_runtime.h>

#include "pic_push_dev.cuh"

namespace pic {

// Direct-load variant: each thread loads its quads with 128-bit loads.
// !MOVE: the deposit of the particles where they are (after an import, a
// sort or a state load), through the same shared-memory windows.
template <bool GATHER, bool DEPOSIT, bool AGG, bool MOVE = true>
__global__ void __launch_bounds__(256, 4) push_kernel(PushArgs A)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const long long n = *A.d_n;
    const long long base = (long long)blockIdx.x * A.chunk;
    if (base >= n) return;  // block-uniform
    const long long n4 = (n + 3) & ~3ll;
    push_block<GATHER, DEPOSIT, AGG, MOVE>(A, A.geo, smem, base, min(base + (long long)A.chunk, n4),
                                           A.anchor[blockIdx.x]);
}

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
    return window_bytes(g.wcx, g.wcy) + 32;
}

// set on every launch: the attribute belongs to the current device, and a
// process may drive several
pic_status allow_dynamic_smem(const void *kernel, size_t bytes)
{
    if (bytes > 48 * 1024)
        PIC_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return PIC_OK;
}

static PushArgs push_args(pic_handle *h, int s, int src, float dt_scale)
{
    SpeciesBuf &B = h->sp[s];
    const pic_species_desc &D = h->cfg.species[s];
    const Geometry &g = h->g;
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
    A.geo.ex = h->e;
    A.geo.ey = h->e + (size_t)g.nx * g.ny;
    A.geo.rho = h->rho_fix;
    A.geo.dev = h->dev;
    A.geo.nx = g.nx;
    A.geo.ny = g.ny;
    A.geo.tw = g.tw;
    A.geo.th = g.th;
    A.geo.hx = g.halo;
    A.geo.hy = g.halo;
    A.geo.wcx = g.wcx;
    A.geo.wcy = g.wcy;
    A.chunk = g.chunk;
    const double dt = h->cfg.dt * dt_scale;
    const bool move = dt_scale > 0.0f;
    A.geo.qm_dt = (float)(D.q / D.m * dt);
    A.geo.dtdx = move ? (float)(h->cfg.dt / g.dx) : 0.f;
    A.geo.dtdy = move ? (float)(h->cfg.dt / g.dy) : 0.f;
    A.geo.qmul = (unsigned long long)(long long)D.q_int;
    A.geo.ke_scale = move ? 0.25 * D.m : 0.0;
    A.geo.p_scale = 0.5 * D.m;
    // the DSMC species, sorted every step, keeps its cell counts current here
    // so that its sort can skip the histogram
    A.geo.recount = (h->dsmc.on && s == h->dsmc.s) ? h->dsmc.count : nullptr;
    A.geo.ntx = g.ntx;
    return A;
}

pic_status launch_push(pic_handle *h, int s, int src, bool deposit, float dt_scale)
{
    SpeciesBuf &B = h->sp[s];
    const pic_species_desc &D = h->cfg.species[s];
    const Geometry &g = h->g;
    if (B.nchunks == 0) return PIC_OK;
    PushArgs A = push_args(h, s, src, dt_scale);
    const bool charged = D.q != 0.0;
    const bool dep = deposit && D.q_int != 0;
    dim3 grid((unsigned)B.nchunks), block(256);
    if (h->cfg.push_variant == 3) {
        // warp-summed deposit groups: measured 5% slower at 2048^2 x 32 ppc
        // (1.144 vs 1.085 ms), so opt-in
        const size_t sm = push_smem(g);
        if (charged && dep) {
            PIC_TRY(allow_dynamic_smem((const void *)push_kernel<true, true, true>, sm));
            push_kernel<true, true, true><<<grid, block, sm, h->stream>>>(A);
        } else if (charged) {
            PIC_TRY(allow_dynamic_smem((const void *)push_kernel<true, false, false>, sm));
            push_kernel<true, false, false><<<grid, block, sm, h->stream>>>(A);
        } else if (dep) {
            PIC_TRY(allow_dynamic_smem((const void *)push_kernel<false, true, true>, sm));
            push_kernel<false, true, true><<<grid, block, sm, h->stream>>>(A);
        } else {
            PIC_TRY(allow_dynamic_smem((const void *)push_kernel<false, false, false>, sm));
            push_kernel<false, false, false><<<grid, block, sm, h->stream>>>(A);
        }
    } else {
        const size_t sm = push_smem(g);
        if (charged && dep) {
            PIC_TRY(allow_dynamic_smem((const void *)push_kernel<true, true, false>, sm));
            push_kernel<true, true, false><<<grid, block, sm, h->stream>>>(A);
        } else if (charged) {
            PIC_TRY(allow_dynamic_smem((const void *)push_kernel<true, false, false>, sm));
            push_kernel<true, false, false><<<grid, block, sm, h->stream>>>(A);
        } else if (dep) {
            PIC_TRY(allow_dynamic_smem((const void *)push_kernel<false, true, false>, sm));
            push_kernel<false, true, false><<<grid, block, sm, h->stream>>>(A);
        } else {
            PIC_TRY(allow_dynamic_smem((const void *)push_kernel<false, false, false>, sm));
            push_kernel<false, false, false><<<grid, block, sm, h->stream>>>(A);
        }
    }
    PIC_CUDA(cudaGetLastError());
    return PIC_OK;
}

// Deposit of buffer 0 where it stands: shared-memory windows at the chunk
// anchors (particles outside a stale window go straight to the grid), the
// particle arrays only read.
pic_status launch_deposit(pic_handle *h, int s)
{
    SpeciesBuf &B = h->sp[s];
    const pic_species_desc &D = h->cfg.species[s];
    if (D.q_int == 0 || B.cap == 0 || B.nchunks == 0) return PIC_OK;
    const PushArgs A = push_args(h, s, 0, 0.f);
    PIC_TRY(allow_dynamic_smem((const void *)push_kernel<false, true, false, false>, push_smem(h->g)));
    push_kernel<false, true, false, false><<<(unsigned)B.nchunks, 256, push_smem(h->g), h->stream>>>(A);
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
