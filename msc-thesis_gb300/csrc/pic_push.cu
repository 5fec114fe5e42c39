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

// ------------------------------------------------------------------------
// Bulk-copy variant.  Thread 0 streams the chunk into shared memory through
// a ring of PIPE_STAGES stages of STAGE_PARTICLES particles (five
// cp.async.bulk copies per stage, completion counted in bytes on the
// stage's mbarrier); all threads consume the stage from shared memory and
// store results straight to global memory.  Memory parallelism comes from
// the stages in flight, not from the number of resident warps.  Every wait
// is bounded: on expiry the block raises PIC_DEVERR_TIMEOUT, waits (bounded)
// for the copies it issued and leaves.
// ------------------------------------------------------------------------
constexpr int STAGE_PARTICLES = 1024;
constexpr int PIPE_STAGES = 3;
constexpr unsigned WAIT_LIMIT = 1u << 20;

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity)
{
    for (unsigned it = 0; it < WAIT_LIMIT; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes,
                                         unsigned long long *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// shared memory of the bulk-copy variant: the window, the diagnostics, the
// stage barriers, then the stage ring (16-byte aligned)
__host__ __device__ __forceinline__ size_t tma_ring_offset(size_t wbytes)
{
    return ((wbytes + 32 + PIPE_STAGES * 8) + 127) & ~(size_t)127;
}

template <bool GATHER, bool DEPOSIT>
__global__ void __launch_bounds__(256) push_kernel_bulk(PushArgs A)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const long long n = *A.d_n;
    const long long base = (long long)blockIdx.x * A.chunk;
    if (base >= n) return;  // block-uniform
    const long long n4 = (n + 3) & ~3ll;
    const long long end = min(base + (long long)A.chunk, n4);
    const Window W = setup_window(A.geo, smem, A.anchor[blockIdx.x]);
    const size_t wb = window_bytes(A.geo.wcx, A.geo.wcy);
    double *sAcc = reinterpret_cast<double *>(smem + wb);
    unsigned long long *bar = reinterpret_cast<unsigned long long *>(smem + wb + 32);
    unsigned char *ring = smem + tma_ring_offset(wb);
    const int nstages = (int)((end - base + STAGE_PARTICLES - 1) / STAGE_PARTICLES);
    const size_t field_bytes = (size_t)STAGE_PARTICLES * 4;
    const size_t stage_bytes = 5 * field_bytes;

    auto issue = [&](int k) {  // thread 0 only
        const long long s0 = base + (long long)k * STAGE_PARTICLES;
        const unsigned cnt = (unsigned)min((long long)STAGE_PARTICLES, end - s0);  // multiple of 4
        const unsigned bytes = cnt * 4u;
        unsigned char *dst = ring + (size_t)(k % PIPE_STAGES) * stage_bytes;
        unsigned long long *b = bar + (k % PIPE_STAGES);
        mbar_expect_tx(b, 5u * bytes);
        bulk_g2s(dst + 0 * field_bytes, A.cin + s0, bytes, b);
        bulk_g2s(dst + 1 * field_bytes, A.oxin + s0, bytes, b);
        bulk_g2s(dst + 2 * field_bytes, A.oyin + s0, bytes, b);
        bulk_g2s(dst + 3 * field_bytes, A.vxin + s0, bytes, b);
        bulk_g2s(dst + 4 * field_bytes, A.vyin + s0, bytes, b);
    };

    if (threadIdx.x == 0) {
        for (int k = 0; k < PIPE_STAGES; ++k) mbar_init(bar + k, 1u);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    load_window<GATHER, DEPOSIT>(A.geo, W);
    if (threadIdx.x < 3) sAcc[threadIdx.x] = 0.0;
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < PIPE_STAGES && k < nstages; ++k) issue(k);

    float ke = 0.f, px = 0.f, py = 0.f;
    bool bad = false;
    int k = 0;
    bool timed_out = false;
    for (; k < nstages; ++k) {
        const bool ok = mbar_wait_bounded(bar + (k % PIPE_STAGES), (unsigned)((k / PIPE_STAGES) & 1));
        if (__syncthreads_or(ok ? 0 : 1)) {  // block-uniform decision
            timed_out = true;
            break;
        }
        const unsigned char *st = ring + (size_t)(k % PIPE_STAGES) * stage_bytes;
        const long long s0 = base + (long long)k * STAGE_PARTICLES;
        const int cnt = (int)min((long long)STAGE_PARTICLES, end - s0);
        for (int l = 4 * threadIdx.x; l < cnt; l += 4 * blockDim.x) {
            const int4 c4 = *reinterpret_cast<const int4 *>(st + 0 * field_bytes + 4 * l);
            const float4 a4 = *reinterpret_cast<const float4 *>(st + 1 * field_bytes + 4 * l);
            const float4 b4 = *reinterpret_cast<const float4 *>(st + 2 * field_bytes + 4 * l);
            const float4 u4 = *reinterpret_cast<const float4 *>(st + 3 * field_bytes + 4 * l);
            const float4 v4 = *reinterpret_cast<const float4 *>(st + 4 * field_bytes + 4 * l);
            int cc[4] = {c4.x, c4.y, c4.z, c4.w};
            float xo[4] = {a4.x, a4.y, a4.z, a4.w}, yo[4] = {b4.x, b4.y, b4.z, b4.w};
            float xv[4] = {u4.x, u4.y, u4.z, u4.w}, yv[4] = {v4.x, v4.y, v4.z, v4.w};
            push_quad<GATHER, DEPOSIT, false>(A.geo, W, cc, xo, yo, xv, yv, ke, px, py, bad);
            store_quad(A, s0 + l, cc, xo, yo, xv, yv);
        }
        __syncthreads();  // every thread is done with this stage's buffer
        if (threadIdx.x == 0 && k + PIPE_STAGES < nstages) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(k + PIPE_STAGES);
        }
    }
    if (timed_out) {
        // wait (bounded) for the copies still in flight into this block's
        // shared memory, report, and leave without flushing partial results
        if (threadIdx.x == 0) {
            for (int j = k; j < nstages && j < k + PIPE_STAGES; ++j)
                mbar_wait_bounded(bar + (j % PIPE_STAGES), (unsigned)((j / PIPE_STAGES) & 1));
            atomicOr(&A.geo.dev->err, (unsigned)PIC_DEVERR_TIMEOUT);
        }
        return;
    }
    finish_block<DEPOSIT>(A.geo, W, sAcc, ke, px, py, bad);
}

// ------------------------------------------------------------------------
// Warp-specialised pipeline.  One producer warp streams the chunk into a
// ring of WS_STAGES shared-memory stages of WS_STAGE particles (five
// cp.async.bulk copies per stage on the bulk-copy engine, completion counted
// in bytes on the stage's "full" mbarrier); WS_CONSUMERS consumer warps each
// wait on a stage's full barrier, push one quad per thread straight from
// shared memory, store the results to global memory and arrive on the
// stage's "empty" barrier, which the producer waits on before refilling the
// slot.  No block-wide barrier inside the loop, so the copies of later
// stages stay in flight while the consumers compute.  Every wait is bounded:
// on expiry the block raises PIC_DEVERR_TIMEOUT, waits (bounded) for the
// copies still in flight into its shared memory and leaves without flushing.
// ------------------------------------------------------------------------
constexpr int WS_CONSUMERS = 8;
constexpr int WS_THREADS = 32 * (WS_CONSUMERS + 1);
constexpr int WS_STAGE = 4 * 32 * WS_CONSUMERS;  // one quad per consumer thread
// two stages: 3 blocks (24 consumer warps) per SM at 2048^2 x 32 ppc, 1.095
// ms per push against 1.277 with three or 1.283 with four stages (2 blocks
// per SM) and 1.046 for the direct kernel's 32 warps, whose latency hiding
// the consumers' gather and deposit need more than the copies' depth
constexpr int WS_STAGES = 2;

__device__ __forceinline__ void mbar_arrive(unsigned long long *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// the window, the diagnostics, full and empty barriers, then the ring
__host__ __device__ __forceinline__ size_t ws_ring_offset(size_t wbytes)
{
    return ((wbytes + 32 + 2 * WS_STAGES * 8) + 127) & ~(size_t)127;
}

template <bool GATHER, bool DEPOSIT>
__global__ void __launch_bounds__(WS_THREADS) push_kernel_ws(PushArgs A)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const long long n = *A.d_n;
    const long long base = (long long)blockIdx.x * A.chunk;
    if (base >= n) return;  // block-uniform
    const long long n4 = (n + 3) & ~3ll;
    const long long end = min(base + (long long)A.chunk, n4);
    const Window W = setup_window(A.geo, smem, A.anchor[blockIdx.x]);
    const size_t wb = window_bytes(A.geo.wcx, A.geo.wcy);
    double *sAcc = reinterpret_cast<double *>(smem + wb);
    unsigned long long *full = reinterpret_cast<unsigned long long *>(smem + wb + 32);
    unsigned long long *empty = full + WS_STAGES;
    unsigned char *ring = smem + ws_ring_offset(wb);
    const int nstages = (int)((end - base + WS_STAGE - 1) / WS_STAGE);
    constexpr size_t field_bytes = (size_t)WS_STAGE * 4;
    constexpr size_t stage_bytes = 5 * field_bytes;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int k = 0; k < WS_STAGES; ++k) {
            mbar_init(full + k, 1u);
            mbar_init(empty + k, (unsigned)WS_CONSUMERS);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    load_window<GATHER, DEPOSIT>(A.geo, W);
    if (threadIdx.x < 3) sAcc[threadIdx.x] = 0.0;
    __syncthreads();

    float ke = 0.f, px = 0.f, py = 0.f;
    bool bad = false, timed_out = false;
    int issued = 0;
    if (warp == WS_CONSUMERS) {
        if (lane == 0) {
            for (int k = 0; k < nstages; ++k) {
                const int sl = k % WS_STAGES;
                if (k >= WS_STAGES) {  // the consumers of stage k - WS_STAGES released the slot
                    if (!mbar_wait_bounded(empty + sl, (unsigned)((k / WS_STAGES - 1) & 1))) {
                        timed_out = true;
                        break;
                    }
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                }
                const long long s0 = base + (long long)k * WS_STAGE;
                const unsigned bytes = (unsigned)min((long long)WS_STAGE, end - s0) * 4u;  // 16-byte multiple
                unsigned char *dst = ring + (size_t)sl * stage_bytes;
                mbar_expect_tx(full + sl, 5u * bytes);
                bulk_g2s(dst + 0 * field_bytes, A.cin + s0, bytes, full + sl);
                bulk_g2s(dst + 1 * field_bytes, A.oxin + s0, bytes, full + sl);
                bulk_g2s(dst + 2 * field_bytes, A.oyin + s0, bytes, full + sl);
                bulk_g2s(dst + 3 * field_bytes, A.vxin + s0, bytes, full + sl);
                bulk_g2s(dst + 4 * field_bytes, A.vyin + s0, bytes, full + sl);
                issued = k + 1;
            }
        }
    } else {
        const int l = 4 * threadIdx.x;  // this thread's quad in every stage
        for (int k = 0; k < nstages; ++k) {
            const int sl = k % WS_STAGES;
            if (!mbar_wait_bounded(full + sl, (unsigned)((k / WS_STAGES) & 1))) {
                timed_out = true;
                break;
            }
            const long long s0 = base + (long long)k * WS_STAGE;
            const int cnt = (int)min((long long)WS_STAGE, end - s0);
            if (l < cnt) {
                const unsigned char *st = ring + (size_t)sl * stage_bytes;
                const int4 c4 = *reinterpret_cast<const int4 *>(st + 0 * field_bytes + 4 * l);
                const float4 a4 = *reinterpret_cast<const float4 *>(st + 1 * field_bytes + 4 * l);
                const float4 b4 = *reinterpret_cast<const float4 *>(st + 2 * field_bytes + 4 * l);
                const float4 u4 = *reinterpret_cast<const float4 *>(st + 3 * field_bytes + 4 * l);
                const float4 v4 = *reinterpret_cast<const float4 *>(st + 4 * field_bytes + 4 * l);
                int cc[4] = {c4.x, c4.y, c4.z, c4.w};
                float xo[4] = {a4.x, a4.y, a4.z, a4.w}, yo[4] = {b4.x, b4.y, b4.z, b4.w};
                float xv[4] = {u4.x, u4.y, u4.z, u4.w}, yv[4] = {v4.x, v4.y, v4.z, v4.w};
                push_quad<GATHER, DEPOSIT, false>(A.geo, W, cc, xo, yo, xv, yv, ke, px, py, bad);
                store_quad(A, s0 + l, cc, xo, yo, xv, yv);
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(empty + sl);
        }
    }
    if (__syncthreads_or(timed_out ? 1 : 0)) {
        // wait (bounded) for the copies still in flight into this block's
        // shared memory, report, and leave without flushing partial results
        if (warp == WS_CONSUMERS && lane == 0) {
            for (int j = max(0, issued - WS_STAGES); j < issued; ++j)
                mbar_wait_bounded(full + j % WS_STAGES, (unsigned)((j / WS_STAGES) & 1));
            atomicOr(&A.geo.dev->err, (unsigned)PIC_DEVERR_TIMEOUT);
        }
        return;
    }
    finish_block<DEPOSIT>(A.geo, W, sAcc, ke, px, py, bad);
}

size_t push_ws_smem(const Geometry &g)
{
    return ws_ring_offset(window_bytes(g.wcx, g.wcy)) + (size_t)WS_STAGES * 5 * WS_STAGE * 4;
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

size_t push_bulk_smem(const Geometry &g)
{
    return tma_ring_offset(window_bytes(g.wcx, g.wcy)) + (size_t)PIPE_STAGES * 5 * STAGE_PARTICLES * 4;
}

// set on every launch: the attribute belongs to the current device, and a
// process may drive several
template <bool G, bool D> static pic_status bulk_attr(size_t sm)
{
    PIC_CUDA(cudaFuncSetAttribute(push_kernel_bulk<G, D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sm));
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
    if (h->use_bulk) {
        const size_t sm = push_bulk_smem(g);
        if (charged && dep) {
            PIC_TRY((bulk_attr<true, true>(sm)));
            push_kernel_bulk<true, true><<<grid, block, sm, h->stream>>>(A);
        } else if (charged) {
            PIC_TRY((bulk_attr<true, false>(sm)));
            push_kernel_bulk<true, false><<<grid, block, sm, h->stream>>>(A);
        } else if (dep) {
            PIC_TRY((bulk_attr<false, true>(sm)));
            push_kernel_bulk<false, true><<<grid, block, sm, h->stream>>>(A);
        } else {
            PIC_TRY((bulk_attr<false, false>(sm)));
            push_kernel_bulk<false, false><<<grid, block, sm, h->stream>>>(A);
        }
    } else if (h->cfg.push_variant == 4) {
        const size_t sm = push_ws_smem(g);
        const dim3 wsb(WS_THREADS);
        auto attr = [&](const void *f) -> pic_status {
            PIC_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
            return PIC_OK;
        };
        if (charged && dep) {
            PIC_TRY(attr((const void *)push_kernel_ws<true, true>));
            push_kernel_ws<true, true><<<grid, wsb, sm, h->stream>>>(A);
        } else if (charged) {
            PIC_TRY(attr((const void *)push_kernel_ws<true, false>));
            push_kernel_ws<true, false><<<grid, wsb, sm, h->stream>>>(A);
        } else if (dep) {
            PIC_TRY(attr((const void *)push_kernel_ws<false, true>));
            push_kernel_ws<false, true><<<grid, wsb, sm, h->stream>>>(A);
        } else {
            PIC_TRY(attr((const void *)push_kernel_ws<false, false>));
            push_kernel_ws<false, false><<<grid, wsb, sm, h->stream>>>(A);
        }
    } else if (h->cfg.push_variant == 3) {
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
