// pic_ensemble.cu -- many independent collisionless runs advanced together.
//
// Layout: all runs share one set of pools.  Run r (in slot order, runs of
// one grid size adjacent) owns particle slots [poff, poff + cap4) of every
// particle array, nodes [goff, goff + ncp) of rho_fix and rho, the field
// planes e[2 goff ...] (Ex, then Ey ncp later), the half spectra
// rhohat[khoff ...] and ehat[khoff ...] (Ex^, then Ey^ nk later; the
// spectrum pools hold 2 nk per run, rhohat uses the first nk), and sort
// keys [key_off, key_off + nx ny] (the last one is its bin of empty slots).
// ncp is nx*ny rounded up to 4 so that every run's grids start 32-byte
// aligned.  Each step is one launch per stage over all runs, driven by
// per-block work tables (run, first item, item count):
//   push      chunks of `chunk` particles of one run (fused gather + push +
//             deposit, the single-run device code with the run's geometry)
//   sort      SORT_CHUNK slots of one run; one global key space, so one
//             histogram, one scan and one scatter sort every run at once and
//             each run's particles land in its own slots
//   convert   2048 nodes of one run; k-space: 2048 modes of one run
//   FFTs      one batched cuFFT plan per grid size (R2C over the runs' rho,
//             C2R over their Ex^, Ey^ pairs)
// The steps are captured in CUDA graphs as in the single-run handle.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "pic_ensemble.cuh"
#include "pic_field_dev.cuh"
#include "pic_push_dev.cuh"

namespace pic {


// ------------------------------------------------------------------ kernels
template <bool GATHER, bool DEPOSIT>
__global__ void __launch_bounds__(256, 4)
ens_push_kernel(PushArgs A, const SegBlock *__restrict__ blk, const EnsRun *__restrict__ runs,
                const int32_t *__restrict__ anchor, float kick, float drift)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const SegBlock b = blk[blockIdx.x];
    const EnsRun &R = runs[b.run];
    PushGeo G;
    G.ex = A.geo.ex + 2 * R.goff;
    G.ey = G.ex + R.ncp;
    G.rho = A.geo.rho + R.goff;
    G.dev = A.geo.dev + b.run;
    G.nx = R.nx;
    G.ny = R.ny;
    G.tw = R.tw;
    G.th = R.th;
    G.hx = R.hx;
    G.hy = R.hy;
    G.wcx = R.wcx;
    G.wcy = R.wcy;
    G.qm_dt = R.qm_dt * kick;
    G.dtdx = R.dtdx * drift;
    G.dtdy = R.dtdy * drift;
    G.qmul = R.qmul;
    G.ke_scale = drift > 0.f ? R.ke_scale : 0.0;
    G.p_scale = R.p_scale;
    G.recount = nullptr;
    G.ntx = R.ntx;
    push_block<GATHER, DEPOSIT, false>(A, G, smem, b.base, b.base + b.count, anchor[blockIdx.x]);
}

__device__ __forceinline__ KeyGeo run_geo(const EnsRun &R, int rows)
{
    return key_geo(R.nx, R.ny, R.tw, R.th, R.ntx, R.key_off, rows);
}

// histogram blocks count HIST_BLOCK consecutive particles of one run
__global__ void __launch_bounds__(SORT_THREADS)
ens_sort_hist_kernel(SortArgs A, const SegBlock *__restrict__ blk, const EnsRun *__restrict__ runs)
{
    __shared__ uint32_t cnt[SORT_KEYS];
    const SegBlock b = blk[blockIdx.x];
    sort_hist_segments(A, run_geo(runs[b.run], A.rows), cnt, b.base, b.base + b.count);
}

// The scatter loops over the sort-block table with a grid of resident
// blocks, each fetching its next table entry's particles into L2 while it
// moves the current one.

__global__ void __launch_bounds__(SORT_THREADS, 4)
ens_sort_scatter_kernel(SortArgs A, const SegBlock *__restrict__ blk,
                        const EnsRun *__restrict__ runs, int nblk)
{
    extern __shared__ __align__(16) unsigned char smem[];
    ScatterSmem &S = *reinterpret_cast<ScatterSmem *>(smem);
    for (int i = blockIdx.x; i < nblk; i += gridDim.x) {
        if (i + (int)gridDim.x < nblk) {
            const SegBlock nb = blk[i + gridDim.x];
            prefetch_chunk(A, nb.base, nb.base + nb.count);
        }
        const SegBlock b = blk[i];
        sort_scatter_block(A, run_geo(runs[b.run], A.rows), S, b.base, b.base + b.count);
        __syncthreads();  // the next entry reuses the shared memory
    }
}

// tile of the first particle of every push block, from the sorted buffer
__global__ void ens_anchor_kernel(const int32_t *__restrict__ cell, const SegBlock *__restrict__ blk,
                                  const EnsRun *__restrict__ runs, int nblk, int32_t *anchor)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nblk) return;
    const SegBlock b = blk[i];
    const EnsRun &R = runs[b.run];
    const int c = cell[b.base];
    if (c < 0 || (c & 0xFFFF) >= R.nx || (c >> 16) >= R.ny) {
        anchor[i] = -1;
        return;
    }
    const int t = cell_key(c, R.tw, R.th, R.ntx) / (R.tw * R.th);
    anchor[i] = (t % R.ntx) | ((t / R.ntx) << 16);
}

// rho = (rho_fix - mean) * scale per run, exact charge sum per run.  Nodes
// in pairs (ncp is a multiple of 4); nodes past nx*ny are padding.
__global__ void __launch_bounds__(256)
ens_convert_kernel(const unsigned long long *__restrict__ rho_fix, float *__restrict__ rho,
                   const SegBlock *__restrict__ blk, const EnsRun *__restrict__ runs, DevState *devs)
{
    __shared__ unsigned long long s_part[8];
    const SegBlock b = blk[blockIdx.x];
    const EnsRun &R = runs[b.run];
    const long long ncell = (long long)R.nx * R.ny;
    const long long mean = R.mean_fix;
    const float scale = R.rho_scale;
    unsigned long long qs = 0;
    for (long long j = 2ll * threadIdx.x; j < b.count; j += 2ll * blockDim.x) {
        const long long node = b.base + j;       // local node index (even)
        const long long g = R.goff + node;
        const ulonglong2 v = *reinterpret_cast<const ulonglong2 *>(rho_fix + g);
        if (node + 1 < ncell) {
            qs += v.x + v.y;
            *reinterpret_cast<float2 *>(rho + g) =
                make_float2(fixed_to_float(v.x, mean, scale), fixed_to_float(v.y, mean, scale));
        } else if (node < ncell) {
            qs += v.x;
            rho[g] = fixed_to_float(v.x, mean, scale);
        }
    }
    qs = warp_sum_u64(qs);
    if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = qs;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_part[w];
        atomicAdd(&devs[b.run].q[acc_slot()], t);
    }
}

__global__ void __launch_bounds__(256)
ens_kspace_kernel(const float2 *__restrict__ rhohat, float2 *__restrict__ ehat,
                  const SegBlock *__restrict__ blk, const EnsRun *__restrict__ runs, DevState *devs)
{
    __shared__ double s_part[8];
    const SegBlock b = blk[blockIdx.x];
    const EnsRun &R = runs[b.run];
    float fe = 0.f;
    for (long long j = threadIdx.x; j < b.count; j += blockDim.x) {
        const long long idx = b.base + j;  // local mode index
        const int my = (int)idx / R.nh;  // a run's modes fit in 32 bits
        const int mx = (int)idx - my * R.nh;
        const KMode K = kspace_mode(rhohat[R.khoff + idx], mx, my, R.nx, R.ny, R.kx1, R.ky1,
                                    R.inv_eps0_n, idx == 0);
        ehat[R.khoff + idx] = K.ex;
        ehat[R.khoff + R.nk + idx] = K.ey;
        fe += K.fe;
    }
    double d = warp_sum_d((double)fe);
    if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = d;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_part[w];
        atomicAdd(&devs[b.run].fe[acc_slot()], t);
    }
}

// diagnostics fold, one warp per run
__global__ void ens_advance_kernel(DevState *devs, double *hist, int cap, int kind,
                                   const EnsRun *__restrict__ runs)
{
    const int r = blockIdx.x;
    advance_state(devs + r, hist + (size_t)r * 6 * cap, cap, kind, runs[r].fe_scale);
}

}  // namespace pic

// ------------------------------------------------------------------ host side
using namespace pic;

namespace pic {

pic_status ens_bad(const std::string &m)
{
    set_error("pic_ensemble_create: " + m);
    return PIC_ERR_INVALID_ARG;
}

size_t window_smem(const EnsRun &R)
{
    return window_bytes(R.wcx, R.wcy) + 32;
}

void ens_free(pic_ensemble *E)
{
    if (!E) return;
    cudaSetDevice(E->device);
    if (E->stream) cudaStreamSynchronize(E->stream);
    void *ptrs[] = {E->d_runs, E->cell[0], E->cell[1], E->ox[0], E->ox[1], E->oy[0], E->oy[1],
                    E->vx[0], E->vx[1], E->vy[0], E->vy[1], E->pid[0], E->pid[1], E->rho_fix,
                    E->rho, E->e, E->rhohat, E->ehat, E->count, E->offset, E->cursor, E->bsum,
                    E->bsum_s, E->bsum2, E->d_total, E->push_blk, E->sort_blk, E->node_blk,
                    E->mode_blk, E->hist_blk, E->anchor, E->dev, E->hist, E->stage};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (auto &G : E->groups) {
        if (G.r2c) cufftDestroy(G.r2c);
        if (G.c2r) cufftDestroy(G.c2r);
        if (G.r2c2) cufftDestroy(G.r2c2);
        if (G.c2r1) cufftDestroy(G.c2r1);
        if (G.tw) cudaFree(G.tw);
    }
    if (E->g_one) cudaGraphExecDestroy(E->g_one);
    if (E->g_period) cudaGraphExecDestroy(E->g_period);
    if (E->g_sortstep) cudaGraphExecDestroy(E->g_sortstep);
    if (E->stream) cudaStreamDestroy(E->stream);
    delete E;
}

template <class T> pic_status upload(T **d, const std::vector<T> &h)
{
    PIC_TRY(ens_alloc(d, h.size()));
    if (!h.empty()) PIC_CUDA(cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    return PIC_OK;
}

// blocks of at most `per` items over [0, len) of one run
void add_blocks(std::vector<SegBlock> &v, int run, long long start, long long len, long long per)
{
    for (long long b = 0; b < len; b += per)
        v.push_back(SegBlock{start + b, (int)std::min(per, len - b), run});
}

pic_status ens_layout(pic_ensemble *E)
{
    const int nr = E->nruns;
    std::vector<int> order(nr);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        const pic_config &A = E->cfg[a], &B = E->cfg[b];
        return A.nx != B.nx ? A.nx < B.nx : A.ny < B.ny;
    });
    E->run_of = order;
    E->slot_of.assign(nr, 0);
    for (int s = 0; s < nr; ++s) E->slot_of[order[s]] = s;
    E->runs.resize(nr);
    long long poff = 0, goff = 0, khoff = 0;
    long long koff = 0;
    std::vector<SegBlock> sb, nb, mb, hb;
    for (int s = 0; s < nr; ++s) {
        const pic_config &c = E->cfg[order[s]];
        const pic_species_desc &D = c.species[0];
        EnsRun &R = E->runs[s];
        memset(&R, 0, sizeof R);
        R.nx = c.nx;
        R.ny = c.ny;
        R.nh = c.nx / 2 + 1;
        R.dx = c.Lx / c.nx;
        R.dy = c.Ly / c.ny;
        const long long ncell = (long long)c.nx * c.ny;
        const double ppc = std::max(1.0, (double)D.capacity / (double)ncell);
        const int tcells = std::max(1, (int)std::lround(E->chunk / ppc));
        R.tw = pick_divisor(c.nx, std::min(16, tcells));
        R.th = pick_tile_h(c.ny, tcells, R.tw);
        R.ntx = c.nx / R.tw;
        R.nty = c.ny / R.th;
        R.hx = R.hy = E->halo;
        R.wcx = 2 * R.tw + 2 * R.hx;
        R.wcy = R.th + 2 * R.hy;
        if (window_smem(R) > WINDOW_SMEM_MAX) return ens_bad("shared-memory window too large for a run");
        R.cap4 = (D.capacity + 3) & ~3ll;
        R.poff = poff;
        R.ncp = (ncell + 3) & ~3ll;
        R.goff = goff;
        R.nk = (long long)c.ny * R.nh;
        R.khoff = khoff;
        if (koff + ncell + 1 >= (1ll << 30)) return ens_bad("key space of the runs exceeds 2^30");
        R.key_off = (int)koff;
        R.qm_dt = (float)(D.q / D.m * c.dt);
        R.dtdx = (float)(c.dt / R.dx);
        R.dtdy = (float)(c.dt / R.dy);
        const double q_unit = D.q / D.q_int;
        R.rho_scale = (float)(q_unit / (4294967296.0 * R.dx * R.dy));
        R.kx1 = (float)(2.0 * 3.14159265358979323846 / c.Lx);
        R.ky1 = (float)(2.0 * 3.14159265358979323846 / c.Ly);
        R.inv_eps0_n = (float)(1.0 / (c.eps0 * (double)c.nx * (double)c.ny));
        R.qmul = (unsigned long long)(long long)D.q_int;
        R.dt = (float)c.dt;
        R.inv_dx = (float)(1.0 / R.dx);
        R.inv_dy = (float)(1.0 / R.dy);
        R.q_dA = (float)(D.q / (R.dx * R.dy));
        R.eps0_dA = (float)(c.eps0 * R.dx * R.dy);
        R.ke_scale = 0.25 * D.m;
        R.p_scale = 0.5 * D.m;
        R.fe_scale = 0.5 * c.eps0 * R.dx * R.dy * (double)c.nx * (double)c.ny;
        poff += R.cap4;
        goff += R.ncp;
        khoff += 2 * R.nk;
        koff += ncell + 1;
        add_blocks(sb, s, R.poff, R.cap4, SORT_CHUNK);
        add_blocks(hb, s, R.poff, R.cap4, HIST_BLOCK);
        add_blocks(nb, s, 0, R.ncp, ENS_NODES_PER_BLOCK);
        add_blocks(mb, s, 0, R.nk, ENS_NODES_PER_BLOCK);
    }
    E->nslots = poff;
    E->nnodes = goff;
    E->nmodes = khoff;
    E->nkeys = koff;
    PIC_TRY(upload(&E->sort_blk, sb));
    PIC_TRY(upload(&E->hist_blk, hb));
    E->nhist = (int)hb.size();
    PIC_TRY(upload(&E->node_blk, nb));
    PIC_TRY(upload(&E->mode_blk, mb));
    E->nsort = (int)sb.size();
    E->nnode_blk = (int)nb.size();
    E->nmode_blk = (int)mb.size();
    // FFT groups
    for (int s = 0; s < nr;) {
        int t = s;
        while (t < nr && E->runs[t].nx == E->runs[s].nx && E->runs[t].ny == E->runs[s].ny) ++t;
        pic_ensemble::Group G;
        G.nx = E->runs[s].nx;
        G.ny = E->runs[s].ny;
        G.first = s;
        G.count = t - s;
        E->groups.push_back(G);
        s = t;
    }
    return PIC_OK;
}

// Window halos from the fastest particles of each run's load: the halo
// along an axis covers half the drift of a sort period (the mean
// displacement at which a particle is pushed), at least the configured halo,
// as far as a window of WINDOW_SMEM_TARGET bytes allows.
void ens_windows(pic_ensemble *E, const pic_init_spec *specs)
{
    E->push_smem = 0;
    for (int s = 0; s < E->nruns; ++s) {
        EnsRun &R = E->runs[s];
        const int r = E->run_of[s];
        const pic_init_spec &S = specs[r];
        const double dt = E->cfg[r].dt;
        double ux = std::fabs(S.vdrift[0]) + std::fabs(S.beam_v) + 4.0 * std::fabs(S.vth[0]);
        for (int b = 0; b < 2; ++b) ux += std::hypot(S.beam_u[b][0], S.beam_u[b][1]);
        const double uy = std::fabs(S.vdrift[1]) + 4.0 * std::fabs(S.vth[1]);
        const double half = 0.5 * E->sort_every * dt;
        R.hx = std::max(E->halo, std::min(24, (int)std::ceil(ux * half / R.dx)));
        R.hy = std::max(E->halo, std::min(24, (int)std::ceil(uy * half / R.dy)));
        for (;;) {
            R.wcx = 2 * R.tw + 2 * R.hx;
            R.wcy = R.th + 2 * R.hy;
            if (window_smem(R) <= WINDOW_SMEM_TARGET || (R.hx <= E->halo && R.hy <= E->halo)) break;
            if (R.hx >= R.hy && R.hx > E->halo)
                --R.hx;
            else
                --R.hy;
        }
        E->push_smem = std::max(E->push_smem, window_smem(R));
    }
}

// push blocks need the particle counts, known at init
pic_status ens_push_table(pic_ensemble *E, const std::vector<long long> &n_slot)
{
    std::vector<SegBlock> pb;
    for (int s = 0; s < E->nruns; ++s) {
        EnsRun &R = E->runs[s];
        R.n = n_slot[s];
        add_blocks(pb, s, R.poff, (R.n + 3) & ~3ll, E->chunk);
    }
    if (E->push_blk) cudaFree(E->push_blk);
    if (E->anchor) cudaFree(E->anchor);
    E->push_blk = nullptr;
    E->anchor = nullptr;
    PIC_TRY(upload(&E->push_blk, pb));
    E->npush = (int)pb.size();
    PIC_TRY(ens_alloc(&E->anchor, (size_t)E->npush));
    PIC_CUDA(cudaMemset(E->anchor, 0xFF, sizeof(int32_t) * std::max(1, E->npush)));
    PIC_CUDA(cudaMemcpy(E->d_runs, E->runs.data(), sizeof(EnsRun) * E->runs.size(),
                        cudaMemcpyHostToDevice));
    return PIC_OK;
}

pic_status ens_plans(pic_ensemble *E)
{
    E->spectral = true;
    for (auto &G : E->groups) E->spectral = E->spectral && spectral_wanted(G.nx, G.ny);
    if (E->spectral)
        for (auto &G : E->groups) PIC_TRY(spectral_twiddles(G.nx, G.ny, &G.tw));
    for (auto &G : E->groups) {
        const EnsRun &R = E->runs[G.first];
        // explicit embeddings: with NULL ones cuFFT ignores the batch distances
        int dims[2] = {G.ny, G.nx}, real_emb[2] = {G.ny, G.nx}, cplx_emb[2] = {G.ny, R.nh};
        // R2C: rho planes (stride ncp) -> rhohat (stride 2 nk)
        PIC_CUFFT(cufftPlanMany(&G.r2c, 2, dims, real_emb, 1, (int)R.ncp, cplx_emb, 1,
                                (int)(2 * R.nk), CUFFT_R2C, G.count));
        PIC_CUFFT(cufftSetStream(G.r2c, E->stream));
        // C2R: Ex^, Ey^ of every run (stride nk) -> Ex, Ey planes (stride ncp)
        PIC_CUFFT(cufftPlanMany(&G.c2r, 2, dims, cplx_emb, 1, (int)R.nk, real_emb, 1, (int)R.ncp,
                                CUFFT_C2R, 2 * G.count));
        PIC_CUFFT(cufftSetStream(G.c2r, E->stream));
    }
    return PIC_OK;
}

PushArgs ens_push_args(pic_ensemble *E, int src)
{
    PushArgs A;
    memset(&A, 0, sizeof A);
    A.cin = E->cell[src];
    A.oxin = E->ox[src];
    A.oyin = E->oy[src];
    A.vxin = E->vx[src];
    A.vyin = E->vy[src];
    A.cout = E->cell[0];
    A.oxout = E->ox[0];
    A.oyout = E->oy[0];
    A.vxout = E->vx[0];
    A.vyout = E->vy[0];
    A.pidin = src ? E->pid[1] : nullptr;
    A.pidout = E->pid[0];
    A.geo.ex = E->e;
    A.geo.rho = E->rho_fix;
    A.geo.dev = E->dev;
    A.chunk = E->chunk;
    return A;
}

pic_status ens_launch_push(pic_ensemble *E, int src, int kind)
{
    if (!E->npush) return PIC_OK;
    const PushArgs A = ens_push_args(E, src);
    dim3 grid((unsigned)E->npush), block(256);
    const size_t sm = E->push_smem;
    cudaStream_t st = E->stream;
    PIC_TRY(allow_dynamic_smem((const void *)ens_push_kernel<true, true>, sm));
    PIC_TRY(allow_dynamic_smem((const void *)ens_push_kernel<true, false>, sm));
    PIC_TRY(allow_dynamic_smem((const void *)ens_push_kernel<false, true>, sm));
    if (kind == 0)
        ens_push_kernel<true, true><<<grid, block, sm, st>>>(A, E->push_blk, E->d_runs, E->anchor, 1.f, 1.f);
    else if (kind == 1)
        ens_push_kernel<true, false><<<grid, block, sm, st>>>(A, E->push_blk, E->d_runs, E->anchor, -0.5f, 0.f);
    else if (kind == 2)
        ens_push_kernel<false, true><<<grid, block, sm, st>>>(A, E->push_blk, E->d_runs, E->anchor, 0.f, 0.f);
    else
        ens_push_kernel<false, true><<<grid, block, sm, st>>>(A, E->push_blk, E->d_runs, E->anchor, 0.f, -1.f);
    PIC_CUDA(cudaGetLastError());
    return PIC_OK;
}

pic_status ens_advance(pic_ensemble *E, int kind)
{
    ens_advance_kernel<<<E->nruns, ACC_SLOTS, 0, E->stream>>>(E->dev, E->hist, E->hist_cap, kind,
                                                               E->d_runs);
    PIC_CUDA(cudaGetLastError());
    return PIC_OK;
}

pic_status ens_poisson(pic_ensemble *E)
{
    cudaStream_t st = E->stream;
    if (E->spectral) {
        for (auto &G : E->groups)
            PIC_TRY(launch_spectral_runs(E->d_runs, G.first, G.count, G.nx, G.ny, E->rho_fix,
                                         E->rho, E->rhohat, E->ehat, E->e, G.tw, E->dev, st));
        PIC_CUDA(cudaMemsetAsync(E->rho_fix, 0, sizeof(unsigned long long) * (size_t)E->nnodes, st));
        return ens_advance(E, ADV_FIELD);
    }
    ens_convert_kernel<<<E->nnode_blk, 256, 0, st>>>(E->rho_fix, E->rho, E->node_blk, E->d_runs, E->dev);
    PIC_CUDA(cudaGetLastError());
    PIC_CUDA(cudaMemsetAsync(E->rho_fix, 0, sizeof(unsigned long long) * (size_t)E->nnodes, st));
    for (auto &G : E->groups) {
        const EnsRun &R = E->runs[G.first];
        PIC_CUFFT(cufftExecR2C(G.r2c, E->rho + R.goff, (cufftComplex *)(E->rhohat + R.khoff)));
    }
    ens_kspace_kernel<<<E->nmode_blk, 256, 0, st>>>(E->rhohat, E->ehat, E->mode_blk, E->d_runs, E->dev);
    PIC_CUDA(cudaGetLastError());
    for (auto &G : E->groups) {
        const EnsRun &R = E->runs[G.first];
        PIC_CUFFT(cufftExecC2R(G.c2r, (cufftComplex *)(E->ehat + R.khoff), E->e + 2 * R.goff));
    }
    return ens_advance(E, ADV_FIELD);
}

SortArgs ens_sort_args(pic_ensemble *E, const float *const *xin, float *const *xout)
{
    SortArgs A;
    memset(&A, 0, sizeof A);
    A.cin = E->cell[0];
    A.oxin = E->ox[0];
    A.oyin = E->oy[0];
    A.vxin = E->vx[0];
    A.vyin = E->vy[0];
    A.vzin = nullptr;
    A.pidin = E->pid[0];
    A.cout = E->cell[1];
    A.oxout = E->ox[1];
    A.oyout = E->oy[1];
    A.vxout = E->vx[1];
    A.vyout = E->vy[1];
    A.vzout = nullptr;
    A.pidout = E->pid[1];
    A.count = E->count;
    A.cursor = E->cursor;
    A.nkeys = E->nkeys;
    A.nslots = E->nslots;
    A.err = &E->dev[0].err;
    // keys are tile rows; the sparsest run (particles per row) sizes the window
    A.rows = 1;
    double density = 1e30;
    for (const EnsRun &R : E->runs)
        if (R.n) density = std::min(density, (double)R.n * R.tw / ((double)R.nx * R.ny));
    sort_sizes_for(density, &A.wkeys, &A.hbits);
    for (int k = 0; k < 4; ++k) {
        A.xin[k] = xin ? reinterpret_cast<const uint32_t *>(xin[k]) : nullptr;
        A.xout[k] = xout ? reinterpret_cast<uint32_t *>(xout[k]) : nullptr;
    }
    return A;
}

// sort every run from buffer 0 into buffer 1; push-block anchors
pic_status ens_sort(pic_ensemble *E, const float *const *xin, float *const *xout)
{
    cudaStream_t st = E->stream;
    const SortArgs A = ens_sort_args(E, xin, xout);
    PIC_CUDA(cudaMemsetAsync(E->count, 0, sizeof(uint32_t) * (size_t)E->nkeys, st));
    ens_sort_hist_kernel<<<E->nhist, SORT_THREADS, 0, st>>>(A, E->hist_blk, E->d_runs);
    PIC_CUDA(cudaGetLastError());
    PIC_TRY(launch_key_scan(E->count, E->offset, E->cursor, E->nkeys, E->bsum, E->bsum_s, E->bsum2,
                            E->d_total, st));
    PIC_TRY(scatter_smem_attr((const void *)ens_sort_scatter_kernel));
    ens_sort_scatter_kernel<<<sort_grid(E->nsort, 4), SORT_THREADS, SCATTER_SMEM, st>>>(
        A, E->sort_blk, E->d_runs, E->nsort);
    PIC_CUDA(cudaGetLastError());
    if (E->npush) {
        ens_anchor_kernel<<<(E->npush + 255) / 256, 256, 0, st>>>(E->cell[1], E->push_blk, E->d_runs,
                                                                  E->npush, E->anchor);
        PIC_CUDA(cudaGetLastError());
    }
    return PIC_OK;
}

pic_status ens_step_body(pic_ensemble *E, int src)
{
    PIC_TRY(ens_launch_push(E, src, 0));
    PIC_TRY(ens_advance(E, ADV_PUSH));
    return ens_poisson(E);
}

template <class F> pic_status ens_capture(pic_ensemble *E, cudaGraphExec_t *out, F &&body)
{
    cudaGraph_t graph = nullptr;
    PIC_CUDA(cudaStreamBeginCapture(E->stream, cudaStreamCaptureModeThreadLocal));
    pic_status s = body();
    cudaError_t e = cudaStreamEndCapture(E->stream, &graph);
    if (s != PIC_OK) {
        if (graph) cudaGraphDestroy(graph);
        return s;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    return PIC_OK;
}

pic_status ens_graphs(pic_ensemble *E)
{
    if (E->g_one) cudaGraphExecDestroy(E->g_one);
    if (E->g_period) cudaGraphExecDestroy(E->g_period);
    if (E->g_sortstep) cudaGraphExecDestroy(E->g_sortstep);
    E->g_one = E->g_period = E->g_sortstep = nullptr;
    PIC_TRY(ens_capture(E, &E->g_one, [&] { return ens_step_body(E, 0); }));
    PIC_TRY(ens_capture(E, &E->g_sortstep, [&] {
        PIC_TRY(ens_sort(E));
        return ens_step_body(E, 1);
    }));
    PIC_TRY(ens_capture(E, &E->g_period, [&] {
        PIC_TRY(ens_sort(E));
        PIC_TRY(ens_step_body(E, 1));
        for (int k = 1; k < E->sort_every; ++k) PIC_TRY(ens_step_body(E, 0));
        return PIC_OK;
    }));
    return PIC_OK;
}

pic_status ens_need(pic_ensemble *E, int run)
{
    if (!E) {
        set_error("null ensemble");
        return PIC_ERR_INVALID_ARG;
    }
    PIC_CUDA(cudaSetDevice(E->device));
    if (run >= 0 && run >= E->nruns) {
        set_error("run index out of range");
        return PIC_ERR_INVALID_ARG;
    }
    return PIC_OK;
}

}  // namespace pic

// ------------------------------------------------------------------ C ABI
extern "C" {

pic_status pic_ensemble_create(const pic_config *runs, int nruns, pic_ensemble **out)
{
    if (!out) return ens_bad("null output");
    *out = nullptr;
    if (!runs || nruns < 1) return ens_bad("need at least one run");
    const pic_config &c0 = runs[0];
    if (c0.chunk < 0 || c0.chunk % 4 || c0.chunk > MAX_CHUNK || c0.halo < 0 || c0.sort_every < 0 ||
        c0.history < 0)
        return ens_bad("bad chunk, halo, sort_every or history in runs[0]");
    for (int r = 0; r < nruns; ++r) {
        const pic_config &c = runs[r];
        if (c.nx < 2 || c.ny < 2 || c.nx > 32768 || c.ny > 32768 || (long long)c.nx * c.ny >= (1 << 24))
            return ens_bad("run " + std::to_string(r) + ": nx, ny out of range");
        if (!(c.Lx > 0) || !(c.Ly > 0) || !(c.dt > 0) || !(c.eps0 > 0))
            return ens_bad("run " + std::to_string(r) + ": Lx, Ly, dt, eps0 must be positive");
        if (c.nspecies != 1) return ens_bad("run " + std::to_string(r) + ": one species per run");
        const pic_species_desc &D = c.species[0];
        if (D.capacity < 0 || D.capacity > (1ll << 31) - 4096 || !(D.m > 0) || D.q_int == 0 ||
            !(D.q / D.q_int > 0))
            return ens_bad("run " + std::to_string(r) + ": species needs capacity, m > 0 and q, q_int of one sign");
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0 || c0.device < 0 || c0.device >= ndev) {
        set_error("pic_ensemble_create: no usable CUDA device");
        return PIC_ERR_NO_DEVICE;
    }
    pic_ensemble *E = new pic_ensemble();
    E->device = c0.device;
    E->nruns = nruns;
    E->cfg.assign(runs, runs + nruns);
    E->chunk = c0.chunk ? c0.chunk : 8192;
    E->halo = c0.halo ? c0.halo : 2;
    E->sort_every = c0.sort_every ? c0.sort_every : 20;
    E->hist_cap = c0.history ? c0.history : 4096;
    auto fail = [&](pic_status s) {
        ens_free(E);
        return s;
    };
#define E_TRY(call)                                                                            \
    do {                                                                                       \
        pic_status s_ = (call);                                                                \
        if (s_ != PIC_OK) return fail(s_);                                                     \
    } while (0)
    if (cudaSetDevice(E->device) != cudaSuccess) return fail(PIC_ERR_CUDA);
    if (cudaStreamCreateWithFlags(&E->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(PIC_ERR_CUDA);
    E_TRY(ens_layout(E));
    E_TRY(ens_alloc(&E->d_runs, (size_t)nruns));
    const size_t ns = (size_t)E->nslots;
    for (int b = 0; b < 2; ++b) {
        E_TRY(ens_alloc(&E->cell[b], ns));
        E_TRY(ens_alloc(&E->ox[b], ns));
        E_TRY(ens_alloc(&E->oy[b], ns));
        E_TRY(ens_alloc(&E->vx[b], ns));
        E_TRY(ens_alloc(&E->vy[b], ns));
        E_TRY(ens_alloc(&E->pid[b], ns));
        if (cudaMemset(E->cell[b], 0xFF, ns * 4) != cudaSuccess) return fail(PIC_ERR_CUDA);
        if (cudaMemset(E->pid[b], 0, ns * 4) != cudaSuccess) return fail(PIC_ERR_CUDA);
    }
    E_TRY(ens_alloc(&E->rho_fix, (size_t)E->nnodes));
    E_TRY(ens_alloc(&E->rho, (size_t)E->nnodes));
    E_TRY(ens_alloc(&E->e, 2 * (size_t)E->nnodes));
    E_TRY(ens_alloc(&E->rhohat, (size_t)E->nmodes));
    E_TRY(ens_alloc(&E->ehat, (size_t)E->nmodes));
    if (cudaMemset(E->rho_fix, 0, 8 * (size_t)E->nnodes) != cudaSuccess) return fail(PIC_ERR_CUDA);
    if (cudaMemset(E->rho, 0, 4 * (size_t)E->nnodes) != cudaSuccess) return fail(PIC_ERR_CUDA);
    E_TRY(ens_alloc(&E->count, (size_t)E->nkeys));
    E_TRY(ens_alloc(&E->offset, (size_t)E->nkeys + 1));
    E_TRY(ens_alloc(&E->cursor, (size_t)E->nkeys));
    const size_t nb1 = (size_t)((E->nkeys + 4095) / 4096), nb2 = (nb1 + 4095) / 4096;
    E_TRY(ens_alloc(&E->bsum, nb1));
    E_TRY(ens_alloc(&E->bsum_s, nb1));
    E_TRY(ens_alloc(&E->bsum2, nb2));
    E_TRY(ens_alloc(&E->d_total, 1));
    const long long total = E->nslots;
    if (cudaMemcpy(E->d_total, &total, 8, cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(PIC_ERR_CUDA);
    E_TRY(ens_alloc(&E->dev, (size_t)nruns));
    E_TRY(ens_alloc(&E->hist, (size_t)nruns * 6 * E->hist_cap));
    if (cudaMemset(E->dev, 0, sizeof(DevState) * nruns) != cudaSuccess) return fail(PIC_ERR_CUDA);
    E_TRY(ens_plans(E));
    E_TRY(ens_push_table(E, std::vector<long long>(nruns, 0)));
#undef E_TRY
    *out = E;
    return PIC_OK;
}

pic_status pic_ensemble_destroy(pic_ensemble *e)
{
    ens_free(e);
    return PIC_OK;
}

pic_status pic_ensemble_get_stream(pic_ensemble *e, void **stream)
{
    PIC_TRY(ens_need(e, -1));
    if (!stream) return PIC_ERR_INVALID_ARG;
    *stream = (void *)e->stream;
    return PIC_OK;
}

pic_status pic_ensemble_synchronize(pic_ensemble *e)
{
    PIC_TRY(ens_need(e, -1));
    PIC_CUDA(cudaStreamSynchronize(e->stream));
    unsigned err = 0;
    for (int r = 0; r < e->nruns; ++r) {
        unsigned v = 0;
        PIC_CUDA(cudaMemcpy(&v, &e->dev[r].err, sizeof v, cudaMemcpyDeviceToHost));
        err |= v;
    }
    if (err & PIC_DEVERR_CELL) {
        set_error("device: cell index outside the grid");
        return PIC_ERR_STATE;
    }
    if (err & PIC_DEVERR_SORT) {
        set_error("device: a sort destination fell outside the slots");
        return PIC_ERR_STATE;
    }
    if (err & PIC_DEVERR_TIMEOUT) {
        set_error("device: a bounded wait gave up");
        return PIC_ERR_TIMEOUT;
    }
    if (err & PIC_DEVERR_NAN) {
        set_error("device: non-finite particle velocity");
        return PIC_ERR_NAN;
    }
    return PIC_OK;
}

pic_status pic_ensemble_init(pic_ensemble *e, const pic_init_spec *specs)
{
    PIC_TRY(ens_need(e, -1));
    if (!specs) return PIC_ERR_INVALID_ARG;
    std::vector<long long> n_slot(e->nruns);
    std::vector<int> lx(e->nruns, 0), ly(e->nruns, 0);
    for (int r = 0; r < e->nruns; ++r) {
        const pic_init_spec &S = specs[r];
        if (S.n < 0 || S.n > e->cfg[r].species[0].capacity) {
            set_error("pic_ensemble_init: run " + std::to_string(r) + ": count exceeds capacity");
            return PIC_ERR_INVALID_ARG;
        }
        if (S.layout == PIC_LOAD_LATTICE)
            PIC_TRY(lattice_dims_for(e->cfg[r].nx, e->cfg[r].ny, S.n, &lx[r], &ly[r]));
        n_slot[e->slot_of[r]] = S.n;
    }
    cudaStream_t st = e->stream;
    PIC_CUDA(cudaStreamSynchronize(st));
    const size_t ns = (size_t)e->nslots;
    for (int b = 0; b < 2; ++b) PIC_CUDA(cudaMemsetAsync(e->cell[b], 0xFF, ns * 4, st));
    ens_windows(e, specs);
    PIC_TRY(ens_push_table(e, n_slot));
    std::vector<DevState> z(e->nruns);
    memset(z.data(), 0, sizeof(DevState) * z.size());
    for (int s = 0; s < e->nruns; ++s) {
        EnsRun &R = e->runs[s];
        const pic_config &c = e->cfg[e->run_of[s]];
        z[s].n[0] = R.n;
        const __int128 tot = (__int128)c.species[0].q_int * R.n * ((__int128)1 << 32);
        R.mean_fix = (long long)(tot / ((__int128)R.nx * R.ny));
        InitTarget T;
        T.cell = e->cell[0] + R.poff;
        T.ox = e->ox[0] + R.poff;
        T.oy = e->oy[0] + R.poff;
        T.vx = e->vx[0] + R.poff;
        T.vy = e->vy[0] + R.poff;
        T.vz = nullptr;
        T.pid = e->pid[0] + R.poff;
        T.nx = R.nx;
        T.ny = R.ny;
        T.Lx = c.Lx;
        T.Ly = c.Ly;
        const int r = e->run_of[s];
        PIC_TRY(launch_init_target(T, &specs[r], lx[r], ly[r], st));
    }
    PIC_CUDA(cudaMemcpyAsync(e->d_runs, e->runs.data(), sizeof(EnsRun) * e->runs.size(),
                             cudaMemcpyHostToDevice, st));
    PIC_CUDA(cudaMemcpyAsync(e->dev, z.data(), sizeof(DevState) * z.size(), cudaMemcpyHostToDevice, st));
    PIC_CUDA(cudaMemsetAsync(e->hist, 0, sizeof(double) * 6 * e->hist_cap * (size_t)e->nruns, st));
    PIC_CUDA(cudaMemsetAsync(e->rho_fix, 0, 8 * (size_t)e->nnodes, st));
    // radix sort of the loads into buffer 1, deposit while copying back,
    // solve, prime
    {
        uint32_t *scratch = nullptr;
        void *temp = nullptr;
        size_t temp_bytes = 0;
        // packed records when they fit with 1 GiB to spare
        size_t free_b = 0, total_b = 0;
        PIC_CUDA(cudaMemGetInfo(&free_b, &total_b));
        const bool packed = free_b >= 48 * ns + (1ull << 30);
        PIC_CUDA(cudaMalloc(&scratch, (packed ? 48 : 16) * ns));
        pic_status sorted = ens_import_sort(e, scratch, packed, &temp, &temp_bytes);
        if (sorted == PIC_OK && e->npush) {
            ens_anchor_kernel<<<(e->npush + 255) / 256, 256, 0, st>>>(e->cell[1], e->push_blk,
                                                                      e->d_runs, e->npush, e->anchor);
            if (cudaGetLastError() != cudaSuccess) sorted = PIC_ERR_CUDA;
        }
        cudaStreamSynchronize(st);
        cudaFree(scratch);
        if (temp) cudaFree(temp);
        PIC_TRY(sorted);
    }
    PIC_TRY(ens_launch_push(e, 1, 2));
    PIC_TRY(ens_poisson(e));
    PIC_TRY(ens_launch_push(e, 0, 1));
    PIC_CUDA(cudaStreamSynchronize(st));  // z lives on this stack frame
    e->since_sort = 0;
    PIC_TRY(ens_graphs(e));
    e->ready = true;
    return PIC_OK;
}

pic_status pic_ensemble_step(pic_ensemble *e, long long nsteps)
{
    PIC_TRY(ens_need(e, -1));
    if (nsteps < 0) return PIC_ERR_INVALID_ARG;
    if (!e->ready) {
        set_error("pic_ensemble_step: call pic_ensemble_init first");
        return PIC_ERR_STATE;
    }
    const int S = e->sort_every;
    long long n = nsteps;
    while (n > 0) {
        if (e->since_sort >= S) {
            if (n >= S) {
                PIC_CUDA(cudaGraphLaunch(e->g_period, e->stream));
                n -= S;
                e->since_sort = S;
            } else {
                PIC_CUDA(cudaGraphLaunch(e->g_sortstep, e->stream));
                n -= 1;
                e->since_sort = 1;
            }
        } else {
            PIC_CUDA(cudaGraphLaunch(e->g_one, e->stream));
            n -= 1;
            e->since_sort++;
        }
    }
    return PIC_OK;
}

pic_status pic_ensemble_diagnostics(pic_ensemble *e, int run, pic_diag *d)
{
    PIC_TRY(ens_need(e, run));
    if (run < 0 || !d) return PIC_ERR_INVALID_ARG;
    const int s = e->slot_of[run];
    PIC_CUDA(cudaStreamSynchronize(e->stream));
    DevState st;
    PIC_CUDA(cudaMemcpy(&st, e->dev + s, sizeof st, cudaMemcpyDeviceToHost));
    const int cap = e->hist_cap;
    std::vector<double> h(6 * (size_t)cap);
    PIC_CUDA(cudaMemcpy(h.data(), e->hist + (size_t)s * 6 * cap, sizeof(double) * h.size(),
                        cudaMemcpyDeviceToHost));
    memset(d, 0, sizeof *d);
    d->step = st.step;
    d->field_energy = h[st.step % cap];
    d->total_charge_fixed = (long long)h[4 * (size_t)cap + st.step % cap];
    if (st.step > 0) {
        const long long k = (st.step - 1) % cap;
        d->kinetic_energy = h[1 * (size_t)cap + k];
        d->momentum[0] = h[2 * (size_t)cap + k];
        d->momentum[1] = h[3 * (size_t)cap + k];
    }
    d->n[0] = st.n[0];
    d->expected_charge_fixed =
        (long long)((unsigned long long)(long long)e->cfg[run].species[0].q_int *
                    ((unsigned long long)st.n[0] << 32));
    d->error_flags = st.err;
    return PIC_OK;
}

pic_status pic_ensemble_get_history(pic_ensemble *e, int run, int which, long long first,
                                    long long count, double *out)
{
    PIC_TRY(ens_need(e, run));
    if (run < 0 || which < 0 || which > 5 || first < 0 || count < 0 || (count && !out))
        return PIC_ERR_INVALID_ARG;
    const int s = e->slot_of[run];
    PIC_CUDA(cudaStreamSynchronize(e->stream));
    long long step = 0;
    PIC_CUDA(cudaMemcpy(&step, &e->dev[s].step, sizeof step, cudaMemcpyDeviceToHost));
    const bool per_push = (which >= 1 && which <= 3);
    const long long last = per_push ? step - 1 : step;
    const int cap = e->hist_cap;
    if (count && (first + count - 1 > last || first < last - cap + 1)) {
        set_error("pic_ensemble_get_history: range outside the kept history");
        return PIC_ERR_INVALID_ARG;
    }
    std::vector<double> ring((size_t)cap);
    PIC_CUDA(cudaMemcpy(ring.data(), e->hist + ((size_t)s * 6 + which) * cap, sizeof(double) * cap,
                        cudaMemcpyDeviceToHost));
    for (long long i = 0; i < count; ++i) out[i] = ring[(size_t)((first + i) % cap)];
    return PIC_OK;
}

pic_status pic_ensemble_get_particles(pic_ensemble *e, int run, long long *n, double *x, double *y,
                                      double *vx, double *vy)
{
    PIC_TRY(ens_need(e, run));
    if (run < 0) return PIC_ERR_INVALID_ARG;
    const int s = e->slot_of[run];
    const EnsRun &R = e->runs[s];
    if (n) *n = R.n;
    if (!R.n || !(x || y || vx || vy)) return PIC_OK;
    const size_t m = (size_t)R.n;
    if (e->stage_n < 4 * m) {
        cudaFree(e->stage);
        e->stage = nullptr;
        e->stage_n = 0;
        PIC_CUDA(cudaMalloc(&e->stage, 4 * m * sizeof(double)));
        e->stage_n = 4 * m;
    }
    cudaStream_t st = e->stream;
    const pic_config &c = e->cfg[run];
    InitTarget T;
    T.cell = e->cell[0] + R.poff;
    T.ox = e->ox[0] + R.poff;
    T.oy = e->oy[0] + R.poff;
    T.vx = e->vx[0] + R.poff;
    T.vy = e->vy[0] + R.poff;
    T.vz = nullptr;
    T.pid = e->pid[0] + R.poff;
    T.nx = R.nx;
    T.ny = R.ny;
    T.Lx = c.Lx;
    T.Ly = c.Ly;
    double *d = e->stage;
    PIC_TRY(launch_to_global_target(T, &e->dev[s].n[0], R.cap4, d, d + m, d + 2 * m, d + 3 * m, st));
    double *outs[4] = {x, y, vx, vy};
    for (int k = 0; k < 4; ++k)
        if (outs[k])
            PIC_CUDA(cudaMemcpyAsync(outs[k], d + k * m, m * 8, cudaMemcpyDeviceToHost, st));
    PIC_CUDA(cudaStreamSynchronize(st));
    return PIC_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ autotuner
namespace {

pic_status ens_time_candidate(const std::vector<pic_config> &runs, const pic_init_spec *specs,
                              int trial_steps, double *ms)
{
    pic_ensemble *e = nullptr;
    PIC_TRY(pic_ensemble_create(runs.data(), (int)runs.size(), &e));
    pic_status st = pic_ensemble_init(e, specs);
    const int S = e->sort_every;
    const long long steps = ((long long)(trial_steps + S - 1) / S) * S;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (st == PIC_OK) st = pic_ensemble_step(e, 2 * S);  // warm-up (a sort period)
    if (st == PIC_OK) st = pic_ensemble_synchronize(e);
    if (st == PIC_OK && cudaEventCreate(&e0) != cudaSuccess) st = PIC_ERR_CUDA;
    if (st == PIC_OK && cudaEventCreate(&e1) != cudaSuccess) st = PIC_ERR_CUDA;
    if (st == PIC_OK) {
        cudaEventRecord(e0, e->stream);
        st = pic_ensemble_step(e, steps);
        cudaEventRecord(e1, e->stream);
        if (st == PIC_OK) st = pic_ensemble_synchronize(e);
        float t = 0.f;
        if (st == PIC_OK && cudaEventElapsedTime(&t, e0, e1) == cudaSuccess)
            *ms = t / (double)steps;
        else if (st == PIC_OK)
            st = PIC_ERR_CUDA;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    pic_ensemble_destroy(e);
    return st;
}

}  // namespace

extern "C" pic_status pic_ensemble_autotune(pic_config *runs, int nruns, const pic_init_spec *specs,
                                            int trial_steps, pic_tune_result *out)
{
    if (!runs || nruns < 1 || !specs || trial_steps < 1) {
        set_error("pic_ensemble_autotune: null argument, no runs or trial_steps < 1");
        return PIC_ERR_INVALID_ARG;
    }
    std::vector<pic_config> cur(runs, runs + nruns);
    if (!cur[0].sort_every) cur[0].sort_every = 20;
    double best_ms = 1e300;
    int best_chunk = 0, best_se = cur[0].sort_every, tried = 0;
    for (int c : {2048, 4096, 8192, 16384}) {
        cur[0].chunk = c;
        double ms = 0.0;
        const pic_status st = ens_time_candidate(cur, specs, trial_steps, &ms);
        if (st == PIC_ERR_INVALID_ARG) continue;  // a run's window too large for this chunk
        if (st != PIC_OK) return st;
        ++tried;
        if (ms < best_ms) {
            best_ms = ms;
            best_chunk = c;
        }
    }
    if (!tried) {
        set_error("pic_ensemble_autotune: no candidate could be created");
        return PIC_ERR_INVALID_ARG;
    }
    cur[0].chunk = best_chunk;
    const int first_se = cur[0].sort_every;
    for (int se : {1, 2, 3, 5, 10, 20}) {
        if (se == first_se) continue;
        cur[0].sort_every = se;
        double ms = 0.0;
        PIC_TRY(ens_time_candidate(cur, specs, trial_steps, &ms));
        ++tried;
        if (ms < best_ms) {
            best_ms = ms;
            best_se = se;
        }
    }
    runs[0].chunk = best_chunk;
    runs[0].sort_every = best_se;
    if (out) {
        out->chunk = best_chunk;
        out->tile_w = out->tile_h = 0;
        out->sort_every = best_se;
        out->ms_per_step = best_ms;
        out->tried = tried;
    }
    return PIC_OK;
}
