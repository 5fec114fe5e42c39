// pic_sort.cu -- counting sort of a species by cell, in tile-major order.
//
// Replaces the reference's per-cell particle lists (taylorj5/msc-thesis,
// thesisCode/dsmcCollisions/cellTrackerAdvanced/src/main.cc:269-278
// cellTracking on the CPU; src/pic.cu:419-790 cellTrackerSetup / Migration on
// the GPU) with a stable-layout counting sort:
//   key(cell) = ((ty * ntx + tx) * th + ly) * tw + lx  for the tile (tx, ty)
//               and the in-tile coordinates (lx, ly);
//   1. histogram of keys            (block-local shared-memory counts)
//   2. exclusive scan -> offsets    (three-kernel block scan)
//   3. scatter buffer 0 -> buffer 1 (block-local ranks, one global cursor
//                                    atomic per distinct key and block)
// The arrays are already nearly sorted from the previous sort, so the keys of
// a block's SORT_CHUNK consecutive particles fall in a short range: a block
// counts and ranks keys within a window of SORT_KEYS keys around its middle
// particle's key in shared memory and touches global memory once per
// distinct key.  Particles that crossed a tile row since the last sort jump
// by a whole tile row in key space; those stragglers are counted in a small
// open-addressing hash table in shared memory (again one global atomic per
// distinct key and block), and only when its bounded probe fails does a
// run of particles fall back to global atomics of its own.
// Each thread owns eight consecutive particles (128-bit loads of every
// field); the runs of equal keys among them are counted with one shared
// atomic each, whose result is also the run's rank among the block's
// particles of that key, so the scatter counts and ranks in one pass.  The
// scatter then stages every particle as one 32-byte record in shared memory
// in destination order (two 128-bit stores and loads per particle, the
// record rows XOR-swizzled against bank conflicts) and writes the fields
// out with consecutive threads on consecutive slots.
// After the scatter, offset[key] .. offset[key+1] is the slice of cell `key`
// and every push chunk knows the tile of its first particle (anchor).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "pic_sort_dev.cuh"

namespace pic {

// resident scatter blocks per SM that its grid is sized for: each block
// loops over chunks and prefetches its next chunk into L2 while it moves the
// current one (the histogram, one block per HIST_BLOCK particles, measured
// slower that way)
constexpr int SCATTER_BLOCKS_PER_SM = 4;

__global__ void __launch_bounds__(SORT_THREADS) sort_hist_kernel(SortArgs A)
{
    __shared__ uint32_t cnt[SORT_KEYS];
    const long long n = *A.d_n;
    const long long base = (long long)blockIdx.x * HIST_BLOCK;
    if (base >= n) return;
    sort_hist_segments(A, single_geo(A), cnt, base, n);
}

__global__ void __launch_bounds__(SORT_THREADS, SCATTER_BLOCKS_PER_SM) sort_scatter_kernel(SortArgs A)
{
    extern __shared__ __align__(16) unsigned char smem[];
    ScatterSmem &S = *reinterpret_cast<ScatterSmem *>(smem);
    const long long n = *A.d_n;
    const long long stride = (long long)SORT_CHUNK * gridDim.x;
    for (long long base = (long long)blockIdx.x * SORT_CHUNK; base < n; base += stride) {
        prefetch_chunk(A, base + stride, n);
        sort_scatter_block(A, single_geo(A), S, base, n);
        __syncthreads();  // the next iteration reuses the shared memory
    }
}

// blocks of a sort launch over `chunks` chunks: at most the resident blocks
unsigned sort_grid(long long chunks, int per_sm)
{
    const long long cap = (long long)device_sms() * per_sm;
    return (unsigned)std::max(1ll, std::min(chunks, cap));
}

// Exclusive scan, stage 1: each block scans 4096 entries (4 per thread).
__global__ void __launch_bounds__(1024)
scan_blocks_kernel(const uint32_t *__restrict__ in, uint32_t *__restrict__ out, long long n,
                   uint32_t *__restrict__ bsum)
{
    __shared__ uint32_t s_warp[32];
    const long long base = (long long)blockIdx.x * 4096 + 4ll * threadIdx.x;
    uint32_t v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) v[j] = (base + j < n) ? in[base + j] : 0u;
    const uint32_t t = v[0] + v[1] + v[2] + v[3];
    // inclusive warp scan of thread totals
    uint32_t x = t;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = s_warp[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        s_warp[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    uint32_t run = x - t + (warp ? s_warp[warp - 1] : 0u);  // exclusive prefix of this thread
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (base + j < n) out[base + j] = run;
        run += v[j];
    }
    if (threadIdx.x == blockDim.x - 1) bsum[blockIdx.x] = s_warp[31];
}

// Stage 2: exclusive scan of the block sums (at most 4096) in one block.
__global__ void __launch_bounds__(1024) scan_bsum_kernel(uint32_t *bsum, int nb)
{
    __shared__ uint32_t s_warp[32];
    uint32_t v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) v[j] = (4 * (int)threadIdx.x + j < nb) ? bsum[4 * threadIdx.x + j] : 0u;
    const uint32_t t = v[0] + v[1] + v[2] + v[3];
    uint32_t x = t;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = s_warp[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        s_warp[lane] = w;
    }
    __syncthreads();
    uint32_t run = x - t + (warp ? s_warp[warp - 1] : 0u);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (4 * (int)threadIdx.x + j < nb) bsum[4 * threadIdx.x + j] = run;
        run += v[j];
    }
}

// Stage 3: add block offsets; cursor = offset; offset[n] = total.
__global__ void __launch_bounds__(256)
scan_add_kernel(uint32_t *__restrict__ off, uint32_t *__restrict__ cursor, long long n,
                const uint32_t *__restrict__ bsum, const long long *d_total)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t v = off[i] + bsum[i >> 12];
        off[i] = v;
        cursor[i] = v;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) off[n] = (uint32_t)*d_total;
}

// Stage 3 of the second level: add the scanned sums of 4096-entry groups.
__global__ void __launch_bounds__(256)
scan_add_groups_kernel(uint32_t *__restrict__ v, long long n, const uint32_t *__restrict__ gsum)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        v[i] += gsum[i >> 12];
}

pic_status launch_key_scan(const uint32_t *count, uint32_t *offset, uint32_t *cursor,
                           long long nkeys, uint32_t *bsum, uint32_t *bsum_s, uint32_t *bsum2,
                           const long long *d_total, cudaStream_t st)
{
    const long long nb1 = (nkeys + 4095) / 4096;
    const long long nb2 = (nb1 + 4095) / 4096;
    if (nb2 > 4096) {
        set_error("key space too large for the two-level scan");
        return PIC_ERR_INVALID_ARG;
    }
    scan_blocks_kernel<<<(unsigned)nb1, 1024, 0, st>>>(count, offset, nkeys, bsum);
    PIC_CUDA(cudaGetLastError());
    const uint32_t *sums = bsum;
    if (nb1 <= 4096) {
        scan_bsum_kernel<<<1, 1024, 0, st>>>(bsum, (int)nb1);
        PIC_CUDA(cudaGetLastError());
    } else {
        scan_blocks_kernel<<<(unsigned)nb2, 1024, 0, st>>>(bsum, bsum_s, nb1, bsum2);
        PIC_CUDA(cudaGetLastError());
        scan_bsum_kernel<<<1, 1024, 0, st>>>(bsum2, (int)nb2);
        PIC_CUDA(cudaGetLastError());
        scan_add_groups_kernel<<<grid_for(nb1, 256), 256, 0, st>>>(bsum_s, nb1, bsum2);
        PIC_CUDA(cudaGetLastError());
        sums = bsum_s;
    }
    scan_add_kernel<<<grid_for(nkeys, 256), 256, 0, st>>>(offset, cursor, nkeys, sums, d_total);
    PIC_CUDA(cudaGetLastError());
    return PIC_OK;
}

// Tile of the first particle of every push chunk, read from the sorted array.
__global__ void sort_anchor_kernel(SortArgs A, long long nchunks)
{
    const long long n = *A.d_n;
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nchunks || b * A.chunk >= n) return;
    const int c = A.cout[b * A.chunk];
    if (c < 0 || (c & 0xFFFF) >= A.nx || (c >> 16) >= A.ny) return;
    const int t = cell_key(c, A.tw, A.th, A.ntx) / (A.tw * A.th);
    A.anchor[b] = (t % A.ntx) | ((t / A.ntx) << 16);
}

// the scatter kernels use more than the default 48 KB of dynamic shared
// memory, and four of their blocks per SM need the largest carveout
pic_status scatter_smem_attr(const void *kernel)
{
    PIC_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)SCATTER_SMEM));
    PIC_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                  (int)cudaSharedmemCarveoutMaxShared));
    return PIC_OK;
}

// Chunk anchors of species s from the sorted order in buffer `buf`.
pic_status launch_anchors(pic_handle *h, int s, int buf)
{
    SpeciesBuf &B = h->sp[s];
    const Geometry &g = h->g;
    if (!B.nchunks) return PIC_OK;
    SortArgs A;
    memset(&A, 0, sizeof A);
    A.cout = B.cell[buf];
    A.anchor = B.anchor;
    A.d_n = &h->dev->n[s];
    A.nx = g.nx;
    A.ny = g.ny;
    A.tw = g.tw;
    A.th = g.th;
    A.ntx = g.ntx;
    A.chunk = g.chunk;
    PIC_CUDA(cudaMemsetAsync(B.anchor, 0xFF, sizeof(int32_t) * (size_t)B.nchunks, h->stream));
    sort_anchor_kernel<<<(unsigned)((B.nchunks + 255) / 256), 256, 0, h->stream>>>(A, B.nchunks);
    PIC_CUDA(cudaGetLastError());
    return PIC_OK;
}

// Window keys and log2 hash slots for sort blocks over `density` particles
// per cell: a window four times the keys a block of sorted particles spans
// (at least 256, at most SORT_KEYS), a table of half as many slots (128 to
// HASH_SLOTS) for the particles that left the window's tile rows.
void sort_sizes_for(double density, int *wk, int *hb)
{
    const double span = SORT_CHUNK / std::max(density, 1e-9);
    int w = 256;
    while (w < SORT_KEYS && w < 4.0 * span) w *= 2;
    int b = 7;
    while ((1 << b) < HASH_SLOTS && (1 << b) < w / 2) ++b;
    *wk = w;
    *hb = b;
}

// Arguments of a sort of species s from buffer 0 into buffer 1.  The DSMC
// species counts into its own array (kept current by its pushes).
static SortArgs sort_args(pic_handle *h, int s, int from = 0)
{
    SpeciesBuf &B = h->sp[s];
    const Geometry &g = h->g;
    const long long ncell = (long long)g.nx * g.ny;
    SortArgs A;
    memset(&A, 0, sizeof A);
    const int to = 1 - from;
    A.cin = B.cell[from];
    A.oxin = B.ox[from];
    A.oyin = B.oy[from];
    A.vxin = B.vx[from];
    A.vyin = B.vy[from];
    A.vzin = B.vz[from];
    A.pidin = B.pid[from];
    A.cout = B.cell[to];
    A.oxout = B.ox[to];
    A.oyout = B.oy[to];
    A.vxout = B.vx[to];
    A.vyout = B.vy[to];
    A.vzout = B.vz[to];
    A.pidout = B.pid[to];
    const bool dsmc = h->dsmc.on && s == h->dsmc.s && h->dsmc.count;
    A.count = dsmc ? h->dsmc.count : h->count;
    A.cursor = h->cursor;
    A.anchor = B.anchor;
    A.d_n = &h->dev->n[s];
    A.nx = g.nx;
    A.ny = g.ny;
    A.tw = g.tw;
    A.th = g.th;
    A.ntx = g.ntx;
    A.chunk = g.chunk;
    A.err = &h->dev->err;
    A.nkeys = ncell + 1;  // cells + the bin of empty slots
    A.nslots = B.cap;
    // the DSMC species is sorted by cell (its pass pairs particles per cell);
    // every other species by tile row (keys 0 .. ncell / tw - 1 of the same space)
    A.rows = (h->dsmc.on && s == h->dsmc.s) ? 0 : 1;
    sort_sizes_for((double)B.n / (double)ncell * (A.rows ? g.tw : 1), &A.wkeys, &A.hbits);
    return A;
}

// Histogram of species s's buffer 0 into its counts (zeroed first).
static pic_status launch_hist(pic_handle *h, int s, const SortArgs &A)
{
    const SpeciesBuf &B = h->sp[s];
    PIC_CUDA(cudaMemsetAsync(A.count, 0, sizeof(uint32_t) * (size_t)A.nkeys, h->stream));
    sort_hist_kernel<<<(unsigned)((B.cap + HIST_BLOCK - 1) / HIST_BLOCK), SORT_THREADS, 0,
                       h->stream>>>(A);
    PIC_CUDA(cudaGetLastError());
    return PIC_OK;
}

// The DSMC species' counts recomputed from its buffer 0 (after a sort that
// did not count, an import).
pic_status launch_recount(pic_handle *h, int s)
{
    if (!(h->dsmc.on && s == h->dsmc.s && h->dsmc.count) || !h->sp[s].cap) return PIC_OK;
    return launch_hist(h, s, sort_args(h, s));
}

// Sort species s from buffer `from` into the other buffer (0 into 1 in the
// step) and compute the chunk anchors.  With counts_kept the DSMC species'
// pushes have kept its counts current since they were last computed, and
// the histogram is skipped.
pic_status launch_sort(pic_handle *h, int s, bool counts_kept, int from)
{
    SpeciesBuf &B = h->sp[s];
    if (B.cap == 0) return PIC_OK;
    const SortArgs A = sort_args(h, s, from);
    const bool dsmc = h->dsmc.on && s == h->dsmc.s && h->dsmc.count;
    const long long nkeys = A.nkeys;
    PIC_CUDA(cudaMemsetAsync(B.anchor, 0xFF, sizeof(int32_t) * (size_t)B.nchunks, h->stream));
    const unsigned gp = sort_grid((B.cap + SORT_CHUNK - 1) / SORT_CHUNK, SCATTER_BLOCKS_PER_SM);
    if (!(dsmc && counts_kept)) PIC_TRY(launch_hist(h, s, A));
    scan_blocks_kernel<<<h->scan_blocks, 1024, 0, h->stream>>>(A.count, h->offset, nkeys, h->bsum);
    PIC_CUDA(cudaGetLastError());
    scan_bsum_kernel<<<1, 1024, 0, h->stream>>>(h->bsum, h->scan_blocks);
    PIC_CUDA(cudaGetLastError());
    scan_add_kernel<<<grid_for(nkeys, 256), 256, 0, h->stream>>>(h->offset, h->cursor, nkeys,
                                                               h->bsum, &h->dev->n[s]);
    PIC_CUDA(cudaGetLastError());
    PIC_TRY(scatter_smem_attr((const void *)sort_scatter_kernel));
    sort_scatter_kernel<<<gp, SORT_THREADS, SCATTER_SMEM, h->stream>>>(A);
    PIC_CUDA(cudaGetLastError());
    sort_anchor_kernel<<<(unsigned)((B.nchunks + 255) / 256), 256, 0, h->stream>>>(A, B.nchunks);
    PIC_CUDA(cudaGetLastError());
    return PIC_OK;
}

}  // namespace pic
