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
// distinct key; keys outside the window use global atomics directly.
// After the scatter, offset[key] .. offset[key+1] is the slice of cell `key`
// and every push chunk knows the tile of its first particle (anchor).
#include <cuda_runtime.h>

#include "pic_internal.cuh"

namespace pic {

__device__ __forceinline__ int cell_key(int c, int tw, int th, int ntx)
{
    const int cx = c & 0xFFFF, cy = c >> 16;
    const int tx = cx / tw, lx = cx - tx * tw;
    const int ty = cy / th, ly = cy - ty * th;
    return ((ty * ntx + tx) * th + ly) * tw + lx;
}

struct SortArgs {
    const int32_t *cin;
    const float *oxin, *oyin, *vxin, *vyin, *vzin;
    const uint32_t *pidin;
    int32_t *cout;
    float *oxout, *oyout, *vxout, *vyout, *vzout;
    uint32_t *pidout;
    uint32_t *count, *cursor;
    int32_t *anchor;
    const long long *d_n;
    int nx, ny, tw, th, ntx, chunk;
    unsigned int *err;
};

constexpr int SORT_THREADS = 256;
constexpr int SORT_PER_THREAD = 16;
constexpr int SORT_CHUNK = SORT_THREADS * SORT_PER_THREAD;
constexpr int SORT_KEYS = 2048;

// key of particle i; empty slots (cell < 0) inside [0, n) get the extra key
// ncell so that they sort to the end and keep their slot count; a corrupt
// cell is flagged and treated the same way
__device__ __forceinline__ int particle_key(const SortArgs &A, long long i)
{
    const int c = A.cin[i];
    const int empty = A.nx * A.ny;
    if (c < 0) return empty;
    const int cx = c & 0xFFFF, cy = c >> 16;
    if (cx >= A.nx || cy >= A.ny) {
        atomicOr(A.err, (unsigned)PIC_DEVERR_CELL);
        return empty;
    }
    return cell_key(c, A.tw, A.th, A.ntx);
}

// first key of this block's shared-memory window (block-uniform)
__device__ __forceinline__ int window_start(const SortArgs &A, long long base, long long n)
{
    const long long mid = min(base + SORT_CHUNK / 2, n - 1);
    const int c = A.cin[mid];
    int k = 0;
    if (c >= 0 && (c & 0xFFFF) < A.nx && (c >> 16) < A.ny) k = cell_key(c, A.tw, A.th, A.ntx);
    return max(0, k - SORT_KEYS / 2);
}

__global__ void __launch_bounds__(SORT_THREADS) sort_hist_kernel(SortArgs A)
{
    __shared__ uint32_t s_cnt[SORT_KEYS];
    const long long n = *A.d_n;
    const long long base = (long long)blockIdx.x * SORT_CHUNK;
    if (base >= n) return;
    const long long ncell = (long long)A.nx * A.ny;
    const int k0 = window_start(A, base, n);
    for (int r = threadIdx.x; r < SORT_KEYS; r += SORT_THREADS) s_cnt[r] = 0u;
    __syncthreads();
#pragma unroll 4
    for (int j = 0; j < SORT_PER_THREAD; ++j) {
        const long long i = base + (long long)j * SORT_THREADS + threadIdx.x;
        if (i >= n) break;
        const int key = particle_key(A, i);
        const unsigned r = (unsigned)(key - k0);
        if (r < (unsigned)SORT_KEYS)
            atomicAdd(s_cnt + r, 1u);
        else
            atomicAdd(A.count + key, 1u);
    }
    __syncthreads();
    for (int r = threadIdx.x; r < SORT_KEYS; r += SORT_THREADS) {
        const uint32_t v = s_cnt[r];
        if (v && k0 + r <= ncell) atomicAdd(A.count + k0 + r, v);
    }
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

__device__ __forceinline__ void move_particle(const SortArgs &A, long long i, long long d)
{
    A.cout[d] = A.cin[i];
    A.oxout[d] = A.oxin[i];
    A.oyout[d] = A.oyin[i];
    A.vxout[d] = A.vxin[i];
    A.vyout[d] = A.vyin[i];
    A.pidout[d] = A.pidin[i];
    if (A.vzin) A.vzout[d] = A.vzin[i];
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

__global__ void __launch_bounds__(SORT_THREADS) sort_scatter_kernel(SortArgs A)
{
    __shared__ uint32_t s_cnt[SORT_KEYS];
    __shared__ uint32_t s_base[SORT_KEYS];
    const long long n = *A.d_n;
    const long long base = (long long)blockIdx.x * SORT_CHUNK;
    if (base >= n) return;
    const long long ncell = (long long)A.nx * A.ny;
    const int k0 = window_start(A, base, n);
    for (int r = threadIdx.x; r < SORT_KEYS; r += SORT_THREADS) s_cnt[r] = 0u;
    __syncthreads();
    int keys[SORT_PER_THREAD];
#pragma unroll
    for (int j = 0; j < SORT_PER_THREAD; ++j) {
        const long long i = base + (long long)j * SORT_THREADS + threadIdx.x;
        keys[j] = -1;
        if (i < n) {
            const int c = A.cin[i];
            keys[j] = (c >= 0 && (c & 0xFFFF) < A.nx && (c >> 16) < A.ny)
                          ? cell_key(c, A.tw, A.th, A.ntx)
                          : (int)ncell;
        }
        const unsigned r = (unsigned)(keys[j] - k0);
        if (keys[j] >= 0 && r < (unsigned)SORT_KEYS) atomicAdd(s_cnt + r, 1u);
    }
    __syncthreads();
    // reserve each distinct key's slice of the output once per block
    for (int r = threadIdx.x; r < SORT_KEYS; r += SORT_THREADS) {
        const uint32_t v = s_cnt[r];
        s_base[r] = (v && k0 + r <= ncell) ? atomicAdd(A.cursor + k0 + r, v) : 0u;
        s_cnt[r] = 0u;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < SORT_PER_THREAD; ++j) {
        const int key = keys[j];
        if (key < 0) continue;
        const long long i = base + (long long)j * SORT_THREADS + threadIdx.x;
        const unsigned r = (unsigned)(key - k0);
        long long d;
        if (r < (unsigned)SORT_KEYS)
            d = (long long)s_base[r] + atomicAdd(s_cnt + r, 1u);
        else
            d = atomicAdd(A.cursor + key, 1u);
        move_particle(A, i, d);
    }
}

// Sort species s from buffer 0 into buffer 1 and compute the chunk anchors.
pic_status launch_sort(pic_handle *h, int s)
{
    SpeciesBuf &B = h->sp[s];
    const Geometry &g = h->g;
    if (B.cap == 0) return PIC_OK;
    const long long ncell = (long long)g.nx * g.ny;
    SortArgs A;
    A.cin = B.cell[0];
    A.oxin = B.ox[0];
    A.oyin = B.oy[0];
    A.vxin = B.vx[0];
    A.vyin = B.vy[0];
    A.vzin = B.vz[0];
    A.pidin = B.pid[0];
    A.cout = B.cell[1];
    A.oxout = B.ox[1];
    A.oyout = B.oy[1];
    A.vxout = B.vx[1];
    A.vyout = B.vy[1];
    A.vzout = B.vz[1];
    A.pidout = B.pid[1];
    A.count = h->count;
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
    const long long nkeys = ncell + 1;  // cells + the bin of empty slots
    PIC_CUDA(cudaMemsetAsync(h->count, 0, sizeof(uint32_t) * (size_t)nkeys, h->stream));
    PIC_CUDA(cudaMemsetAsync(B.anchor, 0xFF, sizeof(int32_t) * (size_t)B.nchunks, h->stream));
    const unsigned gp = (unsigned)((B.cap + SORT_CHUNK - 1) / SORT_CHUNK);
    sort_hist_kernel<<<gp, SORT_THREADS, 0, h->stream>>>(A);
    PIC_CUDA(cudaGetLastError());
    scan_blocks_kernel<<<h->scan_blocks, 1024, 0, h->stream>>>(h->count, h->offset, nkeys, h->bsum);
    PIC_CUDA(cudaGetLastError());
    scan_bsum_kernel<<<1, 1024, 0, h->stream>>>(h->bsum, h->scan_blocks);
    PIC_CUDA(cudaGetLastError());
    scan_add_kernel<<<grid_for(nkeys, 256), 256, 0, h->stream>>>(h->offset, h->cursor, nkeys,
                                                               h->bsum, &h->dev->n[s]);
    PIC_CUDA(cudaGetLastError());
    sort_scatter_kernel<<<gp, SORT_THREADS, 0, h->stream>>>(A);
    PIC_CUDA(cudaGetLastError());
    sort_anchor_kernel<<<(unsigned)((B.nchunks + 255) / 256), 256, 0, h->stream>>>(A, B.nchunks);
    PIC_CUDA(cudaGetLastError());
    return PIC_OK;
}

}  // namespace pic
