// pic_sort.cu -- counting sort of a species by cell, in tile-major order.
//
// Replaces the reference's per-cell particle lists (taylorj5/msc-thesis,
// thesisCode/dsmcCollisions/cellTrackerAdvanced/src/main.cc:269-278
// cellTracking on the CPU; src/pic.cu:419-790 cellTrackerSetup / Migration on
// the GPU) with a stable-layout counting sort:
//   key(cell) = ((ty * ntx + tx) * th + ly) * tw + lx  for the tile (tx, ty)
//               and the in-tile coordinates (lx, ly);
//   1. histogram of keys            (warp-aggregated atomics)
//   2. exclusive scan -> offsets    (three-kernel block scan)
//   3. scatter buffer 0 -> buffer 1 (warp-aggregated cursor atomics)
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

__global__ void __launch_bounds__(256) sort_hist_kernel(SortArgs A)
{
    const long long n = *A.d_n;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    for (long long b = (long long)blockIdx.x * blockDim.x; b < n; b += stride) {  // warp-uniform
        const long long i = b + threadIdx.x;
        int key = -1 - lane;
        if (i < n) {
            const int c = A.cin[i];
            const int cx = c & 0xFFFF, cy = c >> 16;
            if (c >= 0 && cx < A.nx && cy < A.ny)
                key = cell_key(c, A.tw, A.th, A.ntx);
            else
                atomicOr(A.err, (unsigned)PIC_DEVERR_CELL);
        }
        const unsigned grp = __match_any_sync(0xffffffffu, key);
        if (key >= 0 && lane == __ffs(grp) - 1) atomicAdd(A.count + key, (uint32_t)__popc(grp));
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

__global__ void __launch_bounds__(256) sort_scatter_kernel(SortArgs A)
{
    const long long n = *A.d_n;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    const int tcells = A.tw * A.th;
    for (long long b = (long long)blockIdx.x * blockDim.x; b < n; b += stride) {  // warp-uniform
        const long long i = b + threadIdx.x;
        int key = -1 - lane, c = -1;
        if (i < n) {
            c = A.cin[i];
            const int cx = c & 0xFFFF, cy = c >> 16;
            if (c >= 0 && cx < A.nx && cy < A.ny) key = cell_key(c, A.tw, A.th, A.ntx);
        }
        const unsigned grp = __match_any_sync(0xffffffffu, key);
        const int leader = __ffs(grp) - 1;
        uint32_t base = 0;
        if (key >= 0 && lane == leader) base = atomicAdd(A.cursor + key, (uint32_t)__popc(grp));
        base = __shfl_sync(grp, base, leader);
        if (key < 0) continue;
        const uint32_t rank = __popc(grp & ((1u << lane) - 1u));
        const long long d = (long long)base + rank;
        A.cout[d] = c;
        A.oxout[d] = A.oxin[i];
        A.oyout[d] = A.oyin[i];
        A.vxout[d] = A.vxin[i];
        A.vyout[d] = A.vyin[i];
        A.pidout[d] = A.pidin[i];
        if (A.vzin) A.vzout[d] = A.vzin[i];
        if (d % A.chunk == 0) {
            const int t = key / tcells;
            const int ntx = A.ntx;
            A.anchor[d / A.chunk] = (t % ntx) | ((t / ntx) << 16);
        }
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
    PIC_CUDA(cudaMemsetAsync(h->count, 0, sizeof(uint32_t) * (size_t)ncell, h->stream));
    PIC_CUDA(cudaMemsetAsync(B.anchor, 0xFF, sizeof(int32_t) * (size_t)B.nchunks, h->stream));
    const int gp = grid_for(B.cap, 256);
    sort_hist_kernel<<<gp, 256, 0, h->stream>>>(A);
    PIC_CUDA(cudaGetLastError());
    scan_blocks_kernel<<<h->scan_blocks, 1024, 0, h->stream>>>(h->count, h->offset, ncell, h->bsum);
    PIC_CUDA(cudaGetLastError());
    scan_bsum_kernel<<<1, 1024, 0, h->stream>>>(h->bsum, h->scan_blocks);
    PIC_CUDA(cudaGetLastError());
    scan_add_kernel<<<grid_for(ncell, 256), 256, 0, h->stream>>>(h->offset, h->cursor, ncell,
                                                               h->bsum, &h->dev->n[s]);
    PIC_CUDA(cudaGetLastError());
    sort_scatter_kernel<<<gp, 256, 0, h->stream>>>(A);
    PIC_CUDA(cudaGetLastError());
    return PIC_OK;
}

}  // namespace pic
