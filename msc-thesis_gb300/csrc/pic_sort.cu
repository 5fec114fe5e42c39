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
// particle fall back to a global atomic of its own.
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
constexpr int SORT_PER_THREAD = 8;
constexpr int SORT_CHUNK = SORT_THREADS * SORT_PER_THREAD;
constexpr int SORT_KEYS = 2048;
constexpr int HASH_SLOTS = 1024;  // power of two
constexpr int HASH_PROBES = 8;
constexpr int HASH_EMPTY = -1;
constexpr int FALLBACK_BIT = 1 << 30;  // keys are < 2^24

__device__ __forceinline__ unsigned hash_key(int key)
{
    return ((unsigned)key * 0x9E3779B1u) >> 22;  // top 10 bits: HASH_SLOTS = 1024
}

// slot of `key` in the block's table, inserting it if absent; -1 if the
// bounded probe found no room
__device__ __forceinline__ int hash_insert(int *tab_key, int key)
{
    const unsigned h = hash_key(key);
    for (int p = 0; p < HASH_PROBES; ++p) {
        const int slot = (int)((h + p) & (HASH_SLOTS - 1));
        const int old = atomicCAS(tab_key + slot, HASH_EMPTY, key);
        if (old == HASH_EMPTY || old == key) return slot;
    }
    return -1;
}

// slot of a key that is already in the table
__device__ __forceinline__ int hash_find(const int *tab_key, int key)
{
    const unsigned h = hash_key(key);
    for (int p = 0; p < HASH_PROBES; ++p) {
        const int slot = (int)((h + p) & (HASH_SLOTS - 1));
        if (tab_key[slot] == key) return slot;
    }
    return 0;  // not reached for keys counted in the table
}

// Key of a particle with cell c.  Empty slots (cell < 0) inside [0, n) get
// the extra key ncell so that they sort to the end and keep their slot
// count; a corrupt cell is flagged and treated the same way.
__device__ __forceinline__ int particle_key(const SortArgs &A, int c)
{
    const int empty = A.nx * A.ny;
    if (c < 0) return empty;
    if ((c & 0xFFFF) >= A.nx || (c >> 16) >= A.ny) {
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

// Shared state of one sort block: dense window counts and the straggler table.
struct SortSmem {
    uint32_t cnt[SORT_KEYS];
    uint32_t base[SORT_KEYS];
    int hkey[HASH_SLOTS];
    uint32_t hcnt[HASH_SLOTS];
    uint32_t hbase[HASH_SLOTS];
};

__device__ __forceinline__ void init_smem(SortSmem &S)
{
    for (int r = threadIdx.x; r < SORT_KEYS; r += SORT_THREADS) S.cnt[r] = 0u;
    for (int r = threadIdx.x; r < HASH_SLOTS; r += SORT_THREADS) {
        S.hkey[r] = HASH_EMPTY;
        S.hcnt[r] = 0u;
    }
}

// Runs of equal keys across the 32 lanes of a warp (lanes hold consecutive
// particles, so in nearly sorted data a warp holds one or two runs).  Built
// from full-warp shuffles and ballots only: the head lane of each run does
// one atomic for the whole run and every lane knows its rank in the run.
struct Run {
    bool head;
    int hidx;  // lane of the run's head
    int len;   // run length (meaningful on the head)
    int rank;  // position of this lane in its run
};

__device__ __forceinline__ Run warp_run(int key)
{
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int prev = __shfl_up_sync(full, key, 1);
    const bool head = (lane == 0) || (key != prev);
    const unsigned heads = __ballot_sync(full, head);
    const unsigned upto = 0xffffffffu >> (31 - lane);  // lanes 0..lane
    const unsigned above = heads & ~upto;
    Run r;
    r.head = head;
    r.hidx = 31 - __clz(heads & upto);
    r.len = (above ? __ffs(above) - 1 : 32) - lane;
    r.rank = lane - r.hidx;
    return r;
}

// Pass 1 of both kernels: keys of this thread's particles, counted in the
// window or the table; a run the table had no room for gets FALLBACK_BIT.
__device__ __forceinline__ void count_keys(const SortArgs &A, SortSmem &S, long long base,
                                           long long n, int k0, int (&keys)[SORT_PER_THREAD])
{
#pragma unroll
    for (int j = 0; j < SORT_PER_THREAD; ++j) {
        const long long i = base + (long long)j * SORT_THREADS + threadIdx.x;
        keys[j] = (i < n) ? particle_key(A, A.cin[i]) : -1;
    }
#pragma unroll
    for (int j = 0; j < SORT_PER_THREAD; ++j) {  // warp-uniform
        const int key = keys[j];
        const Run R = warp_run(key);
        int fb = 0;
        if (R.head && key >= 0) {
            const unsigned r = (unsigned)(key - k0);
            if (r < (unsigned)SORT_KEYS) {
                atomicAdd(S.cnt + r, (uint32_t)R.len);
            } else {
                const int slot = hash_insert(S.hkey, key);
                if (slot >= 0)
                    atomicAdd(S.hcnt + slot, (uint32_t)R.len);
                else
                    fb = 1;
            }
        }
        fb = __shfl_sync(0xffffffffu, fb, R.hidx);
        if (fb && key >= 0) keys[j] = key | FALLBACK_BIT;
    }
}

__global__ void __launch_bounds__(SORT_THREADS) sort_hist_kernel(SortArgs A)
{
    __shared__ SortSmem S;
    const long long n = *A.d_n;
    const long long base = (long long)blockIdx.x * SORT_CHUNK;
    if (base >= n) return;
    const long long ncell = (long long)A.nx * A.ny;
    const int k0 = window_start(A, base, n);
    init_smem(S);
    __syncthreads();
    int keys[SORT_PER_THREAD];
    count_keys(A, S, base, n, k0, keys);
#pragma unroll
    for (int j = 0; j < SORT_PER_THREAD; ++j) {  // warp-uniform
        const Run R = warp_run(keys[j]);
        if (R.head && keys[j] >= 0 && (keys[j] & FALLBACK_BIT))
            atomicAdd(A.count + (keys[j] & ~FALLBACK_BIT), (uint32_t)R.len);
    }
    __syncthreads();
    for (int r = threadIdx.x; r < SORT_KEYS; r += SORT_THREADS) {
        const uint32_t v = S.cnt[r];
        if (v && k0 + r <= ncell) atomicAdd(A.count + k0 + r, v);
    }
    for (int r = threadIdx.x; r < HASH_SLOTS; r += SORT_THREADS)
        if (S.hcnt[r]) atomicAdd(A.count + S.hkey[r], S.hcnt[r]);
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

__global__ void __launch_bounds__(SORT_THREADS, 5) sort_scatter_kernel(SortArgs A)
{
    __shared__ SortSmem S;
    const long long n = *A.d_n;
    const long long base = (long long)blockIdx.x * SORT_CHUNK;
    if (base >= n) return;
    const long long ncell = (long long)A.nx * A.ny;
    const int k0 = window_start(A, base, n);
    init_smem(S);
    __syncthreads();
    int keys[SORT_PER_THREAD];
    count_keys(A, S, base, n, k0, keys);
    __syncthreads();
    // reserve each distinct key's slice of the output once per block
    for (int r = threadIdx.x; r < SORT_KEYS; r += SORT_THREADS) {
        const uint32_t v = S.cnt[r];
        S.base[r] = (v && k0 + r <= ncell) ? atomicAdd(A.cursor + k0 + r, v) : 0u;
        S.cnt[r] = 0u;
    }
    for (int r = threadIdx.x; r < HASH_SLOTS; r += SORT_THREADS) {
        const uint32_t v = S.hcnt[r];
        S.hbase[r] = v ? atomicAdd(A.cursor + S.hkey[r], v) : 0u;
        S.hcnt[r] = 0u;
    }
    __syncthreads();
    // destinations of this thread's particles: one reservation per run ...
#pragma unroll
    for (int j = 0; j < SORT_PER_THREAD; ++j) {  // warp-uniform
        const int key = keys[j];
        const Run R = warp_run(key);
        uint32_t d = 0;
        if (R.head && key >= 0) {
            if (key & FALLBACK_BIT) {
                d = atomicAdd(A.cursor + (key & ~FALLBACK_BIT), (uint32_t)R.len);
            } else if ((unsigned)(key - k0) < (unsigned)SORT_KEYS) {
                const int r = key - k0;
                d = S.base[r] + atomicAdd(S.cnt + r, (uint32_t)R.len);
            } else {
                const int slot = hash_find(S.hkey, key);  // counted in the table in pass 1
                d = S.hbase[slot] + atomicAdd(S.hcnt + slot, (uint32_t)R.len);
            }
        }
        d = __shfl_sync(0xffffffffu, d, R.hidx) + (uint32_t)R.rank;
        keys[j] = key >= 0 ? (int)d : -1;  // n < 2^31
    }
    // ... then the copies, four particles at a time with their loads first
#pragma unroll
    for (int g = 0; g < SORT_PER_THREAD; g += 4) {
        int c[4];
        uint32_t p[4];
        float a[4], b[4], u[4], v[4], z[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const long long i = base + (long long)(g + t) * SORT_THREADS + threadIdx.x;
            if (i < n) {
                c[t] = A.cin[i];
                a[t] = A.oxin[i];
                b[t] = A.oyin[i];
                u[t] = A.vxin[i];
                v[t] = A.vyin[i];
                p[t] = A.pidin[i];
                z[t] = A.vzin ? A.vzin[i] : 0.f;
            }
        }
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const long long i = base + (long long)(g + t) * SORT_THREADS + threadIdx.x;
            if (i >= n || keys[g + t] < 0) continue;
            const long long d = keys[g + t];
            A.cout[d] = c[t];
            A.oxout[d] = a[t];
            A.oyout[d] = b[t];
            A.vxout[d] = u[t];
            A.vyout[d] = v[t];
            A.pidout[d] = p[t];
            if (A.vzin) A.vzout[d] = z[t];
        }
    }
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
