// pic_sort_dev.cuh -- device functions of the counting sort, shared by the
// single-run kernels (pic_sort.cu) and the ensemble kernels
// (pic_ensemble.cu).  The algorithm is described at the top of pic_sort.cu.
#pragma once
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
    long long nkeys;  // keys of the whole key space (cells + empty bins)
    unsigned int *err;
};

// Key geometry of the run a sort block works on: the run's grid and tiles
// and the first key of its range (0 for a single run).  Key key_off + nx*ny
// is the run's bin of empty slots.
struct KeyGeo {
    int nx, ny, tw, th, ntx, key_off;
};

__device__ __forceinline__ KeyGeo single_geo(const SortArgs &A)
{
    return KeyGeo{A.nx, A.ny, A.tw, A.th, A.ntx, 0};
}

constexpr int SORT_THREADS = 256;
constexpr int SORT_PER_THREAD = 8;
constexpr int SORT_CHUNK = SORT_THREADS * SORT_PER_THREAD;
constexpr int SORT_KEYS = 2048;
constexpr int HASH_SLOTS = 1024;  // power of two
constexpr int HASH_PROBES = 8;
constexpr int HASH_EMPTY = -1;
constexpr int FALLBACK_BIT = 1 << 30;  // keys are < 2^30

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

// Key of a particle with cell c.  Empty slots (cell < 0) get the run's
// empty key so that they sort to the end of the run and keep their slot
// count; a corrupt cell is flagged and treated the same way.
__device__ __forceinline__ int particle_key(const KeyGeo &G, unsigned int *err, int c)
{
    const int empty = G.key_off + G.nx * G.ny;
    if (c < 0) return empty;
    if ((c & 0xFFFF) >= G.nx || (c >> 16) >= G.ny) {
        atomicOr(err, (unsigned)PIC_DEVERR_CELL);
        return empty;
    }
    return G.key_off + cell_key(c, G.tw, G.th, G.ntx);
}

// first key of this block's shared-memory window (block-uniform)
__device__ __forceinline__ int window_start(const SortArgs &A, const KeyGeo &G, long long base,
                                            long long end)
{
    const long long mid = min(base + SORT_CHUNK / 2, end - 1);
    const int c = A.cin[mid];
    int k = G.key_off;
    if (c >= 0 && (c & 0xFFFF) < G.nx && (c >> 16) < G.ny) k += cell_key(c, G.tw, G.th, G.ntx);
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
__device__ __forceinline__ void count_keys(const SortArgs &A, const KeyGeo &G, SortSmem &S,
                                           long long base, long long end, int k0,
                                           int (&keys)[SORT_PER_THREAD])
{
#pragma unroll
    for (int j = 0; j < SORT_PER_THREAD; ++j) {
        const long long i = base + (long long)j * SORT_THREADS + threadIdx.x;
        keys[j] = (i < end) ? particle_key(G, A.err, A.cin[i]) : -1;
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

// Histogram of the keys of particles [base, end) (one sort block).
__device__ __forceinline__ void sort_hist_block(const SortArgs &A, const KeyGeo &G, SortSmem &S,
                                                long long base, long long end)
{
    const int k0 = window_start(A, G, base, end);
    init_smem(S);
    __syncthreads();
    int keys[SORT_PER_THREAD];
    count_keys(A, G, S, base, end, k0, keys);
#pragma unroll
    for (int j = 0; j < SORT_PER_THREAD; ++j) {  // warp-uniform
        const Run R = warp_run(keys[j]);
        if (R.head && keys[j] >= 0 && (keys[j] & FALLBACK_BIT))
            atomicAdd(A.count + (keys[j] & ~FALLBACK_BIT), (uint32_t)R.len);
    }
    __syncthreads();
    for (int r = threadIdx.x; r < SORT_KEYS; r += SORT_THREADS) {
        const uint32_t v = S.cnt[r];
        if (v && k0 + r < A.nkeys) atomicAdd(A.count + k0 + r, v);
    }
    for (int r = threadIdx.x; r < HASH_SLOTS; r += SORT_THREADS)
        if (S.hcnt[r]) atomicAdd(A.count + S.hkey[r], S.hcnt[r]);
}

// Scatter of particles [base, end) (one sort block) to their sorted slots.
__device__ __forceinline__ void sort_scatter_block(const SortArgs &A, const KeyGeo &G, SortSmem &S,
                                                   long long base, long long end)
{
    const int k0 = window_start(A, G, base, end);
    init_smem(S);
    __syncthreads();
    int keys[SORT_PER_THREAD];
    count_keys(A, G, S, base, end, k0, keys);
    __syncthreads();
    // reserve each distinct key's slice of the output once per block
    for (int r = threadIdx.x; r < SORT_KEYS; r += SORT_THREADS) {
        const uint32_t v = S.cnt[r];
        S.base[r] = (v && k0 + r < A.nkeys) ? atomicAdd(A.cursor + k0 + r, v) : 0u;
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
            if (i < end) {
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
            if (i >= end || keys[g + t] < 0) continue;
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

}  // namespace pic
