// pic_sort_dev.cuh -- device functions of the counting sort, shared by the
// single-run kernels (pic_sort.cu) and the ensemble kernels
// (pic_ensemble.cu).  The algorithm is described at the top of pic_sort.cu.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

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
    const uint32_t *xin[4];  // optional extra per-particle arrays moved along
    uint32_t *xout[4];       // (all four or none)
    int wkeys, hbits;        // window keys and log2 hash slots in use (0: the maxima)
    long long nslots;        // slots of the destination arrays (scatter bound)
};

// Key geometry of the run a sort block works on: the run's grid and tiles
// and the first key of its range (0 for a single run).  Key key_off + nx*ny
// is the run's bin of empty slots.  mtw, mth: multipliers that divide a
// cell coordinate by tw and th (div_coord); 0 divides directly.
struct KeyGeo {
    int nx, ny, tw, th, ntx, key_off;
    unsigned mtw, mth;
};

// m = floor((2^32 - 1) / d) + 1 gives floor(n / d) = umulhi(n, m) for every
// n < 2^16 and 2 <= d <= 2^16: m = 2^32/d + e with 0 < e <= 1, so n m / 2^32
// exceeds n/d by less than 2^-16 <= 1/d, less than the gap from n/d to the
// next integer.  d = 1 gets 0 (n itself).
__host__ __device__ __forceinline__ unsigned div_magic(int d)
{
    return d > 1 ? 0xFFFFFFFFu / (unsigned)d + 1u : 0u;
}

__host__ __device__ __forceinline__ KeyGeo key_geo(int nx, int ny, int tw, int th, int ntx,
                                                   int key_off)
{
    return KeyGeo{nx, ny, tw, th, ntx, key_off, div_magic(tw), div_magic(th)};
}

__device__ __forceinline__ int div_coord(int n, int d, unsigned m)
{
    return m ? (int)__umulhi((unsigned)n, m) : n / d;
}

// cell_key with the divisions done by multiplication
__device__ __forceinline__ int cell_key(int c, const KeyGeo &G)
{
    const int cx = c & 0xFFFF, cy = c >> 16;
    const int tx = div_coord(cx, G.tw, G.mtw), lx = cx - tx * G.tw;
    const int ty = div_coord(cy, G.th, G.mth), ly = cy - ty * G.th;
    return ((ty * G.ntx + tx) * G.th + ly) * G.tw + lx;
}

__device__ __forceinline__ KeyGeo single_geo(const SortArgs &A)
{
    return key_geo(A.nx, A.ny, A.tw, A.th, A.ntx, 0);
}

constexpr int SORT_THREADS = 256;
constexpr int SORT_PER_THREAD = 8;
constexpr int SORT_CHUNK = SORT_THREADS * SORT_PER_THREAD;
constexpr int SORT_KEYS = 2048;
constexpr int HASH_SLOTS = 1024;  // power of two
constexpr int HASH_PROBES = 8;
constexpr int HASH_EMPTY = -1;
constexpr int FALLBACK_BIT = 1 << 30;  // keys are < 2^30
constexpr uint32_t SORT_NO_SLOT = 0xFFFFFFFFu;  // a destination outside the slots

// Window and table in use by a sort launch: the arrays are sized for the
// maxima, and a launch over dense data (few keys per block) uses a prefix so
// that clearing and walking them costs less than its particles.
struct SortSizes {
    int wk;  // window keys
    int hb;  // log2 of the hash slots
};

__device__ __forceinline__ SortSizes sort_sizes(const SortArgs &A)
{
    return SortSizes{A.wkeys ? A.wkeys : SORT_KEYS, A.hbits ? A.hbits : 10};
}

__device__ __forceinline__ unsigned hash_key(int key, int hb)
{
    return ((unsigned)key * 0x9E3779B1u) >> (32 - hb);  // top hb bits
}

// slot of `key` in the block's table, inserting it if absent; -1 if the
// bounded probe found no room
__device__ __forceinline__ int hash_insert(int *tab_key, int key, int hb)
{
    const unsigned h = hash_key(key, hb);
    for (int p = 0; p < HASH_PROBES; ++p) {
        const int slot = (int)((h + p) & ((1u << hb) - 1));
        const int old = atomicCAS(tab_key + slot, HASH_EMPTY, key);
        if (old == HASH_EMPTY || old == key) return slot;
    }
    return -1;
}

// slot of a key that is already in the table
__device__ __forceinline__ int hash_find(const int *tab_key, int key, int hb)
{
    const unsigned h = hash_key(key, hb);
    for (int p = 0; p < HASH_PROBES; ++p) {
        const int slot = (int)((h + p) & ((1u << hb) - 1));
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
    return G.key_off + cell_key(c, G);
}

// first key of this block's shared-memory window (block-uniform)
__device__ __forceinline__ int window_start(const SortArgs &A, const KeyGeo &G, long long base,
                                            long long end, int wk)
{
    const long long mid = min(base + SORT_CHUNK / 2, end - 1);
    const int c = A.cin[mid];
    int k = G.key_off;
    if (c >= 0 && (c & 0xFFFF) < G.nx && (c >> 16) < G.ny) k += cell_key(c, G);
    return max(0, k - wk / 2);
}

// Shared state of one sort block: dense window counts and the straggler table.
struct SortSmem {
    uint32_t cnt[SORT_KEYS];
    uint32_t base[SORT_KEYS];
    int hkey[HASH_SLOTS];
    uint32_t hcnt[HASH_SLOTS];
    uint32_t hbase[HASH_SLOTS];
};

__device__ __forceinline__ void init_smem(SortSmem &S, SortSizes Z)
{
    for (int r = threadIdx.x; r < Z.wk; r += SORT_THREADS) S.cnt[r] = 0u;
    for (int r = threadIdx.x; r < (1 << Z.hb); r += SORT_THREADS) {
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

// a Run in one word (head bit 0, head lane bits 1-5, length bits 6-11,
// rank bits 12-16), kept from the count to the ranking phase
__device__ __forceinline__ int pack_run(const Run &r)
{
    return (int)r.head | (r.hidx << 1) | (r.len << 6) | (r.rank << 12);
}

__device__ __forceinline__ Run unpack_run(int w)
{
    Run r;
    r.head = w & 1;
    r.hidx = (w >> 1) & 31;
    r.len = (w >> 6) & 63;
    r.rank = (w >> 12) & 31;
    return r;
}

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

// Cells of this thread's particles (-1 past the end), loaded before the
// window setup so that the two loads' latencies overlap.
__device__ __forceinline__ void load_cells(const SortArgs &A, long long base, long long end,
                                           int (&cells)[SORT_PER_THREAD])
{
#pragma unroll
    for (int j = 0; j < SORT_PER_THREAD; ++j) {
        const long long i = base + (long long)j * SORT_THREADS + threadIdx.x;
        cells[j] = (i < end) ? A.cin[i] : -1;
    }
}

// Pass 1 of both kernels: keys of this thread's particles (`keys` holds
// their cells from load_cells on entry), counted in the window or the
// table; a run the table had no room for gets FALLBACK_BIT (on all its
// lanes, so the runs stay the same).  KEEP: each key's run, packed, to
// `runs` for the ranking phase.
template <bool KEEP>
__device__ __forceinline__ void count_keys(const SortArgs &A, const KeyGeo &G, SortSmem &S,
                                           long long base, long long end, int k0, SortSizes Z,
                                           int (&keys)[SORT_PER_THREAD], int (&runs)[SORT_PER_THREAD])
{
#pragma unroll
    for (int j = 0; j < SORT_PER_THREAD; ++j) {
        const long long i = base + (long long)j * SORT_THREADS + threadIdx.x;
        keys[j] = (i < end) ? particle_key(G, A.err, keys[j]) : -1;
    }
#pragma unroll
    for (int j = 0; j < SORT_PER_THREAD; ++j) {  // warp-uniform
        const int key = keys[j];
        const Run R = warp_run(key);
        int fb = 0;
        if (R.head && key >= 0) {
            const unsigned r = (unsigned)(key - k0);
            if (r < (unsigned)Z.wk) {
                atomicAdd(S.cnt + r, (uint32_t)R.len);
            } else {
                const int slot = hash_insert(S.hkey, key, Z.hb);
                if (slot >= 0)
                    atomicAdd(S.hcnt + slot, (uint32_t)R.len);
                else
                    fb = 1;
            }
        }
        const unsigned fbm = __ballot_sync(0xffffffffu, fb);  // heads whose run falls back
        if (fbm && key >= 0 && ((fbm >> R.hidx) & 1u)) keys[j] = key | FALLBACK_BIT;
        if (KEEP) runs[j] = pack_run(R);
    }
}

// Histogram of the keys of particles [base, end) (one sort block).
__device__ __forceinline__ void sort_hist_block(const SortArgs &A, const KeyGeo &G, SortSmem &S,
                                                long long base, long long end)
{
    const SortSizes Z = sort_sizes(A);
    int keys[SORT_PER_THREAD];
    load_cells(A, base, end, keys);
    const int k0 = window_start(A, G, base, end, Z.wk);
    init_smem(S, Z);
    __syncthreads();
    int unused[SORT_PER_THREAD];
    count_keys<false>(A, G, S, base, end, k0, Z, keys, unused);
#pragma unroll
    for (int j = 0; j < SORT_PER_THREAD; ++j) {  // warp-uniform
        // keys the block's table had no room for (rare): counted straight
        // to the global histogram, one atomic per run
        if (!__any_sync(0xffffffffu, keys[j] >= 0 && (keys[j] & FALLBACK_BIT))) continue;
        const Run R = warp_run(keys[j]);
        if (R.head && keys[j] >= 0 && (keys[j] & FALLBACK_BIT))
            atomicAdd(A.count + (keys[j] & ~FALLBACK_BIT), (uint32_t)R.len);
    }
    __syncthreads();
    for (int r = threadIdx.x; r < Z.wk; r += SORT_THREADS) {
        const uint32_t v = S.cnt[r];
        if (v && k0 + r < A.nkeys) atomicAdd(A.count + k0 + r, v);
    }
    for (int r = threadIdx.x; r < (1 << Z.hb); r += SORT_THREADS)
        if (S.hcnt[r]) atomicAdd(A.count + S.hkey[r], S.hcnt[r]);
}

// Shared memory of a scatter block: the counting state with each key's
// first slot in a block-local staging order, and the global destination of
// every staged particle.  Once the destinations are known, the staging
// buffers (up to six fields at a time) take the counting state's place.
// 56 KB: four blocks fill an SM's 228 KB with their 1 KB reserves.
struct ScatterCount {
    SortSmem s;
    uint32_t lbase[SORT_KEYS];
    uint32_t hlbase[HASH_SLOTS];
    uint32_t total;
};
constexpr int STAGE_FIELDS = 6;
struct ScatterSmem {
    union {
        ScatterCount c;
        uint32_t stage[STAGE_FIELDS * SORT_CHUNK];
    };
    uint32_t dst[SORT_CHUNK];
};
static_assert(sizeof(ScatterCount) <= STAGE_FIELDS * SORT_CHUNK * sizeof(uint32_t),
              "the counting state must fit in the staging buffers");
constexpr size_t SCATTER_SMEM = sizeof(ScatterSmem);

// one staging phase: up to six 32-bit fields moved through shared memory
// so that the global stores follow the destination order (consecutive
// threads write consecutive slots of a key's slice); `total` = particles
// staged by the block
template <int NF>
__device__ __forceinline__ void stage_fields(ScatterSmem &S, long long base, long long end,
                                             const int (&lpos)[SORT_PER_THREAD], int total,
                                             const uint32_t *const (&src)[NF], uint32_t *const (&dst)[NF])
{
    static_assert(NF <= STAGE_FIELDS, "staging buffers hold six fields");
    uint32_t *stage = S.stage;
    __syncthreads();  // the previous phase (or the counting state) has left the staging buffers
#pragma unroll
    for (int j = 0; j < SORT_PER_THREAD; ++j) {
        const long long i = base + (long long)j * SORT_THREADS + threadIdx.x;
        if (i < end && lpos[j] >= 0) {
#pragma unroll
            for (int f = 0; f < NF; ++f) stage[f * SORT_CHUNK + lpos[j]] = src[f][i];
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < total; t += SORT_THREADS) {
        const uint32_t d = S.dst[t];
        if (d == SORT_NO_SLOT) continue;
#pragma unroll
        for (int f = 0; f < NF; ++f) dst[f][d] = stage[f * SORT_CHUNK + t];
    }
}

// Scatter of particles [base, end) (one sort block) to their sorted slots.
// Each distinct key reserves its global slice (one global atomic per key and
// block) and a block-local staging range; particles are staged in
// shared memory in slice order and written out with consecutive threads on
// consecutive slots.
__device__ __forceinline__ void sort_scatter_block(const SortArgs &A, const KeyGeo &G,
                                                   ScatterSmem &S, long long base, long long end)
{
    const SortSizes Z = sort_sizes(A);
    int keys[SORT_PER_THREAD];
    load_cells(A, base, end, keys);
    const int k0 = window_start(A, G, base, end, Z.wk);
    ScatterCount &C = S.c;
    init_smem(C.s, Z);
    if (threadIdx.x == 0) C.total = 0u;
    __syncthreads();
    int runs[SORT_PER_THREAD];
    count_keys<true>(A, G, C.s, base, end, k0, Z, keys, runs);
    __syncthreads();
    // reserve each distinct key's slice of the output and of the staging order
    for (int r = threadIdx.x; r < Z.wk; r += SORT_THREADS) {
        const uint32_t v = C.s.cnt[r];
        const bool use = v && k0 + r < A.nkeys;
        C.s.base[r] = use ? atomicAdd(A.cursor + k0 + r, v) : 0u;
        C.lbase[r] = use ? atomicAdd(&C.total, v) : 0u;
        C.s.cnt[r] = 0u;
    }
    for (int r = threadIdx.x; r < (1 << Z.hb); r += SORT_THREADS) {
        const uint32_t v = C.s.hcnt[r];
        C.s.hbase[r] = v ? atomicAdd(A.cursor + C.s.hkey[r], v) : 0u;
        C.hlbase[r] = v ? atomicAdd(&C.total, v) : 0u;
        C.s.hcnt[r] = 0u;
    }
    __syncthreads();
    // destination and staging slot of every particle: one reservation per run
#pragma unroll
    for (int j = 0; j < SORT_PER_THREAD; ++j) {  // warp-uniform
        const int key = keys[j];
        const Run R = unpack_run(runs[j]);
        uint32_t d = 0, l = 0;
        if (R.head && key >= 0) {
            if (key & FALLBACK_BIT) {
                d = atomicAdd(A.cursor + (key & ~FALLBACK_BIT), (uint32_t)R.len);
                l = atomicAdd(&C.total, (uint32_t)R.len);
            } else if ((unsigned)(key - k0) < (unsigned)Z.wk) {
                const int r = key - k0;
                const uint32_t o = atomicAdd(C.s.cnt + r, (uint32_t)R.len);
                d = C.s.base[r] + o;
                l = C.lbase[r] + o;
            } else {
                const int slot = hash_find(C.s.hkey, key, Z.hb);  // counted in the table in pass 1
                const uint32_t o = atomicAdd(C.s.hcnt + slot, (uint32_t)R.len);
                d = C.s.hbase[slot] + o;
                l = C.hlbase[slot] + o;
            }
        }
        d = __shfl_sync(0xffffffffu, d, R.hidx) + (uint32_t)R.rank;
        l = __shfl_sync(0xffffffffu, l, R.hidx) + (uint32_t)R.rank;
        if (key >= 0 && (long long)d >= A.nslots) {  // counts that do not match the particles
            atomicOr(A.err, (unsigned)PIC_DEVERR_SORT);
            d = SORT_NO_SLOT;
        }
        if (key >= 0) S.dst[l] = d;
        keys[j] = key >= 0 ? (int)l : -1;
    }
    __syncthreads();  // the fallback runs' staging reservations are in
    const int total = (int)C.total;  // read before the staging buffers overwrite it
    {
        const uint32_t *const src[6] = {reinterpret_cast<const uint32_t *>(A.cin),
                                        reinterpret_cast<const uint32_t *>(A.oxin),
                                        reinterpret_cast<const uint32_t *>(A.oyin),
                                        reinterpret_cast<const uint32_t *>(A.vxin),
                                        reinterpret_cast<const uint32_t *>(A.vyin), A.pidin};
        uint32_t *const dst[6] = {reinterpret_cast<uint32_t *>(A.cout),
                                  reinterpret_cast<uint32_t *>(A.oxout),
                                  reinterpret_cast<uint32_t *>(A.oyout),
                                  reinterpret_cast<uint32_t *>(A.vxout),
                                  reinterpret_cast<uint32_t *>(A.vyout), A.pidout};
        stage_fields<6>(S, base, end, keys, total, src, dst);
    }
    if (A.vzin) {
        const uint32_t *const src[1] = {reinterpret_cast<const uint32_t *>(A.vzin)};
        uint32_t *const dst[1] = {reinterpret_cast<uint32_t *>(A.vzout)};
        stage_fields<1>(S, base, end, keys, total, src, dst);
    }
    if (A.xin[0]) {
        const uint32_t *const src[4] = {A.xin[0], A.xin[1], A.xin[2], A.xin[3]};
        uint32_t *const dst[4] = {A.xout[0], A.xout[1], A.xout[2], A.xout[3]};
        stage_fields<4>(S, base, end, keys, total, src, dst);
    }
}

}  // namespace pic
