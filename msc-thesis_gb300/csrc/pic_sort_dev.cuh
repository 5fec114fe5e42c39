// pic_sort_dev.cuh -- device functions of the counting sort, shared by the
// single-run kernels (pic_sort.cu) and the ensemble kernels
// (pic_ensemble.cu).  The algorithm is described at the top of pic_sort.cu.
#pragma once
#include <cuda_runtime.h>

#include <climits>
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
    int rows;                // sort by tile row (tw cells per key) instead of by cell
    const uint32_t *xin[4];  // optional extra per-particle arrays moved along
    uint32_t *xout[4];       // (all four or none)
    int wkeys, hbits;        // window keys and log2 hash slots in use (0: the maxima)
    long long nslots;        // slots of the destination arrays (scatter bound)
};

// Key geometry of the run a sort block works on: the run's grid and tiles
// and the first key of its range (0 for a single run).  Key key_off + nx*ny
// is the run's bin of empty slots.  mtw, mth: multipliers that divide a
// cell coordinate by tw and th (div_coord); 0 divides directly.  rows: keys
// are tile rows (tw cells each) rather than cells.
struct KeyGeo {
    int nx, ny, tw, th, ntx, key_off;
    unsigned mtw, mth;
    int rows;
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
                                                   int key_off, int rows = 0)
{
    return KeyGeo{nx, ny, tw, th, ntx, key_off, div_magic(tw), div_magic(th), rows};
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

// Sort key of an on-grid cell c: its tile-major cell index, or with G.rows
// the tile-major index of its row within its tile (cell index / tw).  The
// push only needs a block's particles to stay within its tiles, and
// measured no slower on row-sorted particles; the DSMC pass needs cells.
__device__ __forceinline__ int sort_key(int c, const KeyGeo &G)
{
    const int cx = c & 0xFFFF, cy = c >> 16;
    const int tx = div_coord(cx, G.tw, G.mtw);
    const int ty = div_coord(cy, G.th, G.mth), ly = cy - ty * G.th;
    const int row = (ty * G.ntx + tx) * G.th + ly;
    return G.rows ? row : row * G.tw + (cx - tx * G.tw);
}

__device__ __forceinline__ KeyGeo single_geo(const SortArgs &A)
{
    return key_geo(A.nx, A.ny, A.tw, A.th, A.ntx, 0, A.rows);
}

// Work of a sort block: SORT_CHUNK consecutive particles, thread t owning the
// quad of four consecutive particles base + 4t ... base + 4t + 3, so that a
// warp's 128-bit loads are fully coalesced and a warp holds 128 consecutive
// particles (base is a multiple of 4, so every quad is 16-byte aligned).
constexpr int SORT_THREADS = 256;
constexpr int SORT_PER_THREAD = 4;
constexpr int SORT_CHUNK = SORT_THREADS * SORT_PER_THREAD;
constexpr int SORT_KEYS = 1024;
constexpr int HASH_SLOTS = 512;  // power of two
constexpr int HASH_PROBES = 8;
constexpr int HASH_EMPTY = -1;
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
    return SortSizes{A.wkeys ? A.wkeys : SORT_KEYS, A.hbits ? A.hbits : 9};
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
    return G.key_off + sort_key(c, G);
}

// first key of the shared-memory window of a block over particles
// [base, end) (block-uniform): centred on the middle particle's key
__device__ __forceinline__ int window_start(const SortArgs &A, const KeyGeo &G, long long base,
                                            long long end, int wk)
{
    const long long mid = base + (end - base - 1) / 2;
    const int c = A.cin[mid];
    int k = G.key_off;
    if (c >= 0 && (c & 0xFFFF) < G.nx && (c >> 16) < G.ny) k += sort_key(c, G);
    return max(0, k - wk / 2);
}

// Counting state of one sort block: dense window counts and the straggler
// table.
struct SortSmem {
    uint32_t cnt[SORT_KEYS];
    int hkey[HASH_SLOTS];
    uint32_t hcnt[HASH_SLOTS];
};

__device__ __forceinline__ void init_smem(SortSmem &S, SortSizes Z)
{
    for (int r = threadIdx.x; r < Z.wk; r += SORT_THREADS) S.cnt[r] = 0u;
    for (int r = threadIdx.x; r < (1 << Z.hb); r += SORT_THREADS) {
        S.hkey[r] = HASH_EMPTY;
        S.hcnt[r] = 0u;
    }
}

// first particle of this thread's quad
__device__ __forceinline__ long long quad_start(long long base)
{
    return base + (long long)SORT_PER_THREAD * threadIdx.x;
}

__device__ __forceinline__ void prefetch_l2(const void *p)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// This thread's quad of every field the scatter moves, for the chunk at
// `base`, fetched into L2 ahead of its use by a later iteration of the same
// block.  No registers are held.
__device__ __forceinline__ void prefetch_chunk(const SortArgs &A, long long base, long long end)
{
    const long long q = quad_start(base);
    if (q >= end) return;
    prefetch_l2(A.cin + q);
    prefetch_l2(A.oxin + q);
    prefetch_l2(A.oyin + q);
    prefetch_l2(A.vxin + q);
    prefetch_l2(A.vyin + q);
    prefetch_l2(A.pidin + q);
    if (A.vzin) prefetch_l2(A.vzin + q);
}

// The thread's quad of cells (one 128-bit load); slots at or past `end` get
// INT_MIN (no particle).
__device__ __forceinline__ void load_cells(const SortArgs &A, long long base, long long end,
                                           int (&cells)[SORT_PER_THREAD])
{
    const long long q = quad_start(base);
    int4 c = make_int4(INT_MIN, INT_MIN, INT_MIN, INT_MIN);
    if (q < end) c = *reinterpret_cast<const int4 *>(A.cin + q);
    cells[0] = c.x;
    cells[1] = q + 1 < end ? c.y : INT_MIN;
    cells[2] = q + 2 < end ? c.z : INT_MIN;
    cells[3] = q + 3 < end ? c.w : INT_MIN;
}

// Runs of equal keys over the warp's 128 consecutive particles (lane l holds
// positions 4l .. 4l + 3), from shuffles and ballots: every run is counted
// by the lane holding its first particle, with its full length, so that a
// run costs one atomic whatever the lanes it spans.
struct QuadRuns {
    unsigned head;  // bit j: particle j starts a run
    int len[SORT_PER_THREAD];  // run length at each head
    int lin;        // lane holding the head of the run that enters this lane
    int pin;        // that head's position in the warp (0..127)
};

__device__ __forceinline__ QuadRuns quad_runs(const int (&k)[SORT_PER_THREAD])
{
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int prev = __shfl_up_sync(full, k[3], 1);
    QuadRuns R;
    R.head = (lane == 0 || k[0] != prev ? 1u : 0u) | (k[1] != k[0] ? 2u : 0u) |
             (k[2] != k[1] ? 4u : 0u) | (k[3] != k[2] ? 8u : 0u);
    const unsigned lanes = __ballot_sync(full, R.head != 0u);  // lanes holding a head (lane 0 does)
    const int firstj = __ffs(R.head) - 1;                       // -1: no head
    const int lastj = 31 - __clz(R.head);                       // -1: no head
    // first head after this lane: its position, or 128
    const unsigned later = lanes & ~(0xffffffffu >> (31 - lane));
    const int fl = later ? __ffs(later) - 1 : 0;
    const int ffj = __shfl_sync(full, firstj, fl);
    const int next_pos = later ? 4 * fl + ffj : 4 * 32;
    // the run holding this lane's first particle, when it starts in an
    // earlier lane: at the last head of the nearest earlier lane with one
    const unsigned before = lanes & ((1u << lane) - 1u);
    R.lin = before ? 31 - __clz(before) : 0;
    R.pin = 4 * R.lin + __shfl_sync(full, lastj, R.lin);
#pragma unroll
    for (int j = 0; j < SORT_PER_THREAD; ++j) {
        int nxt = next_pos;
#pragma unroll
        for (int i = SORT_PER_THREAD - 1; i > j; --i)
            if (R.head & (1u << i)) nxt = 4 * lane + i;
        R.len[j] = nxt - (4 * lane + j);
    }
    return R;
}

// Pass 1 of the scatter: the keys of the thread's quad (`keys` holds its
// cells on entry; INT_MIN becomes -1) and one shared atomic per run of equal
// keys (quad_runs), in the window or the table; every particle gets its rank
// among the block's particles of its key: the run's atomic result plus its
// position in the run.  A run the table has no room for falls back: its
// particles are marked in `fbm` and take their slots one by one after the
// reservations.
__device__ __forceinline__ void count_keys(const SortArgs &A, const KeyGeo &G, SortSmem &S,
                                           int k0, SortSizes Z, int (&keys)[SORT_PER_THREAD],
                                           uint32_t (&rank)[SORT_PER_THREAD], unsigned &fbm)
{
#pragma unroll
    for (int j = 0; j < SORT_PER_THREAD; ++j)
        keys[j] = keys[j] == INT_MIN ? -1 : particle_key(G, A.err, keys[j]);
    const QuadRuns R = quad_runs(keys);
    uint32_t base[SORT_PER_THREAD];
    bool fbh[SORT_PER_THREAD];
#pragma unroll
    for (int j = 0; j < SORT_PER_THREAD; ++j) {
        base[j] = 0u;
        fbh[j] = false;
        const int key = keys[j];
        if (((R.head >> j) & 1u) && key >= 0) {
            const unsigned w = (unsigned)(key - k0);
            if (w < (unsigned)Z.wk) {
                base[j] = atomicAdd(S.cnt + w, (uint32_t)R.len[j]);
            } else {
                const int slot = hash_insert(S.hkey, key, Z.hb);
                if (slot >= 0) {
                    base[j] = atomicAdd(S.hcnt + slot, (uint32_t)R.len[j]);
                } else {
                    fbh[j] = true;
                }
            }
        }
    }
    fbm = 0u;
    // the run entering this lane takes its base and fallback flag from the
    // lane holding its head (that lane's last head)
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned hb = R.head;
    const uint32_t lastbase = (hb & 8u) ? base[3] : (hb & 4u) ? base[2] : (hb & 2u) ? base[1] : base[0];
    const bool lastfb = (hb & 8u) ? fbh[3] : (hb & 4u) ? fbh[2] : (hb & 2u) ? fbh[1] : fbh[0];
    const uint32_t in_base = __shfl_sync(full, lastbase, R.lin);
    const bool in_fb = __shfl_sync(full, lastfb ? 1 : 0, R.lin) != 0;
    uint32_t r = in_base + (uint32_t)(4 * lane - R.pin);
    bool fb = in_fb;
#pragma unroll
    for (int j = 0; j < SORT_PER_THREAD; ++j) {
        if ((hb >> j) & 1u) {
            r = base[j];
            fb = fbh[j];
        } else if (j > 0) {
            r += 1u;
        }
        rank[j] = r;
        if (fb && keys[j] >= 0) fbm |= 1u << j;
    }
}

// Histogram of the keys of particles [base, end) (one block of HIST_BLOCK
// consecutive particles): each thread counts the HIST_SEG consecutive
// particles from base + HIST_SEG t, one atomic per run of equal keys, into a
// shared window of wk keys around the block's middle key, or straight into
// the global histogram outside it.  Particles sorted by key a few steps ago
// make long runs: about one atomic per thread.  cnt: SORT_KEYS entries.
constexpr int HIST_SEG = 16;
constexpr int HIST_BLOCK = HIST_SEG * SORT_THREADS;

__device__ __forceinline__ void sort_hist_segments(const SortArgs &A, const KeyGeo &G, uint32_t *cnt,
                                                   long long base, long long end)
{
    const int wk = sort_sizes(A).wk;
    const long long s0 = base + (long long)HIST_SEG * threadIdx.x;
    int c[HIST_SEG];
#pragma unroll
    for (int u = 0; u < HIST_SEG / 4; ++u) {
        const long long q = s0 + 4 * u;
        int4 v = make_int4(INT_MIN, INT_MIN, INT_MIN, INT_MIN);
        if (q < end) v = __ldg(reinterpret_cast<const int4 *>(A.cin + q));
        c[4 * u] = v.x;
        c[4 * u + 1] = q + 1 < end ? v.y : INT_MIN;
        c[4 * u + 2] = q + 2 < end ? v.z : INT_MIN;
        c[4 * u + 3] = q + 3 < end ? v.w : INT_MIN;
    }
    const int k0 = window_start(A, G, base, min(end, base + (long long)HIST_BLOCK), wk);
    for (int r = threadIdx.x; r < wk; r += SORT_THREADS) cnt[r] = 0u;
    __syncthreads();
    int cur = -1;  // key of the open run (-1: none)
    uint32_t run = 0u;
    auto flush = [&]() {
        if (cur < 0) return;
        const unsigned w = (unsigned)(cur - k0);
        if (w < (unsigned)wk)
            atomicAdd(cnt + w, run);
        else
            atomicAdd(A.count + cur, run);
    };
#pragma unroll
    for (int j = 0; j < HIST_SEG; ++j) {
        const int key = c[j] == INT_MIN ? -1 : particle_key(G, A.err, c[j]);
        if (key != cur) {
            flush();
            cur = key;
            run = 0u;
        }
        ++run;
    }
    flush();
    __syncthreads();
    for (int r = threadIdx.x; r < wk; r += SORT_THREADS) {
        const uint32_t v = cnt[r];
        if (v && k0 + r < A.nkeys) atomicAdd(A.count + k0 + r, v);
    }
}

// Shared memory of a scatter block: the counting state with each key's
// first global slot (gb) and first block-local staging slot (lb), later
// replaced by the staging records.  A record is one particle's 32 bytes,
// two 16-byte chunks {cell, ox, oy, vx} {vy, pid, destination, vz}; the
// second staging pass (the optional extra arrays) reuses the first chunk.
struct ScatterCount {
    SortSmem s;
    uint32_t gb[SORT_KEYS];
    uint32_t lb[SORT_KEYS];
    uint32_t hgb[HASH_SLOTS];
    uint32_t hlb[HASH_SLOTS];
};
struct ScatterSmem {
    union {
        ScatterCount c;
        uint4 rec[2 * SORT_CHUNK];
    };
    uint32_t total;  // particles staged by the block
};
static_assert(sizeof(ScatterCount) <= sizeof(uint4) * 2 * SORT_CHUNK,
              "the counting state must fit in the staging records");
constexpr size_t SCATTER_SMEM = sizeof(ScatterSmem);

// Chunk c of staging record l: record l sits in 128-byte row l >> 2 at
// chunk position 2 (l & 3) + c, XOR-swizzled by the row's low three bits.
// Eight lanes whose records are four apart (particles four apart in one
// cell) then write eight rows at eight distinct positions, and eight lanes
// reading consecutive records read two rows at positions of opposite
// parity: no bank conflicts either way.
__device__ __forceinline__ uint4 *rec_chunk(uint4 *rec, uint32_t l, int c)
{
    const uint32_t row = l >> 2;
    const uint32_t p = (((l & 3u) << 1) | (uint32_t)c) ^ (row & 7u);
    return rec + row * 8u + p;
}

// Scatter of particles [base, end) (one sort block) to their sorted slots.
// Every field of the thread's quad is loaded first, so that those loads'
// latency overlaps the counting.  Each distinct key reserves its global
// slice (one global atomic per key and block) and a block-local staging
// range; the particles are staged in shared memory in slice order and
// written out with consecutive threads on consecutive slots.
__device__ __forceinline__ void sort_scatter_block(const SortArgs &A, const KeyGeo &G,
                                                   ScatterSmem &S, long long base, long long end)
{
    const SortSizes Z = sort_sizes(A);
    const long long q = quad_start(base);
    const bool live = q < end;
    int keys[SORT_PER_THREAD];
    load_cells(A, base, end, keys);
    const int cs[SORT_PER_THREAD] = {keys[0], keys[1], keys[2], keys[3]};
    float4 x4 = make_float4(0.f, 0.f, 0.f, 0.f), y4 = x4, u4 = x4, v4 = x4, z4 = x4;
    uint4 i4 = make_uint4(0u, 0u, 0u, 0u);
    if (live) {
        x4 = *reinterpret_cast<const float4 *>(A.oxin + q);
        y4 = *reinterpret_cast<const float4 *>(A.oyin + q);
        u4 = *reinterpret_cast<const float4 *>(A.vxin + q);
        v4 = *reinterpret_cast<const float4 *>(A.vyin + q);
        i4 = *reinterpret_cast<const uint4 *>(A.pidin + q);
        if (A.vzin) z4 = *reinterpret_cast<const float4 *>(A.vzin + q);
    }
    const int k0 = window_start(A, G, base, min(end, base + (long long)SORT_CHUNK), Z.wk);
    ScatterCount &C = S.c;
    init_smem(C.s, Z);
    if (threadIdx.x == 0) S.total = 0u;
    __syncthreads();
    uint32_t rank[SORT_PER_THREAD];
    unsigned fbm;
    count_keys(A, G, C.s, k0, Z, keys, rank, fbm);
    __syncthreads();
    // reserve each distinct key's slice of the output and of the staging order
    for (int r = threadIdx.x; r < Z.wk; r += SORT_THREADS) {
        const uint32_t v = C.s.cnt[r];
        const bool use = v && k0 + r < A.nkeys;
        C.gb[r] = use ? atomicAdd(A.cursor + k0 + r, v) : 0u;
        C.lb[r] = use ? atomicAdd(&S.total, v) : 0u;
    }
    for (int r = threadIdx.x; r < (1 << Z.hb); r += SORT_THREADS) {
        const uint32_t v = C.s.hcnt[r];
        C.hgb[r] = v ? atomicAdd(A.cursor + C.s.hkey[r], v) : 0u;
        C.hlb[r] = v ? atomicAdd(&S.total, v) : 0u;
    }
    __syncthreads();
    // destination and staging slot of every particle
    uint32_t dst[SORT_PER_THREAD], stg[SORT_PER_THREAD];
#pragma unroll
    for (int j = 0; j < SORT_PER_THREAD; ++j) {
        const int key = keys[j];
        uint32_t d = SORT_NO_SLOT, l = SORT_NO_SLOT;
        if (key >= 0) {
            if (fbm & (1u << j)) {  // a run the table had no room for (rare)
                d = atomicAdd(A.cursor + key, 1u);
                l = atomicAdd(&S.total, 1u);
            } else if ((unsigned)(key - k0) < (unsigned)Z.wk) {
                const int w = key - k0;
                d = C.gb[w] + rank[j];
                l = C.lb[w] + rank[j];
            } else {
                const int slot = hash_find(C.s.hkey, key, Z.hb);  // counted in the table in pass 1
                d = C.hgb[slot] + rank[j];
                l = C.hlb[slot] + rank[j];
            }
            if ((long long)d >= A.nslots) {  // counts that do not match the particles
                atomicOr(A.err, (unsigned)PIC_DEVERR_SORT);
                d = SORT_NO_SLOT;
            }
        }
        dst[j] = d;
        stg[j] = l;
    }
    __syncthreads();  // every thread has read the reservations and taken its slots
    const uint32_t total = S.total;
    {
        const float xs[4] = {x4.x, x4.y, x4.z, x4.w}, ys[4] = {y4.x, y4.y, y4.z, y4.w};
        const float us[4] = {u4.x, u4.y, u4.z, u4.w}, vs[4] = {v4.x, v4.y, v4.z, v4.w};
        const float zs[4] = {z4.x, z4.y, z4.z, z4.w};
        const uint32_t is[4] = {i4.x, i4.y, i4.z, i4.w};
#pragma unroll
        for (int j = 0; j < SORT_PER_THREAD; ++j) {
            if (stg[j] == SORT_NO_SLOT) continue;
            *rec_chunk(S.rec, stg[j], 0) = make_uint4((uint32_t)cs[j], __float_as_uint(xs[j]),
                                                      __float_as_uint(ys[j]), __float_as_uint(us[j]));
            *rec_chunk(S.rec, stg[j], 1) = make_uint4(__float_as_uint(vs[j]), is[j], dst[j],
                                                      __float_as_uint(zs[j]));
        }
    }
    __syncthreads();
    // store: consecutive threads take consecutive staged records, so the
    // stores of one key's slice are consecutive slots
    for (uint32_t t = threadIdx.x; t < total; t += SORT_THREADS) {
        const uint4 a = *rec_chunk(S.rec, t, 0);
        const uint4 b = *rec_chunk(S.rec, t, 1);
        const uint32_t d = b.z;
        if (d == SORT_NO_SLOT) continue;
        A.cout[d] = (int32_t)a.x;
        A.oxout[d] = __uint_as_float(a.y);
        A.oyout[d] = __uint_as_float(a.z);
        A.vxout[d] = __uint_as_float(a.w);
        A.vyout[d] = __uint_as_float(b.x);
        A.pidout[d] = b.y;
        if (A.vzin) A.vzout[d] = __uint_as_float(b.w);
    }
    if (!A.xin[0]) return;
    // the four extra arrays, through the first chunk of the same records
    __syncthreads();
    if (live) {
        const uint4 e0 = *reinterpret_cast<const uint4 *>(A.xin[0] + q);
        const uint4 e1 = *reinterpret_cast<const uint4 *>(A.xin[1] + q);
        const uint4 e2 = *reinterpret_cast<const uint4 *>(A.xin[2] + q);
        const uint4 e3 = *reinterpret_cast<const uint4 *>(A.xin[3] + q);
        const uint32_t a0[4] = {e0.x, e0.y, e0.z, e0.w}, a1[4] = {e1.x, e1.y, e1.z, e1.w};
        const uint32_t a2[4] = {e2.x, e2.y, e2.z, e2.w}, a3[4] = {e3.x, e3.y, e3.z, e3.w};
#pragma unroll
        for (int j = 0; j < SORT_PER_THREAD; ++j) {
            if (stg[j] == SORT_NO_SLOT) continue;
            *rec_chunk(S.rec, stg[j], 0) = make_uint4(a0[j], a1[j], a2[j], a3[j]);
        }
    }
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < total; t += SORT_THREADS) {
        const uint4 a = *rec_chunk(S.rec, t, 0);
        const uint32_t d = rec_chunk(S.rec, t, 1)->z;
        if (d == SORT_NO_SLOT) continue;
        A.xout[0][d] = a.x;
        A.xout[1][d] = a.y;
        A.xout[2][d] = a.z;
        A.xout[3][d] = a.w;
    }
}

}  // namespace pic
