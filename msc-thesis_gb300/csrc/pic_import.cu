// pic_import.cu -- sorting particles that arrive in arbitrary order.
//
// The periodic counting sort (pic_sort.cu) relies on the previous order:
// a block's keys fall in a short range.  After an import (host arrays,
// a random load, a state file) the order is arbitrary, and that sort
// degenerates to one global atomic and one scattered store per field and
// particle.  Here the cell keys are sorted as (key, slot) pairs with the
// CUDA toolkit's radix sort (CUB, a library sort of 32-bit pairs over the
// key's significant bits only) and the particle fields then follow in key
// order: as one 32-byte record per particle fetched with a single sector
// read, or field by field when memory for the records is short.  Runs once
// per import, never in the step.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include <cub/device/device_radix_sort.cuh>

#include "pic_ensemble.cuh"
#include "pic_internal.cuh"
#include "pic_sort_dev.cuh"

namespace pic {

__global__ void import_keys_kernel(const int32_t *__restrict__ cell, long long n, KeyGeo G,
                                   unsigned *err, uint32_t *__restrict__ keys,
                                   uint32_t *__restrict__ idx)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        keys[i] = (uint32_t)particle_key(G, err, cell[i]);
        idx[i] = (uint32_t)i;
    }
}

// ensemble: every slot of every run, keys in the shared key space
__global__ void import_keys_ens_kernel(const int32_t *__restrict__ cell,
                                       const SegBlock *__restrict__ blk,
                                       const EnsRun *__restrict__ runs, unsigned *err,
                                       uint32_t *__restrict__ keys, uint32_t *__restrict__ idx)
{
    const SegBlock b = blk[blockIdx.x];
    const EnsRun &R = runs[b.run];
    const KeyGeo G = key_geo(R.nx, R.ny, R.tw, R.th, R.ntx, R.key_off);
    for (long long i = b.base + threadIdx.x; i < b.base + b.count; i += blockDim.x) {
        keys[i] = (uint32_t)particle_key(G, err, cell[i]);
        idx[i] = (uint32_t)i;
    }
}

struct Fields {
    const uint32_t *in[7];
    uint32_t *out[7];
    int nf;
};

// out_f[i] = in_f[src[i]]
__global__ void import_gather_kernel(Fields F, const uint32_t *__restrict__ src, long long n)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t j = src[i];
#pragma unroll
        for (int f = 0; f < 7; ++f)
            if (f < F.nf) F.out[f][i] = F.in[f][j];
    }
}

// Keys and slots as above, and every field of the slot packed into one
// 32-byte record {cell, ox, oy, vx}, {vy, pid, vz, 0}: after the sort the
// permuted read of a particle touches one DRAM sector instead of one per
// field (vz may be absent).
__global__ void import_pack_kernel(Fields F, long long n, KeyGeo G, unsigned *err,
                                   uint32_t *__restrict__ keys, uint32_t *__restrict__ idx,
                                   uint4 *__restrict__ rec)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t c = F.in[0][i];
        keys[i] = (uint32_t)particle_key(G, err, (int)c);
        idx[i] = (uint32_t)i;
        rec[2 * i] = make_uint4(c, F.in[1][i], F.in[2][i], F.in[3][i]);
        rec[2 * i + 1] = make_uint4(F.in[4][i], F.in[5][i], F.nf > 6 ? F.in[6][i] : 0u, 0u);
    }
}

// The records alone (the ensemble's keys come from its own work table).
__global__ void import_pack_fields_kernel(Fields F, long long n, uint4 *__restrict__ rec)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        rec[2 * i] = make_uint4(F.in[0][i], F.in[1][i], F.in[2][i], F.in[3][i]);
        rec[2 * i + 1] = make_uint4(F.in[4][i], F.in[5][i], F.nf > 6 ? F.in[6][i] : 0u, 0u);
    }
}

// out_f[i] = field f of record src[i]
__global__ void import_unpack_kernel(Fields F, const uint4 *__restrict__ rec,
                                     const uint32_t *__restrict__ src, long long n)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const size_t j = src[i];
        const uint4 a = rec[2 * j], b = rec[2 * j + 1];
        F.out[0][i] = a.x;
        F.out[1][i] = a.y;
        F.out[2][i] = a.z;
        F.out[3][i] = a.w;
        F.out[4][i] = b.x;
        F.out[5][i] = b.y;
        if (F.nf > 6) F.out[6][i] = b.z;
    }
}

namespace {

int key_bits(long long nkeys)
{
    int b = 1;
    while ((1ll << b) < nkeys) ++b;
    return b;
}

// (key, slot) radix sort in `scratch` (4 arrays of n words) plus CUB's
// temporary storage (grown on demand in *temp / *temp_bytes)
pic_status radix_pairs(uint32_t *scratch, long long n, int bits, void **temp, size_t *temp_bytes,
                       cudaStream_t st, const uint32_t **sorted_idx)
{
    uint32_t *k0 = scratch, *k1 = scratch + n, *v0 = scratch + 2 * n, *v1 = scratch + 3 * n;
    cub::DoubleBuffer<uint32_t> keys(k0, k1), vals(v0, v1);
    size_t need = 0;
    PIC_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, need, keys, vals, (int)n, 0, bits, st));
    if (need > *temp_bytes) {
        if (*temp) cudaFree(*temp);
        *temp = nullptr;
        *temp_bytes = 0;
        PIC_CUDA(cudaMalloc(temp, need));
        *temp_bytes = need;
    }
    PIC_CUDA(cub::DeviceRadixSort::SortPairs(*temp, need, keys, vals, (int)n, 0, bits, st));
    *sorted_idx = vals.Current();
    return PIC_OK;
}

}  // namespace

// Species s of a handle, live in buffer 0 in arbitrary order -> key order,
// with the chunk anchors.  The fields travel as packed records when the
// stage can hold them (48 bytes per slot) and land back in buffer 0
// (*in_buffer0 = true); else each field is gathered on its own into buffer 1
// (16 bytes per slot) and the caller copies back.
pic_status import_sort(pic_handle *h, int s, bool *in_buffer0)
{
    *in_buffer0 = false;
    SpeciesBuf &B = h->sp[s];
    const long long n = B.cap;  // padding slots (cell -1) sort to the end
    if (!n) return PIC_OK;
    if (n >= (1ll << 31)) {
        set_error("import sort: more than 2^31 slots");
        return PIC_ERR_INVALID_ARG;
    }
    const Geometry &g = h->g;
    const bool ready = B.records_ready;  // keys, slots and records written by the conversion
    B.records_ready = false;
    const bool packed = ready || stage_fits(h, (size_t)n * 48);
    if (!ready) PIC_TRY(ensure_stage(h, (size_t)n * (packed ? 48 : 16)));
    uint32_t *scratch = (uint32_t *)h->stage;
    uint4 *rec = reinterpret_cast<uint4 *>(scratch + 4 * n);
    const KeyGeo G = key_geo(g.nx, g.ny, g.tw, g.th, g.ntx, 0);
    Fields F;
    memset(&F, 0, sizeof F);
    const void *in[7] = {B.cell[0], B.ox[0], B.oy[0], B.vx[0], B.vy[0], B.pid[0], B.vz[0]};
    const int ob = packed ? 0 : 1;
    void *out[7] = {B.cell[ob], B.ox[ob], B.oy[ob], B.vx[ob], B.vy[ob], B.pid[ob], B.vz[ob]};
    F.nf = B.vz[0] ? 7 : 6;
    for (int f = 0; f < F.nf; ++f) {
        F.in[f] = (const uint32_t *)in[f];
        F.out[f] = (uint32_t *)out[f];
    }
    if (ready) {
    } else if (packed) {
        import_pack_kernel<<<grid_for(n, 256), 256, 0, h->stream>>>(F, n, G, &h->dev->err, scratch,
                                                                    scratch + 2 * n, rec);
    } else {
        import_keys_kernel<<<grid_for(n, 256), 256, 0, h->stream>>>(B.cell[0], n, G, &h->dev->err,
                                                                    scratch, scratch + 2 * n);
    }
    PIC_CUDA(cudaGetLastError());
    const uint32_t *idx = nullptr;
    PIC_TRY(radix_pairs(scratch, n, key_bits((long long)g.nx * g.ny + 1), &h->cub_temp,
                        &h->cub_temp_bytes, h->stream, &idx));
    if (packed)
        import_unpack_kernel<<<grid_for(n, 256), 256, 0, h->stream>>>(F, rec, idx, n);
    else
        import_gather_kernel<<<grid_for(n, 256), 256, 0, h->stream>>>(F, idx, n);
    PIC_CUDA(cudaGetLastError());
    *in_buffer0 = packed;
    return launch_anchors(h, s, ob);
}

// Page-locked host arrays of species s (n live particles of its cap slots)
// into buffer 1, in key order within each of IMPORT_PARTS slot ranges: the
// conversion kernel reads range k over the link on the handle's stream
// while range k - 1 is radix-sorted and unpacked on the copy stream, so
// that only the last range's sort follows the transfer.  Each range holds
// particles of the whole grid at an eighth of the density, where a push
// chunk would span eight tiles, so the caller then runs one counting sort
// from buffer 1 into buffer 0: cheap on such data, whose every block of
// particles spans a few cells of one range.
// Conversion blocks of a range import: four 256-thread blocks per SM keep
// enough loads in flight for the link and leave the SMs' remaining threads
// to the previous range's sort on the copy stream (2048^2 x 32 ppc, the
// one-call run of 20 steps: 70.4 ms against 70.7, 71.0-71.8, 74.7 and
// 72.8 ms with 3, 2, 0.5 and 8 blocks per SM, and 72.8 ms for the
// whole-array import)
static int import_blocks() { return 4 * device_sms(); }

pic_status import_records_in_parts(pic_handle *h, int s, long long n, const double *x_dev,
                                   const double *y_dev, const double *vx_dev,
                                   const double *vy_dev, const double *vz_dev)
{
    SpeciesBuf &B = h->sp[s];
    const long long cap = B.cap;
    if (cap >= (1ll << 31)) {
        set_error("import sort: more than 2^31 slots");
        return PIC_ERR_INVALID_ARG;
    }
    PIC_TRY(ensure_copy_stream(h));
    const Geometry &g = h->g;
    const int bits = key_bits((long long)g.nx * g.ny + 1);
    uint32_t *scratch = (uint32_t *)h->stage;
    const uint4 *rec = reinterpret_cast<const uint4 *>(scratch + 4 * cap);
    long long bnd[IMPORT_PARTS + 1];
    for (int k = 0; k < IMPORT_PARTS; ++k) bnd[k] = ((cap * k / IMPORT_PARTS) + 3) & ~3ll;
    bnd[IMPORT_PARTS] = cap;
    // CUB's temporary storage for the largest range, allocated before the
    // first range is converted (an allocation would wait for the device)
    size_t need = 0;
    for (int k = 0; k < IMPORT_PARTS; ++k) {
        cub::DoubleBuffer<uint32_t> kk(scratch, scratch + cap), vv(scratch + 2 * cap, scratch + 3 * cap);
        size_t b = 0;
        PIC_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, b, kk, vv, (int)(bnd[k + 1] - bnd[k]), 0,
                                                 bits, h->copy_stream));
        need = std::max(need, b);
    }
    if (need > h->cub_temp_bytes) {
        if (h->cub_temp) cudaFree(h->cub_temp);
        h->cub_temp = nullptr;
        h->cub_temp_bytes = 0;
        PIC_CUDA(cudaMalloc(&h->cub_temp, need));
        h->cub_temp_bytes = need;
    }
    void *out[7] = {B.cell[1], B.ox[1], B.oy[1], B.vx[1], B.vy[1], B.pid[1], B.vz[1]};
    const int nf = B.vz[1] ? 7 : 6;
    for (int k = 0; k < IMPORT_PARTS; ++k) {
        const long long lo = bnd[k], m = bnd[k + 1] - bnd[k];
        if (m <= 0) continue;
        PIC_TRY(launch_from_global_records_range(h, s, n, lo, lo + m, x_dev, y_dev, vx_dev, vy_dev,
                                                 vz_dev, import_blocks()));
        PIC_CUDA(cudaEventRecord(h->field_ready[k], h->stream));
        PIC_CUDA(cudaStreamWaitEvent(h->copy_stream, h->field_ready[k], 0));
        cub::DoubleBuffer<uint32_t> keys(scratch + lo, scratch + cap + lo),
            vals(scratch + 2 * cap + lo, scratch + 3 * cap + lo);
        size_t tb = h->cub_temp_bytes;
        PIC_CUDA(cub::DeviceRadixSort::SortPairs(h->cub_temp, tb, keys, vals, (int)m, 0, bits,
                                                 h->copy_stream));
        Fields F;
        memset(&F, 0, sizeof F);
        F.nf = nf;
        for (int f = 0; f < nf; ++f) F.out[f] = (uint32_t *)out[f] + lo;
        import_unpack_kernel<<<grid_for(m, 256), 256, 0, h->copy_stream>>>(F, rec, vals.Current(), m);
        PIC_CUDA(cudaGetLastError());
    }
    PIC_CUDA(cudaEventRecord(h->copies_done, h->copy_stream));
    PIC_CUDA(cudaStreamWaitEvent(h->stream, h->copies_done, 0));
    B.presorted = true;
    return PIC_OK;
}

// Every run of an ensemble: buffer 0 in arbitrary order -> buffer 1 in key
// order (anchors are the caller's).  `scratch` holds 16 bytes per slot, or
// 48 with `packed` (the fields then travel as 32-byte records, as above).
pic_status ens_import_sort(pic_ensemble *E, uint32_t *scratch, bool packed, void **temp,
                           size_t *temp_bytes)
{
    const long long n = E->nslots;
    if (n >= (1ll << 31)) {
        set_error("import sort: more than 2^31 slots");
        return PIC_ERR_INVALID_ARG;
    }
    cudaStream_t st = E->stream;
    import_keys_ens_kernel<<<E->nsort, 256, 0, st>>>(E->cell[0], E->sort_blk, E->d_runs,
                                                      &E->dev[0].err, scratch, scratch + 2 * n);
    PIC_CUDA(cudaGetLastError());
    Fields F;
    memset(&F, 0, sizeof F);
    const void *in[6] = {E->cell[0], E->ox[0], E->oy[0], E->vx[0], E->vy[0], E->pid[0]};
    void *out[6] = {E->cell[1], E->ox[1], E->oy[1], E->vx[1], E->vy[1], E->pid[1]};
    F.nf = 6;
    for (int f = 0; f < 6; ++f) {
        F.in[f] = (const uint32_t *)in[f];
        F.out[f] = (uint32_t *)out[f];
    }
    uint4 *rec = reinterpret_cast<uint4 *>(scratch + 4 * n);
    if (packed) {
        import_pack_fields_kernel<<<grid_for(n, 256), 256, 0, st>>>(F, n, rec);
        PIC_CUDA(cudaGetLastError());
    }
    const uint32_t *idx = nullptr;
    PIC_TRY(radix_pairs(scratch, n, key_bits(E->nkeys), temp, temp_bytes, st, &idx));
    if (packed)
        import_unpack_kernel<<<grid_for(n, 256), 256, 0, st>>>(F, rec, idx, n);
    else
        import_gather_kernel<<<grid_for(n, 256), 256, 0, st>>>(F, idx, n);
    PIC_CUDA(cudaGetLastError());
    return PIC_OK;
}

}  // namespace pic
