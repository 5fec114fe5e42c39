// pic_init.cu -- creating, importing and exporting particles.
//
// Replaces (taylorj5/msc-thesis, thesisCode/collisionless/double/src/):
//   main.cc:201-244     initialiseParticles (lattice + Gaussian + drift)
//   particle.cc:21-29   Particle::Particle  (cell from position)
//   pic.cu:520-523, 583-584  the host<->device particle copies
// Random numbers come from Philox4x32-10 keyed by (seed) with the counter
// (particle id, block, 0, STREAM_INIT), so every particle's initial state
// depends only on the seed and its id.
#include <cuda_runtime.h>

#include <algorithm>
#include <math.h>

#include "pic_internal.cuh"
#include "pic_sort_dev.cuh"

namespace pic {

struct InitArgs {
    int32_t *cell;
    float *ox, *oy, *vx, *vy, *vz;
    uint32_t *pid;
    long long n;
    int nx, ny;
    double Lx, Ly, dx, dy, inv_dx, inv_dy;
    int layout, pert_kind, lat_nx, lat_ny;
    double vth0, vth1, vth2, vd0, vd1, beam_v, amp;
    double kx, ky;  // perturbation wavevector
    double xi[2][2], uu[2][2];  // PIC_PERT_BEAM_MODE amplitudes per beam (re, im)
    uint32_t k0, k1;
};

// global position -> (cell, offset) with periodic wrap; inv_d = 1/d.  FP64
// work is kept to a few multiplies (no division), and the wrap is skipped for
// positions already inside [0, L).
__device__ __forceinline__ void locate(double x, double L, double inv_d, int n, int &c, float &o)
{
    if (!(x >= 0.0 && x < L)) x -= L * floor(x * (1.0 / L));
    double g = x * inv_d;
    double f = floor(g);
    int i = (int)f;
    float fr = (float)(g - f);
    if (fr >= 1.0f) {
        fr = 0.0f;
        i += 1;
    }
    if (i >= n) i -= n;
    if (i < 0) i += n;
    c = i;
    o = fr;
}

__global__ void __launch_bounds__(256) init_kernel(InitArgs A)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += stride) {
        const U4 r0 = philox4x32_10(U4{(uint32_t)i, (uint32_t)(i >> 32), 0u, STREAM_INIT}, A.k0, A.k1);
        const U4 r1 = philox4x32_10(U4{(uint32_t)i, (uint32_t)(i >> 32), 1u, STREAM_INIT}, A.k0, A.k1);
        double x, y;
        if (A.layout == PIC_LOAD_LATTICE) {
            const long long ix = i % A.lat_nx, iy = i / A.lat_nx;
            x = ((double)ix + 0.5) * (A.Lx / A.lat_nx);
            y = ((double)iy + 0.5) * (A.Ly / A.lat_ny);
        } else {
            x = u01d(r0.x) * A.Lx;
            y = u01d(r0.y) * A.Ly;
        }
        double dvx = 0.0;
        if (A.pert_kind == PIC_PERT_XDISP) {
            x += A.amp * cos(A.kx * x);
        } else if (A.pert_kind == PIC_PERT_BEAM_MODE) {
            const int b = (int)(i & 1);
            double sk, ck;
            sincos(A.kx * x, &sk, &ck);
            dvx = A.uu[b][0] * ck - A.uu[b][1] * sk;
            x += A.xi[b][0] * ck - A.xi[b][1] * sk;
        } else if (A.pert_kind == PIC_PERT_DENSITY) {
            // displacement -(amp/|k|^2) k sin(k.x) gives n ~ 1 + amp cos(k.x) to first order
            const double k2 = A.kx * A.kx + A.ky * A.ky;
            const double s = sin(A.kx * x + A.ky * y) * (A.amp / k2);
            x -= A.kx * s;
            y -= A.ky * s;
        }
        int cx, cy;
        float ox, oy;
        locate(x, A.Lx, 1.0 / A.dx, A.nx, cx, ox);
        locate(y, A.Ly, 1.0 / A.dy, A.ny, cy, oy);
        // Box-Muller normals
        const float ra = sqrtf(-2.f * logf(u01f(r0.z)));
        float sa, ca;
        sincospif(2.f * u01f(r0.w), &sa, &ca);
        const float rb = sqrtf(-2.f * logf(u01f(r1.x)));
        float sb, cb;
        sincospif(2.f * u01f(r1.y), &sb, &cb);
        double vx = A.vd0 + A.vth0 * (double)(ra * ca);
        const double vy = A.vd1 + A.vth1 * (double)(ra * sa);
        if (A.beam_v != 0.0) vx += (i & 1) ? -A.beam_v : A.beam_v;
        vx += dvx;
        A.cell[i] = cx | (cy << 16);
        A.ox[i] = ox;
        A.oy[i] = oy;
        A.vx[i] = (float)vx;
        A.vy[i] = (float)vy;
        if (A.vz) A.vz[i] = (float)(A.vth2 * (double)(rb * cb));
        A.pid[i] = (uint32_t)i;
    }
}

__global__ void from_global_kernel(InitArgs A, const double *x, const double *y, const double *vx,
                                   const double *vy, const double *vz)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += stride) {
        int cx, cy;
        float ox, oy;
        locate(x[i], A.Lx, A.inv_dx, A.nx, cx, ox);
        locate(y[i], A.Ly, A.inv_dy, A.ny, cy, oy);
        A.cell[i] = cx | (cy << 16);
        A.ox[i] = ox;
        A.oy[i] = oy;
        A.vx[i] = (float)vx[i];
        A.vy[i] = (float)vy[i];
        if (A.vz) A.vz[i] = vz ? (float)vz[i] : 0.f;
        A.pid[i] = (uint32_t)i;
    }
}

// Host arrays straight to the import sort's input: for every slot of
// [lo, hi) its key and slot number, and its fields as the 32-byte record
// {cell, ox, oy, vx}, {vy, pid, vz, 0}; slots n..cap-1 are empty (cell -1,
// the empty key).
__global__ void from_global_records_kernel(InitArgs A, KeyGeo G, long long lo, long long hi,
                                           unsigned *err,
                                           const double *x, const double *y, const double *vx,
                                           const double *vy, const double *vz,
                                           uint32_t *__restrict__ keys, uint32_t *__restrict__ idx,
                                           uint4 *__restrict__ rec)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = lo + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += stride) {
        idx[i] = (uint32_t)i;
        if (i < A.n) {
            int cx, cy;
            float ox, oy;
            locate(x[i], A.Lx, A.inv_dx, A.nx, cx, ox);
            locate(y[i], A.Ly, A.inv_dy, A.ny, cy, oy);
            const int c = cx | (cy << 16);
            keys[i] = (uint32_t)particle_key(G, err, c);
            rec[2 * i] = make_uint4((uint32_t)c, __float_as_uint(ox), __float_as_uint(oy),
                                    __float_as_uint((float)vx[i]));
            rec[2 * i + 1] = make_uint4(__float_as_uint((float)vy[i]), (uint32_t)i,
                                        vz ? __float_as_uint((float)vz[i]) : 0u, 0u);
        } else {
            keys[i] = (uint32_t)particle_key(G, err, -1);
            rec[2 * i] = make_uint4(0xFFFFFFFFu, 0u, 0u, 0u);
            rec[2 * i + 1] = make_uint4(0u, 0xFFFFFFFFu, 0u, 0u);
        }
    }
}

// Export in id order: out[pid[i]] = particle i.
__global__ void to_global_kernel(const int32_t *cell, const float *ox, const float *oy,
                                 const float *vx, const float *vy, const float *vz,
                                 const uint32_t *pid, const long long *d_n, double dx, double dy,
                                 double *x, double *y, double *ux, double *uy, double *uz)
{
    const long long n = *d_n;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t p = pid[i];
        if ((long long)p >= n) continue;
        const int c = cell[i];
        const int cx = c & 0xFFFF, cy = c >> 16;
        if (x) x[p] = ((double)cx + (double)ox[i]) * dx;
        if (y) y[p] = ((double)cy + (double)oy[i]) * dy;
        if (ux) ux[p] = vx[i];
        if (uy) uy[p] = vy[i];
        if (uz) uz[p] = vz ? (double)vz[i] : 0.0;
    }
}

// inv[pid[i]] = i for the n live slots (ids are a permutation of 0..n-1)
__global__ void id_inverse_kernel(const uint32_t *__restrict__ pid, const long long *d_n,
                                  uint32_t *__restrict__ inv)
{
    const long long n = *d_n;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t p = pid[i];
        if ((long long)p < n) inv[p] = (uint32_t)i;
    }
}

// One exported field in id order: out[p] from slot inv[p] (coalesced writes,
// gathered reads).  field: 0 x, 1 y, 2 vx, 3 vy, 4 vz.
__global__ void id_gather_kernel(const uint32_t *__restrict__ inv, const long long *d_n, int field,
                                 const int32_t *__restrict__ cell, const float *__restrict__ off,
                                 const float *__restrict__ v, double d, double *__restrict__ out)
{
    const long long n = *d_n;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += stride) {
        const uint32_t i = inv[p];
        if ((long long)i >= n || cell[i] < 0) continue;  // an id no live slot carries
        if (field == 0)
            out[p] = ((double)(cell[i] & 0xFFFF) + (double)off[i]) * d;
        else if (field == 1)
            out[p] = ((double)(cell[i] >> 16) + (double)off[i]) * d;
        else
            out[p] = v ? (double)v[i] : 0.0;
    }
}

// Export through packed records, ids [lo, hi) at a time: every slot whose
// id falls in the range scatters its fields to that id's record, {cell, ox,
// oy, vx}, {vy, vz, cell, 0}, one 32-byte sector per particle written whole.
// Records of ids no slot carries keep the 0xFF fill (cell -1).
__global__ void id_record_kernel(const int32_t *__restrict__ cell, const float *__restrict__ ox,
                                 const float *__restrict__ oy, const float *__restrict__ vx,
                                 const float *__restrict__ vy, const float *__restrict__ vz,
                                 const uint32_t *__restrict__ pid, const long long *d_n, long long lo,
                                 long long hi, uint4 *__restrict__ rec)
{
    const long long n = *d_n;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const long long p = pid[i];
        if (p < lo || p >= hi || p >= n) continue;
        const size_t r = 2 * (size_t)(p - lo);
        const uint32_t c = (uint32_t)cell[i];
        rec[r] = make_uint4(c, __float_as_uint(ox[i]), __float_as_uint(oy[i]), __float_as_uint(vx[i]));
        rec[r + 1] = make_uint4(__float_as_uint(vy[i]), vz ? __float_as_uint(vz[i]) : 0u, c, 0u);
    }
}

// One exported field of `count` consecutive ids from their records
// (coalesced both ways).  field: 0 x, 1 y, 2 vx, 3 vy, 4 vz.
__global__ void id_record_field_kernel(const uint4 *__restrict__ rec, long long count, int field,
                                       double d, double *__restrict__ out)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < count; p += stride) {
        if (field <= 2) {
            const uint4 a = rec[2 * p];
            const int c = (int)a.x;
            if (c < 0) continue;  // an id no slot carries
            if (field == 0)
                out[p] = ((double)(c & 0xFFFF) + (double)__uint_as_float(a.y)) * d;
            else if (field == 1)
                out[p] = ((double)(c >> 16) + (double)__uint_as_float(a.z)) * d;
            else
                out[p] = (double)__uint_as_float(a.w);
        } else {
            const uint4 b = rec[2 * p + 1];
            if ((int)b.z < 0) continue;
            out[p] = (double)__uint_as_float(field == 3 ? b.x : b.y);
        }
    }
}

__global__ void fill_padding_kernel(int32_t *c0, int32_t *c1, long long from, long long to)
{
    const long long i = from + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < to) {
        c0[i] = -1;
        c1[i] = -1;
    }
}

static InitArgs target_args(const InitTarget &T)
{
    InitArgs A;
    memset(&A, 0, sizeof(A));
    A.cell = T.cell;
    A.ox = T.ox;
    A.oy = T.oy;
    A.vx = T.vx;
    A.vy = T.vy;
    A.vz = T.vz;
    A.pid = T.pid;
    A.nx = T.nx;
    A.ny = T.ny;
    A.Lx = T.Lx;
    A.Ly = T.Ly;
    A.dx = T.Lx / T.nx;
    A.dy = T.Ly / T.ny;
    A.inv_dx = 1.0 / A.dx;
    A.inv_dy = 1.0 / A.dy;
    return A;
}

InitTarget target_of(pic_handle *h, int s)
{
    SpeciesBuf &B = h->sp[s];
    InitTarget T;
    T.cell = B.cell[0];
    T.ox = B.ox[0];
    T.oy = B.oy[0];
    T.vx = B.vx[0];
    T.vy = B.vy[0];
    T.vz = B.vz[0];
    T.pid = B.pid[0];
    T.nx = h->g.nx;
    T.ny = h->g.ny;
    T.Lx = h->g.Lx;
    T.Ly = h->g.Ly;
    return T;
}

static InitArgs base_args(pic_handle *h, int s)
{
    InitArgs A = target_args(target_of(h, s));
    // the handle's own cell size (identical to L / n up to rounding)
    A.dx = h->g.dx;
    A.dy = h->g.dy;
    A.inv_dx = 1.0 / h->g.dx;
    A.inv_dy = 1.0 / h->g.dy;
    return A;
}

static void spec_args(InitArgs &A, const pic_init_spec *spec, int lat_nx, int lat_ny)
{
    A.n = spec->n;
    A.layout = spec->layout;
    A.pert_kind = spec->pert_kind;
    A.lat_nx = lat_nx;
    A.lat_ny = lat_ny;
    A.vth0 = spec->vth[0];
    A.vth1 = spec->vth[1];
    A.vth2 = spec->vth[2];
    A.vd0 = spec->vdrift[0];
    A.vd1 = spec->vdrift[1];
    A.beam_v = spec->beam_v;
    A.amp = spec->pert_amp;
    A.kx = 2.0 * 3.14159265358979323846 * spec->pert_mx / A.Lx;
    A.ky = 2.0 * 3.14159265358979323846 * spec->pert_my / A.Ly;
    for (int b = 0; b < 2; ++b)
        for (int c = 0; c < 2; ++c) {
            A.xi[b][c] = spec->beam_xi[b][c];
            A.uu[b][c] = spec->beam_u[b][c];
        }
    A.k0 = (uint32_t)spec->seed;
    A.k1 = (uint32_t)(spec->seed >> 32);
}

static pic_status run_init(const InitArgs &A, cudaStream_t st)
{
    if (A.n > 0) {
        init_kernel<<<grid_for(A.n, 256), 256, 0, st>>>(A);
        PIC_CUDA(cudaGetLastError());
    }
    return PIC_OK;
}

pic_status launch_init(pic_handle *h, int s, const pic_init_spec *spec, int lat_nx, int lat_ny)
{
    InitArgs A = base_args(h, s);
    spec_args(A, spec, lat_nx, lat_ny);
    return run_init(A, h->stream);
}

pic_status launch_init_target(const InitTarget &T, const pic_init_spec *spec, int lat_nx,
                              int lat_ny, cudaStream_t st)
{
    InitArgs A = target_args(T);
    spec_args(A, spec, lat_nx, lat_ny);
    return run_init(A, st);
}

// d(x, y)/d(pert_amp) of init_kernel's position, in id order.  XDISP:
// (cos(kx x_lat), 0); DENSITY: -k sin(k.x_lat) / |k|^2; other kinds: 0.
__global__ void init_damp_kernel(InitArgs A, double *dxa, double *dya)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += stride) {
        double x, y;
        if (A.layout == PIC_LOAD_LATTICE) {
            const long long ix = i % A.lat_nx, iy = i / A.lat_nx;
            x = ((double)ix + 0.5) * (A.Lx / A.lat_nx);
            y = ((double)iy + 0.5) * (A.Ly / A.lat_ny);
        } else {
            const U4 r0 = philox4x32_10(U4{(uint32_t)i, (uint32_t)(i >> 32), 0u, STREAM_INIT}, A.k0, A.k1);
            x = u01d(r0.x) * A.Lx;
            y = u01d(r0.y) * A.Ly;
        }
        double gx = 0.0, gy = 0.0;
        if (A.pert_kind == PIC_PERT_XDISP) {
            gx = cos(A.kx * x);
        } else if (A.pert_kind == PIC_PERT_DENSITY) {
            const double k2 = A.kx * A.kx + A.ky * A.ky;
            const double s = sin(A.kx * x + A.ky * y) / k2;
            gx = -A.kx * s;
            gy = -A.ky * s;
        }
        dxa[i] = gx;
        dya[i] = gy;
    }
}

pic_status launch_init_dA_target(const InitTarget &T, const pic_init_spec *spec, int lat_nx,
                                 int lat_ny, double *dxdA, double *dydA, cudaStream_t st)
{
    InitArgs A = target_args(T);
    spec_args(A, spec, lat_nx, lat_ny);
    if (A.n > 0) {
        init_damp_kernel<<<grid_for(A.n, 256), 256, 0, st>>>(A, dxdA, dydA);
        PIC_CUDA(cudaGetLastError());
    }
    return PIC_OK;
}

pic_status launch_init_dA(pic_handle *h, const pic_init_spec *spec, int lat_nx, int lat_ny,
                          double *dxdA, double *dydA)
{
    return launch_init_dA_target(target_of(h, 0), spec, lat_nx, lat_ny, dxdA, dydA, h->stream);
}

pic_status launch_from_global(pic_handle *h, int s, long long n, const double *x_dev,
                              const double *y_dev, const double *vx_dev, const double *vy_dev,
                              const double *vz_dev)
{
    InitArgs A = base_args(h, s);
    A.n = n;
    if (n > 0) {
        from_global_kernel<<<grid_for(n, 256), 256, 0, h->stream>>>(A, x_dev, y_dev, vx_dev, vy_dev,
                                                                  vz_dev);
        PIC_CUDA(cudaGetLastError());
    }
    return PIC_OK;
}

// Slots [lo, hi) of species s from device-visible host arrays into the stage
// (keys, slots and records laid out for a cap-slot import sort), on the
// handle's stream.
pic_status launch_from_global_records_range(pic_handle *h, int s, long long n, long long lo,
                                            long long hi, const double *x_dev, const double *y_dev,
                                            const double *vx_dev, const double *vy_dev,
                                            const double *vz_dev, int max_blocks)
{
    SpeciesBuf &B = h->sp[s];
    const long long cap = B.cap;
    if (!cap || hi <= lo) return PIC_OK;
    InitArgs A = base_args(h, s);
    A.n = n;
    const Geometry &g = h->g;
    const KeyGeo G = key_geo(g.nx, g.ny, g.tw, g.th, g.ntx, 0);
    uint32_t *scratch = (uint32_t *)h->stage;
    int grid = grid_for(hi - lo, 256);
    if (max_blocks > 0) grid = std::min(grid, max_blocks);
    from_global_records_kernel<<<grid, 256, 0, h->stream>>>(
        A, G, lo, hi, &h->dev->err, x_dev, y_dev, vx_dev, vy_dev, vz_dev, scratch,
        scratch + 2 * cap, reinterpret_cast<uint4 *>(scratch + 4 * cap));
    PIC_CUDA(cudaGetLastError());
    return PIC_OK;
}

pic_status launch_from_global_records(pic_handle *h, int s, long long n, const double *x_dev,
                                      const double *y_dev, const double *vx_dev,
                                      const double *vy_dev, const double *vz_dev)
{
    return launch_from_global_records_range(h, s, n, 0, h->sp[s].cap, x_dev, y_dev, vx_dev,
                                            vy_dev, vz_dev, 0);
}

// Export of species s in id order into five device arrays out[0..4] (x, y,
// vx, vy, vz; null entries skipped) through the slot-of-id inverse (`inv`,
// cap words); after each field's gather `ready[k]` is recorded on the
// handle's stream, so that a copy of field k can start while the next
// field is gathered.
pic_status launch_to_global_by_id(pic_handle *h, int s, double *const *out, uint32_t *inv,
                                  cudaEvent_t *ready)
{
    SpeciesBuf &B = h->sp[s];
    if (B.cap == 0) return PIC_OK;
    const long long *d_n = &h->dev->n[s];
    PIC_CUDA(cudaMemsetAsync(inv, 0xFF, sizeof(uint32_t) * (size_t)B.cap, h->stream));
    id_inverse_kernel<<<grid_for(B.cap, 256), 256, 0, h->stream>>>(B.pid[0], d_n, inv);
    PIC_CUDA(cudaGetLastError());
    const float *off[5] = {B.ox[0], B.oy[0], nullptr, nullptr, nullptr};
    const float *vel[5] = {nullptr, nullptr, B.vx[0], B.vy[0], B.vz[0]};
    const double dd[5] = {h->g.dx, h->g.dy, 0.0, 0.0, 0.0};
    for (int k = 0; k < 5; ++k) {
        if (!out[k]) continue;
        id_gather_kernel<<<grid_for(B.cap, 256), 256, 0, h->stream>>>(inv, d_n, k, B.cell[0], off[k],
                                                                       vel[k], dd[k], out[k]);
        PIC_CUDA(cudaGetLastError());
        PIC_CUDA(cudaEventRecord(ready[k], h->stream));
    }
    return PIC_OK;
}

pic_status launch_to_global_by_record(pic_handle *h, int s, long long lo, long long hi,
                                      double *const *out, uint4 *rec, cudaEvent_t *ready)
{
    SpeciesBuf &B = h->sp[s];
    if (B.cap == 0 || hi <= lo) return PIC_OK;
    const long long *d_n = &h->dev->n[s];
    PIC_CUDA(cudaMemsetAsync(rec, 0xFF, 32 * (size_t)(hi - lo), h->stream));
    id_record_kernel<<<grid_for(B.cap, 256), 256, 0, h->stream>>>(
        B.cell[0], B.ox[0], B.oy[0], B.vx[0], B.vy[0], B.vz[0], B.pid[0], d_n, lo, hi, rec);
    PIC_CUDA(cudaGetLastError());
    const double dd[5] = {h->g.dx, h->g.dy, 0.0, 0.0, 0.0};
    for (int k = 0; k < 5; ++k) {
        if (!out[k]) continue;
        id_record_field_kernel<<<grid_for(hi - lo, 256), 256, 0, h->stream>>>(rec, hi - lo, k, dd[k],
                                                                              out[k] + lo);
        PIC_CUDA(cudaGetLastError());
        PIC_CUDA(cudaEventRecord(ready[k], h->stream));
    }
    return PIC_OK;
}

pic_status launch_to_global_target(const InitTarget &T, const long long *d_n, long long cap,
                                   double *x_dev, double *y_dev, double *vx_dev, double *vy_dev,
                                   cudaStream_t st)
{
    if (cap == 0) return PIC_OK;
    to_global_kernel<<<grid_for(cap, 256), 256, 0, st>>>(T.cell, T.ox, T.oy, T.vx, T.vy, nullptr,
                                                         T.pid, d_n, T.Lx / T.nx, T.Ly / T.ny,
                                                         x_dev, y_dev, vx_dev, vy_dev, nullptr);
    PIC_CUDA(cudaGetLastError());
    return PIC_OK;
}

pic_status launch_fill_padding(pic_handle *h, int s, long long from, long long to)
{
    SpeciesBuf &B = h->sp[s];
    if (to <= from) return PIC_OK;
    const long long m = to - from;
    fill_padding_kernel<<<(unsigned)((m + 255) / 256), 256, 0, h->stream>>>(B.cell[0], B.cell[1],
                                                                          from, to);
    PIC_CUDA(cudaGetLastError());
    return PIC_OK;
}

}  // namespace pic
