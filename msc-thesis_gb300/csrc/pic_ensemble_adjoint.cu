// pic_ensemble_adjoint.cu -- discrete adjoint of every run of an ensemble.
//
// The map and its transpose are those of pic_adjoint.cu (priming half kick,
// leapfrog steps, J = final field energy per run).  What differs is how the
// positions and fields of past steps are recovered.  The single-run adjoint
// recomputes each segment forward into a ring; an ensemble holds too many
// particles for that, so each segment is walked backwards by reversing the
// leapfrog from an exact checkpoint of the segment's end state:
//   x_s = x_(s+1) - dt v_(s+1/2)            (push pass with drift -1 + deposit)
//   E(x_s)                                  (the ordinary field solve)
//   v_(s-1/2) = v_(s+1/2) - dt (q/m) F(x_s) (fused into the adjoint kick)
// The reversal is exact up to one rounding per step, and every segment
// restarts from its checkpoint, so the error does not accumulate beyond
// `every` steps.  Per backward step and run:
//   kick      a_v += dt a_x; mu = dt (q/m) a_v; g = sum_i w(x_i) mu_i (shared-
//             memory window as in the push); a_x += local CIC-gradient term
//   solve     psi = S^T g: batched R2C of (gx, gy), k-space kernel, batched C2R
//   gather    a_x += (q / dA) sum_m psi_m grad w_m(x)
// The adjoint arrays move with the particles through the sorts of the
// backward walk; at a checkpoint restore they are permuted into the
// checkpoint's storage order through particle ids.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "pic_adjoint_dev.cuh"
#include "pic_ensemble.cuh"
#include "pic_push_dev.cuh"

namespace pic {

struct EnsAdjArgs {
    const int32_t *cell;
    const float *ox, *oy;
    float *vx, *vy;            // un-kicked in place by the reversal
    const float *e;            // field pool
    float *ax, *ay, *avx, *avy;
    float *g;                  // scatter planes: run r's gx at 2 goff, gy ncp later
    const float *psi;          // S^T g: run r's plane at goff
};

struct Quad4 {
    float *a[4];
};
struct CQuad4 {
    const float *a[4];
};

__device__ __forceinline__ PushGeo adj_geo(const EnsRun &R, const float *e)
{
    PushGeo G = {};
    G.ex = e + 2 * R.goff;
    G.ey = G.ex + R.ncp;
    G.nx = R.nx;
    G.ny = R.ny;
    G.tw = R.tw;
    G.th = R.th;
    G.hx = R.hx;
    G.hy = R.hy;
    G.wcx = R.wcx;
    G.wcy = R.wcy;
    return G;
}

// Sums v[0..7] over each maximal run of consecutive lanes with the same key
// (particles are cell-sorted, so a warp holds few runs); true on the run's
// first lane, which then holds the run's totals.  Every lane of the warp
// must call it; key -1 marks a lane without a particle.  Lane i adds the
// partial of lane i + o only while i + o is before the next run start.
__device__ __forceinline__ bool warp_run_sum8(int key, float (&v)[8])
{
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int prev = __shfl_up_sync(full, key, 1);
    const bool head = lane == 0 || key != prev;
    const unsigned heads = __ballot_sync(full, head);
    const unsigned after = heads & (0xfffffffeu << lane);
    const int seg_end = after ? __ffs(after) - 1 : 32;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float t = __shfl_down_sync(full, v[k], o);
            if (lane + o < seg_end) v[k] += t;
        }
    }
    return head;
}

__device__ __forceinline__ void red_cell(float *gx, float *gy, int c, int nx, int ny, const float (&v)[8])
{
    const Cic w = cic_of(c, 0.f, 0.f, nx, ny);
    atomicAdd(gx + w.i00, v[0]);
    atomicAdd(gy + w.i00, v[1]);
    atomicAdd(gx + w.i10, v[2]);
    atomicAdd(gy + w.i10, v[3]);
    atomicAdd(gx + w.i01, v[4]);
    atomicAdd(gy + w.i01, v[5]);
    atomicAdd(gx + w.i11, v[6]);
    atomicAdd(gy + w.i11, v[7]);
}

// the same eight sums into the block's window (shared-memory float adds)
// when the cell lies in it, else straight to the grid
__device__ __forceinline__ void red_cell_win(const Window &W, int wcx, int wcy, float *gx, float *gy,
                                             int c, int nx, int ny, const float (&v)[8])
{
    int dxl = (c & 0xFFFF) - W.wx0, dyl = (c >> 16) - W.wy0;
    if (dxl < 0) dxl += nx;
    if (dyl < 0) dyl += ny;
    if (W.on && dxl < wcx && dyl < wcy) {
        float *sx = reinterpret_cast<float *>(W.sLo), *sy = reinterpret_cast<float *>(W.sHi);
        const int l = dyl * W.nwx + dxl;
        atomicAdd(sx + l, v[0]);
        atomicAdd(sy + l, v[1]);
        atomicAdd(sx + l + 1, v[2]);
        atomicAdd(sy + l + 1, v[3]);
        atomicAdd(sx + l + W.nwx, v[4]);
        atomicAdd(sy + l + W.nwx, v[5]);
        atomicAdd(sx + l + W.nwx + 1, v[6]);
        atomicAdd(sy + l + W.nwx + 1, v[7]);
    } else {
        red_cell(gx, gy, c, nx, ny, v);
    }
}

// Drift adjoint, kick transpose (scatter of mu and local term) and, with
// UNKICK, the reversal of the kick.  One push block of particles per CTA;
// each lane owns four consecutive particles (128-bit loads), E comes from
// the block's shared-memory window (global loads outside it).  Scatter
// contributions are summed in registers over a lane's particles in one
// cell, then over the warp's lanes in one cell (warp_run_sum8); the run's
// first lane adds them to the block's window (the deposit window's two
// planes, here as float x and y sums), which is flushed to the grid at the
// end.  Cells outside the window go to the grid directly.  Window adds
// without the warp sums measured 8% slower, global reductions without
// the window 4% slower.
template <bool UNKICK>
__global__ void __launch_bounds__(256, 3)
ens_adj_kick_kernel(EnsAdjArgs A, const SegBlock *__restrict__ blk, const EnsRun *__restrict__ runs,
                    const int32_t *__restrict__ anchor, float cscale, float dscale)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const SegBlock b = blk[blockIdx.x];
    const EnsRun &R = runs[b.run];
    const PushGeo G = adj_geo(R, A.e);
    const Window W = setup_window(G, smem, anchor[blockIdx.x]);
    load_window<true, false>(G, W);
    if (W.on)
        for (int i = threadIdx.x; i < W.nw; i += blockDim.x) W.sLo[i] = W.sHi[i] = 0u;
    __syncthreads();
    float *ggx = A.g + 2 * R.goff, *ggy = ggx + R.ncp;
    const float qmdt = R.qm_dt, muc = cscale * R.qm_dt, ddt = dscale * R.dt;
    const int nx = R.nx, ny = R.ny;
    const long long end = b.base + b.count;  // a multiple of 4 from base
    const long long lane4 = 4ll * (threadIdx.x & 31);
    for (long long qw = b.base + 4ll * (threadIdx.x & ~31u); qw < end; qw += 4ll * blockDim.x) {
        const long long q = qw + lane4;
        const bool live = q < end;
        int cc[4] = {-1, -1, -1, -1};
        float ox[4], oy[4], ax[4], ay[4], avx[4], avy[4], vx[4], vy[4];
        if (live) {
            const int4 c4 = *reinterpret_cast<const int4 *>(A.cell + q);
            const float4 a4 = *reinterpret_cast<const float4 *>(A.ox + q);
            const float4 b4 = *reinterpret_cast<const float4 *>(A.oy + q);
            const float4 x4 = *reinterpret_cast<const float4 *>(A.ax + q);
            const float4 y4 = *reinterpret_cast<const float4 *>(A.ay + q);
            const float4 u4 = *reinterpret_cast<const float4 *>(A.avx + q);
            const float4 w4 = *reinterpret_cast<const float4 *>(A.avy + q);
            cc[0] = c4.x, cc[1] = c4.y, cc[2] = c4.z, cc[3] = c4.w;
            ox[0] = a4.x, ox[1] = a4.y, ox[2] = a4.z, ox[3] = a4.w;
            oy[0] = b4.x, oy[1] = b4.y, oy[2] = b4.z, oy[3] = b4.w;
            ax[0] = x4.x, ax[1] = x4.y, ax[2] = x4.z, ax[3] = x4.w;
            ay[0] = y4.x, ay[1] = y4.y, ay[2] = y4.z, ay[3] = y4.w;
            avx[0] = u4.x, avx[1] = u4.y, avx[2] = u4.z, avx[3] = u4.w;
            avy[0] = w4.x, avy[1] = w4.y, avy[2] = w4.z, avy[3] = w4.w;
            if (UNKICK) {
                const float4 p4 = *reinterpret_cast<const float4 *>(A.vx + q);
                const float4 r4 = *reinterpret_cast<const float4 *>(A.vy + q);
                vx[0] = p4.x, vx[1] = p4.y, vx[2] = p4.z, vx[3] = p4.w;
                vy[0] = r4.x, vy[1] = r4.y, vy[2] = r4.z, vy[3] = r4.w;
            }
        }
        int gkey = -1;
        float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = cc[j];
            const int cx = c & 0xFFFF, cy = c >> 16;
            if (c < 0 || cx >= nx || cy >= ny) continue;
            const float avxj = fmaf(ddt, ax[j], avx[j]), avyj = fmaf(ddt, ay[j], avy[j]);
            const float mx = muc * avxj, my = muc * avyj;
            const float gx = 1.f - ox[j], gy = 1.f - oy[j];
            const float w00 = gx * gy, w10 = ox[j] * gy, w01 = gx * oy[j], w11 = ox[j] * oy[j];
            float2 e00, e10, e01, e11;
            int dxl = cx - W.wx0, dyl = cy - W.wy0;
            if (dxl < 0) dxl += nx;
            if (dyl < 0) dyl += ny;
            if (W.on && dxl < G.wcx && dyl < G.wcy) {
                const int l = dyl * W.nwx + dxl;
                e00 = W.sE[l];
                e10 = W.sE[l + 1];
                e01 = W.sE[l + W.nwx];
                e11 = W.sE[l + W.nwx + 1];
            } else {
                const Cic w = cic_of(c, 0.f, 0.f, nx, ny);
                e00 = make_float2(G.ex[w.i00], G.ey[w.i00]);
                e10 = make_float2(G.ex[w.i10], G.ey[w.i10]);
                e01 = make_float2(G.ex[w.i01], G.ey[w.i01]);
                e11 = make_float2(G.ex[w.i11], G.ey[w.i11]);
            }
            const float v[8] = {w00 * mx, w00 * my, w10 * mx, w10 * my,
                                w01 * mx, w01 * my, w11 * mx, w11 * my};
            if (gkey < 0) gkey = c;
            if (c == gkey) {
#pragma unroll
                for (int k = 0; k < 8; ++k) acc[k] += v[k];
            } else {
                red_cell_win(W, G.wcx, G.wcy, ggx, ggy, c, nx, ny, v);
            }
            const float s00 = e00.x * mx + e00.y * my, s10 = e10.x * mx + e10.y * my;
            const float s01 = e01.x * mx + e01.y * my, s11 = e11.x * mx + e11.y * my;
            ax[j] += (gy * (s10 - s00) + oy[j] * (s11 - s01)) * R.inv_dx;
            ay[j] += (gx * (s01 - s00) + ox[j] * (s11 - s10)) * R.inv_dy;
            avx[j] = avxj;
            avy[j] = avyj;
            if (UNKICK) {  // the push's gather, then the kick taken back
                const float Ex = gy * fmaf(gx, e00.x, ox[j] * e10.x) + oy[j] * fmaf(gx, e01.x, ox[j] * e11.x);
                const float Ey = gy * fmaf(gx, e00.y, ox[j] * e10.y) + oy[j] * fmaf(gx, e01.y, ox[j] * e11.y);
                vx[j] = fmaf(-qmdt, Ex, vx[j]);
                vy[j] = fmaf(-qmdt, Ey, vy[j]);
            }
        }
        if (warp_run_sum8(gkey, acc) && gkey >= 0) red_cell_win(W, G.wcx, G.wcy, ggx, ggy, gkey, nx, ny, acc);
        if (live) {
            *reinterpret_cast<float4 *>(A.ax + q) = make_float4(ax[0], ax[1], ax[2], ax[3]);
            *reinterpret_cast<float4 *>(A.ay + q) = make_float4(ay[0], ay[1], ay[2], ay[3]);
            *reinterpret_cast<float4 *>(A.avx + q) = make_float4(avx[0], avx[1], avx[2], avx[3]);
            *reinterpret_cast<float4 *>(A.avy + q) = make_float4(avy[0], avy[1], avy[2], avy[3]);
            if (UNKICK) {
                *reinterpret_cast<float4 *>(A.vx + q) = make_float4(vx[0], vx[1], vx[2], vx[3]);
                *reinterpret_cast<float4 *>(A.vy + q) = make_float4(vy[0], vy[1], vy[2], vy[3]);
            }
        }
    }
    if (!W.on) return;
    __syncthreads();
    const float *sx = reinterpret_cast<const float *>(W.sLo), *sy = reinterpret_cast<const float *>(W.sHi);
    WindowWalk w(W);
    for (int i = threadIdx.x; i < W.nw; i += blockDim.x, w.next(W)) {
        const float fx = sx[i], fy = sy[i];
        if (fx == 0.f && fy == 0.f) continue;
        const size_t o = w.node(W, nx, ny);
        if (fx != 0.f) atomicAdd(ggx + o, fx);
        if (fy != 0.f) atomicAdd(ggy + o, fy);
    }
}

// adjoint of the deposit: a_x += (q/dA) sum_m psi_m grad w_m (four
// consecutive particles per thread, 128-bit loads)
__global__ void __launch_bounds__(256)
ens_adj_gather_kernel(EnsAdjArgs A, const SegBlock *__restrict__ blk, const EnsRun *__restrict__ runs)
{
    const SegBlock b = blk[blockIdx.x];
    const EnsRun &R = runs[b.run];
    const float *psi = A.psi + R.goff;
    const long long end = b.base + b.count;
    for (long long q = b.base + 4ll * threadIdx.x; q < end; q += 4ll * blockDim.x) {
        const int4 c4 = *reinterpret_cast<const int4 *>(A.cell + q);
        const float4 a4 = *reinterpret_cast<const float4 *>(A.ox + q);
        const float4 b4 = *reinterpret_cast<const float4 *>(A.oy + q);
        float4 x4 = *reinterpret_cast<const float4 *>(A.ax + q);
        float4 y4 = *reinterpret_cast<const float4 *>(A.ay + q);
        const int cc[4] = {c4.x, c4.y, c4.z, c4.w};
        const float ox[4] = {a4.x, a4.y, a4.z, a4.w}, oy[4] = {b4.x, b4.y, b4.z, b4.w};
        float ax[4] = {x4.x, x4.y, x4.z, x4.w}, ay[4] = {y4.x, y4.y, y4.z, y4.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const Cic w = cic_of(cc[j], ox[j], oy[j], R.nx, R.ny);
            if (!w.ok) continue;
            const float2 g = grad_dot(w, psi[w.i00], psi[w.i10], psi[w.i01], psi[w.i11], R.inv_dx,
                                      R.inv_dy);
            ax[j] = fmaf(R.q_dA, g.x, ax[j]);
            ay[j] = fmaf(R.q_dA, g.y, ay[j]);
        }
        *reinterpret_cast<float4 *>(A.ax + q) = make_float4(ax[0], ax[1], ax[2], ax[3]);
        *reinterpret_cast<float4 *>(A.ay + q) = make_float4(ay[0], ay[1], ay[2], ay[3]);
    }
}

// psi^ of every run (into the first half of its spectrum pair)
__global__ void __launch_bounds__(256)
ens_adj_kspace_kernel(const float2 *__restrict__ ghat, float2 *__restrict__ psihat,
                      const SegBlock *__restrict__ blk, const EnsRun *__restrict__ runs)
{
    const SegBlock b = blk[blockIdx.x];
    const EnsRun &R = runs[b.run];
    for (long long j = threadIdx.x; j < b.count; j += blockDim.x) {
        const long long idx = b.base + j;
        const int my = (int)idx / R.nh, mx = (int)idx - my * R.nh;  // a run's modes fit in 32 bits
        psihat[R.khoff + idx] = adj_mode(ghat[R.khoff + idx], ghat[R.khoff + R.nk + idx], mx, my,
                                         R.nx, R.ny, R.kx1, R.ky1, R.inv_eps0_n, idx == 0);
    }
}

// terminal condition: g = eps0 dA E
__global__ void ens_adj_terminal_kernel(const float *__restrict__ e, float *__restrict__ g,
                                        const SegBlock *__restrict__ blk, const EnsRun *__restrict__ runs)
{
    const SegBlock b = blk[blockIdx.x];
    const EnsRun &R = runs[b.run];
    for (long long j = threadIdx.x; j < b.count; j += blockDim.x) {
        const long long node = b.base + j;
        g[2 * R.goff + node] = R.eps0_dA * e[2 * R.goff + node];
        g[2 * R.goff + R.ncp + node] = R.eps0_dA * e[2 * R.goff + R.ncp + node];
    }
}

// storage order -> id order (per run, at poff + pid) and back
__global__ void ens_to_id_kernel(const int32_t *__restrict__ cell, const uint32_t *__restrict__ pid,
                                 CQuad4 in, Quad4 out, const SegBlock *__restrict__ blk,
                                 const EnsRun *__restrict__ runs)
{
    const SegBlock b = blk[blockIdx.x];
    const EnsRun &R = runs[b.run];
    const long long end = b.base + b.count;
    for (long long i = b.base + threadIdx.x; i < end; i += blockDim.x) {
        const uint32_t p = pid[i];
        if (cell[i] < 0 || (long long)p >= R.n) continue;
#pragma unroll
        for (int k = 0; k < 4; ++k) out.a[k][R.poff + p] = in.a[k][i];
    }
}

__global__ void ens_from_id_kernel(const int32_t *__restrict__ cell, const uint32_t *__restrict__ pid,
                                   CQuad4 in, Quad4 out, const SegBlock *__restrict__ blk,
                                   const EnsRun *__restrict__ runs)
{
    const SegBlock b = blk[blockIdx.x];
    const EnsRun &R = runs[b.run];
    const long long end = b.base + b.count;
    for (long long i = b.base + threadIdx.x; i < end; i += blockDim.x) {
        const uint32_t p = pid[i];
        const bool ok = cell[i] >= 0 && (long long)p < R.n;
#pragma unroll
        for (int k = 0; k < 4; ++k) out.a[k][i] = ok ? in.a[k][R.poff + p] : 0.f;
    }
}

// One run's gradients in id order (doubles) and its load-parameter sums:
// acc[0] = sum sign(pid) dJ/dvx (beam drift), acc[1] = sum dJ/dx . dx/dA.
__global__ void ens_adj_export_kernel(const int32_t *__restrict__ cell, const uint32_t *__restrict__ pid,
                                      CQuad4 a, long long from, long long to, long long n,
                                      double *out, const double *dxdA, const double *dydA,
                                      double *acc)
{
    __shared__ double s0[8], s1[8];
    double b0 = 0.0, b1 = 0.0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = from + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < to; i += stride) {
        const uint32_t p = pid[i];
        if (cell[i] < 0 || (long long)p >= n) continue;
        const double gx = a.a[0][i], gy = a.a[1][i], gvx = a.a[2][i], gvy = a.a[3][i];
        if (out) {
            out[p] = gx;
            out[n + p] = gy;
            out[2 * n + p] = gvx;
            out[3 * n + p] = gvy;
        }
        b0 += (p & 1u) ? -gvx : gvx;
        if (dxdA) b1 += gx * dxdA[p] + gy * dydA[p];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        b0 += __shfl_xor_sync(0xffffffffu, b0, o);
        b1 += __shfl_xor_sync(0xffffffffu, b1, o);
    }
    if ((threadIdx.x & 31) == 0) {
        s0[threadIdx.x >> 5] = b0;
        s1[threadIdx.x >> 5] = b1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t0 = 0.0, t1 = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            t0 += s0[w];
            t1 += s1[w];
        }
        atomicAdd(acc, t0);
        atomicAdd(acc + 1, t1);
    }
}

// ------------------------------------------------------------------ driver
namespace {

// device buffers of one adjoint run, freed on every exit path
struct AdjBufs {
    std::vector<void *> dev, host;
    ~AdjBufs()
    {
        for (void *p : dev) cudaFree(p);
        for (void *p : host) cudaFreeHost(p);
    }
    template <class T> pic_status dalloc(T **p, size_t n)
    {
        void *q = nullptr;
        PIC_CUDA(cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)));
        dev.push_back(q);
        *p = (T *)q;
        return PIC_OK;
    }
    // device memory if it is available, else pinned host memory (reached
    // by the copies over the CPU-GPU link)
    template <class T> pic_status any_alloc(T **p, size_t n, bool *on_host)
    {
        void *q = nullptr;
        const size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
        if (cudaMalloc(&q, bytes) == cudaSuccess) {
            dev.push_back(q);
            *on_host = false;
        } else {
            cudaGetLastError();
            PIC_CUDA(cudaMallocHost(&q, bytes));
            host.push_back(q);
            *on_host = true;
        }
        *p = (T *)q;
        return PIC_OK;
    }
};

struct Ckpt {
    int32_t *cell;
    float *ox, *oy, *vx, *vy;
    uint32_t *pid;
};

pic_status ck_alloc(AdjBufs &B, Ckpt &C, size_t n, int *host_count)
{
    bool h[6];
    PIC_TRY(B.any_alloc(&C.cell, n, &h[0]));
    PIC_TRY(B.any_alloc(&C.ox, n, &h[1]));
    PIC_TRY(B.any_alloc(&C.oy, n, &h[2]));
    PIC_TRY(B.any_alloc(&C.vx, n, &h[3]));
    PIC_TRY(B.any_alloc(&C.vy, n, &h[4]));
    PIC_TRY(B.any_alloc(&C.pid, n, &h[5]));
    for (bool x : h) *host_count += x ? 1 : 0;
    return PIC_OK;
}

pic_status ck_copy(pic_ensemble *E, Ckpt &C, bool save)
{
    const size_t b = (size_t)E->nslots * 4;
    void *live[6] = {E->cell[0], E->ox[0], E->oy[0], E->vx[0], E->vy[0], E->pid[0]};
    void *ck[6] = {C.cell, C.ox, C.oy, C.vx, C.vy, C.pid};
    for (int k = 0; k < 6; ++k)
        PIC_CUDA(cudaMemcpyAsync(save ? ck[k] : live[k], save ? live[k] : ck[k], b,
                                 cudaMemcpyDefault, E->stream));
    return PIC_OK;
}

pic_status adj_plans(pic_ensemble *E)
{
    for (auto &G : E->groups) {
        if (G.r2c2) continue;
        const EnsRun &R = E->runs[G.first];
        int dims[2] = {G.ny, G.nx}, real_emb[2] = {G.ny, G.nx}, cplx_emb[2] = {G.ny, R.nh};
        // gx, gy of every run (stride ncp) -> gx^, gy^ (stride nk)
        PIC_CUFFT(cufftPlanMany(&G.r2c2, 2, dims, real_emb, 1, (int)R.ncp, cplx_emb, 1, (int)R.nk,
                                CUFFT_R2C, 2 * G.count));
        PIC_CUFFT(cufftSetStream(G.r2c2, E->stream));
        // psi^ (stride 2 nk) -> psi (stride ncp)
        PIC_CUFFT(cufftPlanMany(&G.c2r1, 2, dims, cplx_emb, 1, (int)(2 * R.nk), real_emb, 1,
                                (int)R.ncp, CUFFT_C2R, G.count));
        PIC_CUFFT(cufftSetStream(G.c2r1, E->stream));
    }
    return PIC_OK;
}

}  // namespace

pic_status ens_adjoint(pic_ensemble *E, const pic_init_spec *specs, long long nsteps, int every,
                       double *gx0, double *gy0, double *gvx0, double *gvy0, pic_adjoint_result *out)
{
    if (nsteps < 1 || every < 1 || !specs) {
        set_error("pic_ensemble_adjoint: needs specs, nsteps >= 1 and every >= 1");
        return PIC_ERR_INVALID_ARG;
    }
    PIC_TRY(pic_ensemble_init(E, specs));
    cudaStream_t st = E->stream;
    const int nr = E->nruns;
    const size_t ns = (size_t)E->nslots;
    const int K = (int)std::min<long long>(every, nsteps);
    const long long nseg = (nsteps + K - 1) / K;
    AdjBufs B;
    float *a[2][4], *g;
    float2 *ghat;
    for (int b = 0; b < 2; ++b)
        for (int k = 0; k < 4; ++k) PIC_TRY(B.dalloc(&a[b][k], ns));
    PIC_TRY(B.dalloc(&g, 2 * (size_t)E->nnodes));
    PIC_TRY(B.dalloc(&ghat, (size_t)E->nmodes));
    PIC_TRY(adj_plans(E));
    std::vector<Ckpt> ck((size_t)nseg);  // ck[m-1]: state at step m K; ck[nseg-1]: final state
    int on_host = 0;
    for (auto &C : ck) PIC_TRY(ck_alloc(B, C, ns, &on_host));

    // ---- forward with checkpoints
    for (long long m = 1; m < nseg; ++m) {
        PIC_TRY(pic_ensemble_step(E, K));
        PIC_TRY(ck_copy(E, ck[(size_t)m - 1], true));
    }
    PIC_TRY(pic_ensemble_step(E, nsteps - (nseg - 1) * K));
    PIC_TRY(ck_copy(E, ck[(size_t)nseg - 1], true));
    PIC_TRY(pic_ensemble_synchronize(E));
    // J per run, then the diagnostics state that the backward walk overwrites
    std::vector<DevState> saved(nr);
    PIC_CUDA(cudaMemcpy(saved.data(), E->dev, sizeof(DevState) * nr, cudaMemcpyDeviceToHost));
    const size_t hist_n = (size_t)nr * 6 * E->hist_cap;
    std::vector<double> hist_saved(hist_n);
    PIC_CUDA(cudaMemcpy(hist_saved.data(), E->hist, hist_n * 8, cudaMemcpyDeviceToHost));
    const int since_saved = E->since_sort;

    EnsAdjArgs A;
    A.e = E->e;
    A.g = g;
    A.psi = E->rho;
    int cur = 0;
    auto set_arrays = [&]() {
        A.cell = E->cell[0];
        A.ox = E->ox[0];
        A.oy = E->oy[0];
        A.vx = E->vx[0];
        A.vy = E->vy[0];
        A.ax = a[cur][0];
        A.ay = a[cur][1];
        A.avx = a[cur][2];
        A.avy = a[cur][3];
    };
    auto solve_gather = [&]() -> pic_status {
        for (auto &G : E->groups) {
            const EnsRun &R = E->runs[G.first];
            PIC_CUFFT(cufftExecR2C(G.r2c2, g + 2 * R.goff, (cufftComplex *)(ghat + R.khoff)));
        }
        ens_adj_kspace_kernel<<<E->nmode_blk, 256, 0, st>>>(ghat, E->rhohat, E->mode_blk, E->d_runs);
        PIC_CUDA(cudaGetLastError());
        for (auto &G : E->groups) {
            const EnsRun &R = E->runs[G.first];
            PIC_CUFFT(cufftExecC2R(G.c2r1, (cufftComplex *)(E->rhohat + R.khoff), E->rho + R.goff));
        }
        set_arrays();
        ens_adj_gather_kernel<<<E->npush, 256, 0, st>>>(A, E->push_blk, E->d_runs);
        PIC_CUDA(cudaGetLastError());
        return PIC_OK;
    };
    auto kick = [&](bool unkick, float cscale, float dscale) -> pic_status {
        PIC_CUDA(cudaMemsetAsync(g, 0, sizeof(float) * 2 * (size_t)E->nnodes, st));
        set_arrays();
        PIC_TRY(allow_dynamic_smem((const void *)ens_adj_kick_kernel<true>, E->push_smem));
        PIC_TRY(allow_dynamic_smem((const void *)ens_adj_kick_kernel<false>, E->push_smem));
        if (unkick)
            ens_adj_kick_kernel<true><<<E->npush, 256, E->push_smem, st>>>(A, E->push_blk, E->d_runs,
                                                                       E->anchor, cscale, dscale);
        else
            ens_adj_kick_kernel<false><<<E->npush, 256, E->push_smem, st>>>(A, E->push_blk, E->d_runs,
                                                                        E->anchor, cscale, dscale);
        PIC_CUDA(cudaGetLastError());
        return solve_gather();
    };
    auto quad = [&](int b) {
        Quad4 q;
        for (int k = 0; k < 4; ++k) q.a[k] = a[b][k];
        return q;
    };
    auto cquad = [&](int b) {
        CQuad4 q;
        for (int k = 0; k < 4; ++k) q.a[k] = a[b][k];
        return q;
    };

    // ---- terminal condition a_x = grad J(x_N), a_v = 0
    for (int k = 0; k < 4; ++k) PIC_CUDA(cudaMemsetAsync(a[cur][k], 0, ns * 4, st));
    ens_adj_terminal_kernel<<<E->nnode_blk, 256, 0, st>>>(E->e, g, E->node_blk, E->d_runs);
    PIC_CUDA(cudaGetLastError());
    PIC_TRY(solve_gather());

    // ---- backward walk
    const int S = E->sort_every;
    int since = 0;
    for (long long s = nsteps - 1; s >= 0; --s) {
        if ((s + 1) % K == 0 && s + 1 < nsteps) {
            // exact state at s + 1: adjoint arrays into the checkpoint's order
            ens_to_id_kernel<<<E->nsort, 256, 0, st>>>(E->cell[0], E->pid[0], cquad(cur), quad(1 - cur),
                                                       E->sort_blk, E->d_runs);
            PIC_CUDA(cudaGetLastError());
            PIC_TRY(ck_copy(E, ck[(size_t)((s + 1) / K - 1)], false));
            ens_from_id_kernel<<<E->nsort, 256, 0, st>>>(E->cell[0], E->pid[0], cquad(1 - cur), quad(cur),
                                                         E->sort_blk, E->d_runs);
            PIC_CUDA(cudaGetLastError());
            since = S;
        }
        int src = 0;
        if (since >= S) {
            const float *xin[4] = {a[cur][0], a[cur][1], a[cur][2], a[cur][3]};
            float *xout[4] = {a[1 - cur][0], a[1 - cur][1], a[1 - cur][2], a[1 - cur][3]};
            PIC_TRY(ens_sort(E, xin, xout));
            cur ^= 1;
            src = 1;
            since = 0;
        }
        PIC_TRY(ens_launch_push(E, src, 3));  // x_s, deposit
        PIC_TRY(ens_poisson(E));              // E(x_s)
        PIC_TRY(kick(true, 1.f, 1.f));
        ++since;
    }
    PIC_TRY(kick(false, -0.5f, 0.f));  // the priming half kick

    // ---- outputs
    std::vector<double> acc(2 * (size_t)nr, 0.0);
    double *d_acc, *stage = nullptr, *dA = nullptr;
    PIC_TRY(B.dalloc(&d_acc, 2 * (size_t)nr));
    PIC_CUDA(cudaMemsetAsync(d_acc, 0, 16 * (size_t)nr, st));
    long long nmax = 0;
    for (const EnsRun &R : E->runs) nmax = std::max(nmax, R.n);
    const bool want = gx0 || gy0 || gvx0 || gvy0;
    if (want) PIC_TRY(B.dalloc(&stage, 4 * (size_t)nmax));
    PIC_TRY(B.dalloc(&dA, 2 * (size_t)nmax));
    std::vector<long long> first(nr, 0);
    for (int r = 1; r < nr; ++r) first[r] = first[r - 1] + specs[r - 1].n;
    std::vector<double> host;
    for (int r = 0; r < nr; ++r) {
        const int sidx = E->slot_of[r];
        const EnsRun &R = E->runs[sidx];
        const pic_init_spec &sp = specs[r];
        const bool amp_kind = sp.pert_kind == PIC_PERT_XDISP || sp.pert_kind == PIC_PERT_DENSITY;
        if (amp_kind && R.n) {
            int lx = 0, ly = 0;
            if (sp.layout == PIC_LOAD_LATTICE)
                PIC_TRY(lattice_dims_for(R.nx, R.ny, R.n, &lx, &ly));
            InitTarget T;
            memset(&T, 0, sizeof T);
            T.nx = R.nx;
            T.ny = R.ny;
            T.Lx = E->cfg[r].Lx;
            T.Ly = E->cfg[r].Ly;
            PIC_TRY(launch_init_dA_target(T, &sp, lx, ly, dA, dA + R.n, st));
        }
        ens_adj_export_kernel<<<grid_for(R.cap4, 256), 256, 0, st>>>(
            E->cell[0], E->pid[0], cquad(cur), R.poff, R.poff + R.cap4, R.n, want ? stage : nullptr,
            amp_kind ? dA : nullptr, amp_kind ? dA + R.n : nullptr, d_acc + 2 * r);
        PIC_CUDA(cudaGetLastError());
        if (want && R.n) {
            host.resize(4 * (size_t)R.n);
            PIC_CUDA(cudaMemcpyAsync(host.data(), stage, host.size() * 8, cudaMemcpyDeviceToHost, st));
            PIC_CUDA(cudaStreamSynchronize(st));
            double *dst[4] = {gx0, gy0, gvx0, gvy0};
            for (int k = 0; k < 4; ++k)
                if (dst[k]) std::copy(host.begin() + k * R.n, host.begin() + (k + 1) * R.n, dst[k] + first[r]);
        }
    }
    PIC_CUDA(cudaMemcpyAsync(acc.data(), d_acc, 16 * (size_t)nr, cudaMemcpyDeviceToHost, st));
    // ---- leave the ensemble at step nsteps
    PIC_TRY(ck_copy(E, ck[(size_t)nseg - 1], false));
    PIC_TRY(ens_launch_push(E, 0, 2));  // deposit in place
    PIC_TRY(ens_poisson(E));
    PIC_CUDA(cudaMemcpyAsync(E->dev, saved.data(), sizeof(DevState) * nr, cudaMemcpyHostToDevice, st));
    PIC_CUDA(cudaMemcpyAsync(E->hist, hist_saved.data(), hist_n * 8, cudaMemcpyHostToDevice, st));
    PIC_CUDA(cudaStreamSynchronize(st));
    E->since_sort = std::max(since_saved, S);  // anchors are stale: sort before the next step
    if (out) {
        for (int r = 0; r < nr; ++r) {
            const int sidx = E->slot_of[r];
            const long long step = saved[sidx].step;
            out[r].J = hist_saved[(size_t)sidx * 6 * E->hist_cap + (size_t)(step % E->hist_cap)];
            out[r].dJ_dbeam_v = acc[2 * r];
            out[r].dJ_damp = acc[2 * r + 1];
        }
    }
    (void)on_host;
    return PIC_OK;
}

}  // namespace pic

extern "C" pic_status pic_ensemble_adjoint(pic_ensemble *e, const pic_init_spec *specs,
                                           long long nsteps, int every, double *dJ_dx0,
                                           double *dJ_dy0, double *dJ_dvx0, double *dJ_dvy0,
                                           pic_adjoint_result *out)
{
    PIC_TRY(pic::ens_need(e, -1));
    return pic::ens_adjoint(e, specs, nsteps, every, dJ_dx0, dJ_dy0, dJ_dvx0, dJ_dvy0, out);
}
