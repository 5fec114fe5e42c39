// pic_spectral.cu -- the step's Poisson solve for power-of-two grids
// (16..4096 cells a side) in three hand-written kernels instead of the
// conversion kernel, two cuFFT transforms and the k-space kernel:
//
//   rows_fwd  fixed-point density -> float rho (background removed, charge
//             summed), then the real FFT of each row along x: two rows per
//             complex transform (z = rho_a + i rho_b; A_k = (Z_k + conj
//             Z_-k) / 2, B_k = (Z_k - conj Z_-k) / 2i), modes 0..nx/2 of
//             every row written column-major, S[kx][y];
//   cols      per column kx: FFT along y, the k-space operator of the
//             conversion-free solve (phi^ = rho^ / (eps0 k^2), E^ = -i k
//             phi^, Nyquist derivatives zeroed, Parseval field energy,
//             tracked mode), inverse FFTs along y of phi^ and Ey^; Ex comes
//             from the inverse of phi^ times -i kx (kx is constant along a
//             column), written column-major Tx[kx][y], Ty[kx][y];
//   rows_inv  per row y: Z = Ex~ + i Ey~ extended to all nx modes by
//             Hermitian symmetry (imaginary parts at kx = 0 and nx/2
//             dropped, as a complex-to-real transform does), one inverse
//             complex FFT, Ex = Re z, Ey = Im z.
//
// The same launches serve an ensemble's runs of one grid size (blockIdx.y
// picks the run from the run table) and, in their adjoint mode, the
// adjoint's transposed solve psi = S^T g (rows of gx + i gy forward, two
// forward column transforms, the transposed k-space operator and one
// inverse per column, two psi rows per inverse row transform).
//
// The arithmetic per mode is the k-space kernel's (pic_field_dev.cuh); the
// transforms are pic_fft_dev.cuh's.  Replaces (reference paths inside
// taylorj5/msc-thesis, thesisCode/collisionless/double/src/):
//   fourier.cc:15-126 fftPoissonSolver, grid.cc:85-96 computeElectricField.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <vector>

#include "pic_adjoint_dev.cuh"
#include "pic_ensemble.cuh"
#include "pic_fft_dev.cuh"
#include "pic_field_dev.cuh"

namespace pic {

struct SpecArgs {
    const unsigned long long *rho_fix;
    float *rho;
    float2 *S;           // [nh][ny]: rows transformed along x
    float2 *Tx, *Ty;     // [nh][ny]: Ex~, Ey~ after the inverse along y
    float *ex, *ey;      // [ny][nx]
    const float2 *twx, *twy;
    int nx, ny, nh, lgx, lgy;
    long long mean_fix;
    float scale;
    float kx1, ky1, inv_eps0_n;
    int tmx, tmy;
    // adjoint solve (psi = S^T g): the two gradient planes in, their half
    // spectra in S and Sy, psi^ after the inverse along y in Tx; the inverse
    // rows take rows y ys and y ys + yo of Tx and Ty into ex and ey (ys = 1,
    // yo = 0 for the field; 2 and 1 for psi, two rows per transform)
    const float *gx, *gy;
    float2 *Sy;
    int ys, yo;
    int pairs, cols, rows;  // transforms (row pairs or rows), columns, rows per block
    int sa, sb, sc;         // buffer strides (float2) of the three kernels
    DevState *dev;
    // ensemble: blockIdx.y picks run first + blockIdx.y of this table, whose
    // grids sit at its offsets from the pointers above and whose constants
    // replace the ones above (nullptr: a single run)
    const EnsRun *runs;
    int first;
};

// the arguments of this block's run
__device__ __forceinline__ SpecArgs block_args(const SpecArgs &P)
{
    SpecArgs A = P;
    if (P.runs) {
        const int r = P.first + (int)blockIdx.y;
        const EnsRun &R = P.runs[r];
        A.rho_fix = P.rho_fix + R.goff;
        A.rho = P.rho + R.goff;
        A.S = P.S + R.khoff;
        A.Tx = P.Tx + R.khoff;
        A.Ty = P.Tx + R.khoff + R.nk;
        A.ex = P.ex + 2 * R.goff;
        A.ey = P.ex + 2 * R.goff + R.ncp;
        A.mean_fix = R.mean_fix;
        A.scale = R.rho_scale;
        A.kx1 = R.kx1;
        A.ky1 = R.ky1;
        A.inv_eps0_n = R.inv_eps0_n;
        A.dev = P.dev + r;
    }
    return A;
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) { return warp_sum_u64(v); }
__device__ __forceinline__ double warp_sum(double v) { return warp_sum_d(v); }

// Sum of v over the block, valid in thread 0.  Blocks of the small grids have
// fewer than 32 threads (a partial warp, where full-warp shuffles are not
// defined): their threads add through shared memory.  part: 32 entries.
template <class T>
__device__ __forceinline__ T block_sum(T v, T *part)
{
    if (blockDim.x >= 32) {
        v = warp_sum(v);
        if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
    } else {
        part[threadIdx.x] = v;
    }
    __syncthreads();
    T s = 0;
    if (threadIdx.x == 0) {
        const int np = blockDim.x >= 32 ? (int)(blockDim.x >> 5) : (int)blockDim.x;
        for (int w = 0; w < np; ++w) s += part[w];
    }
    return s;
}

// LGX: log2 nx.  Block: `pairs` transforms, nx/16 threads each: a pair of
// density rows, or with ADJ one row of the two gradient planes (gx + i gy).
template <int LGX, bool ADJ>
__global__ void __launch_bounds__(256) spec_rows_fwd_kernel(SpecArgs P)
{
    const SpecArgs A = block_args(P);
    constexpr int NX = 1 << LGX, TP = NX >> 4;
    extern __shared__ float2 smem[];
    __shared__ unsigned long long s_q[32];
    const int f = threadIdx.x / TP, t = threadIdx.x - f * TP;
    float2 *buf[1] = {smem + f * A.sa};
    float2 v[1][fft::E];
    unsigned long long qs = 0;
    if (ADJ) {
        const size_t r0 = (size_t)(blockIdx.x * A.pairs + f) * NX;
#pragma unroll
        for (int k = 0; k < fft::E; ++k)
            v[0][k] = make_float2(__ldg(A.gx + r0 + t + k * TP), __ldg(A.gy + r0 + t + k * TP));
    } else {
        // all loads first (the density is read-only here), then the
        // conversions and the float density's stores
        const size_t r0 = (size_t)(blockIdx.x * A.pairs + f) * 2 * NX;
        unsigned long long a[fft::E], b[fft::E];
#pragma unroll
        for (int k = 0; k < fft::E; ++k) {
            a[k] = __ldg(A.rho_fix + r0 + t + k * TP);
            b[k] = __ldg(A.rho_fix + r0 + NX + t + k * TP);
        }
#pragma unroll
        for (int k = 0; k < fft::E; ++k) {
            qs += a[k] + b[k];
            const float fa = fixed_to_float(a[k], A.mean_fix, A.scale);
            const float fb = fixed_to_float(b[k], A.mean_fix, A.scale);
            A.rho[r0 + t + k * TP] = fa;
            A.rho[r0 + NX + t + k * TP] = fb;
            v[0][k] = make_float2(fa, fb);
        }
    }
    fft::transform<LGX, false, 1>(v, buf, t, A.twx);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < fft::E; ++k) buf[0][fft::pad(fft::result_index<LGX>(k, t))] = v[0][k];
    __syncthreads();
    // split each transform's spectrum; (mode, transform) with the transform
    // fastest, so that the block's rows of one mode are written together
    const int np = A.pairs;
    for (int w = threadIdx.x; w < A.nh * np; w += blockDim.x) {
        const int ff = w % np, k = w / np;
        const float2 *bb = smem + ff * A.sa;
        const float2 z = bb[fft::pad(k)], m = bb[fft::pad((NX - k) & (NX - 1))];
        const float2 ra = make_float2(0.5f * (z.x + m.x), 0.5f * (z.y - m.y));
        const float2 rb = make_float2(0.5f * (z.y + m.y), 0.5f * (m.x - z.x));
        if (ADJ) {
            const size_t i = (size_t)k * A.ny + blockIdx.x * np + ff;
            A.S[i] = ra;
            A.Sy[i] = rb;
        } else {
            const int yy = (blockIdx.x * np + ff) * 2;
            *reinterpret_cast<float4 *>(A.S + (size_t)k * A.ny + yy) = make_float4(ra.x, ra.y, rb.x, rb.y);
        }
    }
    if (!ADJ) {
        qs = block_sum(qs, s_q);
        if (threadIdx.x == 0) atomicAdd(&A.dev->q[acc_slot()], qs);
    }
}

// LGY: log2 ny.  Block: `cols` columns, ny/16 threads each; two buffers per
// column (phi^, then Ey^).
template <int LGY, bool ADJ>
__global__ void __launch_bounds__(256, 2) spec_cols_kernel(SpecArgs P)
{
    const SpecArgs A = block_args(P);
    constexpr int NY = 1 << LGY, TP = NY >> 4;
    extern __shared__ float2 smem[];
    __shared__ double s_fe[32];
    const int c = threadIdx.x / TP, t = threadIdx.x - c * TP;
    const int mx = blockIdx.x * A.cols + c;
    const bool on = mx < A.nh;
    float2 *const b0 = smem + (2 * c) * A.sb, *const b1 = b0 + A.sb;
    const size_t col = (size_t)(on ? mx : 0) * NY;
    float fe = 0.f;
    float2 v[1][fft::E];
    // forward transform of column `src` along y, left in natural order in `bs`
    auto forward = [&](const float2 *src, float2 *bs) {
        float2 *buf[1] = {bs};
#pragma unroll
        for (int k = 0; k < fft::E; ++k)
            v[0][k] = on ? __ldg(src + col + t + k * TP) : make_float2(0.f, 0.f);
        fft::transform<LGY, false, 1>(v, buf, t, A.twy);
        __syncthreads();
#pragma unroll
        for (int k = 0; k < fft::E; ++k) bs[fft::pad(fft::result_index<LGY>(k, t))] = v[0][k];
        __syncthreads();
    };
    forward(A.S, b0);
    if (ADJ) {
        // psi^ = i (kx g^x + ky g^y) / (eps0 N k^2) per mode, inverse along y
        forward(A.Sy, b1);
#pragma unroll
        for (int k = 0; k < fft::E; ++k) {
            const int my = t + k * TP;
            v[0][k] = adj_mode(b0[fft::pad(my)], b1[fft::pad(my)], mx, my, A.nx, NY, A.kx1, A.ky1,
                               A.inv_eps0_n, mx == 0 && my == 0);
        }
        float2 *buf[1] = {b0};
        fft::transform<LGY, true, 1>(v, buf, t, A.twy);
        if (on) {
#pragma unroll
            for (int k = 0; k < fft::E; ++k) A.Tx[col + fft::result_index<LGY>(k, t)] = v[0][k];
        }
        return;
    }
    // k-space: phi^ stays in registers, Ey^ goes to the second buffer; the
    // two inverse transforms run one after the other
#pragma unroll
    for (int k = 0; k < fft::E; ++k) {
        const int my = t + k * TP;
        const float2 r = b0[fft::pad(my)];
        const KMode K = kspace_mode(r, mx, my, A.nx, NY, A.kx1, A.ky1, A.inv_eps0_n,
                                    mx == 0 && my == 0);
        if (on && mx == A.tmx && my == A.tmy)
            A.dev->mode_amp = sqrt((double)r.x * r.x + (double)r.y * r.y) / ((double)A.nx * NY);
        v[0][k] = K.ph;
        b1[fft::pad(my)] = K.ey;
        fe += on ? K.fe : 0.f;
    }
    // the two inverse transforms share one copy of the code: s = 0 turns
    // phi^ (registers, first buffer) into Ex~ = -i kx phi~ (Nyquist kx
    // zeroed), s = 1 turns Ey^ (second buffer) into Ey~
    const float kxe = (2 * mx == A.nx) ? 0.f : A.kx1 * (float)mx;
#pragma unroll 1
    for (int s = 0; s < 2; ++s) {
        float2 *const bs = s ? b1 : b0;
        if (s) {
            __syncthreads();  // Ey^ in the second buffer is complete
#pragma unroll
            for (int k = 0; k < fft::E; ++k) v[0][k] = b1[fft::pad(t + k * TP)];
        }
        float2 *buf[1] = {bs};
        fft::transform<LGY, true, 1>(v, buf, t, A.twy);
        if (on) {
            float2 *const out = (s ? A.Ty : A.Tx) + col;
#pragma unroll
            for (int k = 0; k < fft::E; ++k) {
                const float2 u = v[0][k];
                out[fft::result_index<LGY>(k, t)] = s ? u : make_float2(kxe * u.y, -kxe * u.x);
            }
        }
    }
    const double sum = block_sum((double)fe, s_fe);
    if (threadIdx.x == 0) atomicAdd(&A.dev->fe[acc_slot()], sum);
}

// LGX: log2 nx.  Block: `rows` transforms, nx/16 threads each: row y of Ex~
// and Ey~ into Ex and Ey, or rows 2y and 2y + 1 of psi~ into psi.
template <int LGX>
__global__ void __launch_bounds__(256) spec_rows_inv_kernel(SpecArgs P)
{
    const SpecArgs A = block_args(P);
    constexpr int NX = 1 << LGX, TP = NX >> 4, HALF = NX >> 1;
    extern __shared__ float2 smem[];
    const int f = threadIdx.x / TP, t = threadIdx.x - f * TP;
    const int nr = A.rows;
    const int y0 = blockIdx.x * nr;
    // (mode, row) with the row fastest: the block's rows of one mode are
    // adjacent in Tx and Ty.  nh nr = (8 + 16 / nx) times the block's
    // threads: at most 9 items per thread, all loads issued before the
    // shared-memory stores
    constexpr int ITEMS = 9;
    const int total = (HALF + 1) * nr;
    float2 X[ITEMS], Y[ITEMS];
#pragma unroll
    for (int q = 0; q < ITEMS; ++q) {
        const int w = threadIdx.x + q * blockDim.x;
        if (w < total) {
            const size_t i = (size_t)(w / nr) * A.ny + (size_t)(y0 + (w % nr)) * A.ys;
            X[q] = __ldg(A.Tx + i);
            Y[q] = __ldg(A.Ty + i + A.yo);
        }
    }
#pragma unroll
    for (int q = 0; q < ITEMS; ++q) {
        const int w = threadIdx.x + q * blockDim.x;
        if (w < total) {
            const int ff = w % nr, k = w / nr;
            float2 x = X[q], y = Y[q];
            if (k == 0 || k == HALF) x.y = y.y = 0.f;
            float2 *bb = smem + ff * A.sc;
            bb[fft::pad(k)] = make_float2(x.x - y.y, x.y + y.x);
            if (k > 0 && k < HALF) bb[fft::pad(NX - k)] = make_float2(x.x + y.y, y.x - x.y);
        }
    }
    __syncthreads();
    float2 v[1][fft::E];
    float2 *buf[1] = {smem + f * A.sc};
#pragma unroll
    for (int k = 0; k < fft::E; ++k) v[0][k] = buf[0][fft::pad(t + k * TP)];
    fft::transform<LGX, true, 1>(v, buf, t, A.twx);
    const size_t rx = (size_t)(y0 + f) * A.ys * NX, ry = rx + (size_t)A.yo * NX;
#pragma unroll
    for (int k = 0; k < fft::E; ++k) {
        const int i = fft::result_index<LGX>(k, t);
        A.ex[rx + i] = v[0][k].x;
        A.ey[ry + i] = v[0][k].y;
    }
}

static int pow2_floor(int n)
{
    int p = 1;
    while (2 * p <= n) p *= 2;
    return p;
}

static int ilog2(int n)
{
    int l = 0;
    while ((1 << l) < n) ++l;
    return l;
}

bool spectral_size_ok(int nx, int ny)
{
    auto ok = [](int n) { return n >= 16 && n <= 4096 && (n & (n - 1)) == 0; };
    return ok(nx) && ok(ny);
}

bool spectral_wanted(int nx, int ny)
{
    const char *solver = getenv("PIC_FIELD_SOLVER");
    return spectral_size_ok(nx, ny) && !(solver && strcmp(solver, "cufft") == 0);
}

// the transforms' per-pass twiddle tables (fft::twiddle_len entries for nx,
// then for ny): pass (lgns, lgr) with lgns > 0 holds W_(Ns R)^(r m) at
// r Ns + m, r < R, m < Ns
static void append_twiddles(std::vector<float2> &t, int lgn)
{
    const double pi = 3.14159265358979323846;
    for (int lgns = 0; lgns < lgn; lgns += fft::pass_lgr(lgn, lgns)) {
        if (lgns == 0) continue;
        const int R = 1 << fft::pass_lgr(lgn, lgns), Ns = 1 << lgns;
        for (int r = 0; r < R; ++r)
            for (int m = 0; m < Ns; ++m) {
                const double a = 2.0 * pi * (double)(r * m) / (double)(Ns * R);
                t.push_back(make_float2((float)std::cos(a), (float)-std::sin(a)));
            }
    }
}

pic_status spectral_twiddles(int nx, int ny, float2 **tw)
{
    std::vector<float2> t;
    append_twiddles(t, ilog2(nx));
    append_twiddles(t, ilog2(ny));
    t.push_back(make_float2(1.f, 0.f));  // never empty (16-point transforms need none)
    PIC_CUDA(cudaMalloc(tw, t.size() * sizeof(float2)));
    PIC_CUDA(cudaMemcpy(*tw, t.data(), t.size() * sizeof(float2), cudaMemcpyHostToDevice));
    return PIC_OK;
}

// The three kernels over `batch` runs of one grid size (A.runs set) or one
// run: the field solve, or with adj the adjoint solve (A.gx, A.gy -> psi in
// A.ex).  The caller clears the fixed-point density afterwards.
static pic_status launch_kernels(SpecArgs &A, int batch, cudaStream_t st, bool adj = false)
{
    const int nx = A.nx, ny = A.ny, nh = A.nh;
    A.lgx = ilog2(nx);
    A.lgy = ilog2(ny);
    A.twy = A.twx + fft::twiddle_len(A.lgx);
    A.ys = adj ? 2 : 1;
    A.yo = adj ? 1 : 0;
    const int tpx = nx >> 4, tpy = ny >> 4;
    // transforms of the forward and the inverse rows: row pairs and rows
    // (field), rows and row pairs (adjoint)
    const int na = adj ? ny : ny / 2, nc = adj ? ny / 2 : ny;
    // transforms per block: at most 256 threads, and no more than spreads the
    // batch's transforms over about one block per SM (small grids otherwise
    // run on a few SMs), but at least a warp's worth where the grid allows
    const int sms = device_sms();
    auto per_block = [&](int tp, int items) {
        const int spread = (int)std::max(1ll, (long long)items * batch / sms);
        int k = std::min(256 / tp, pow2_floor(spread));
        k = std::max(k, std::min(32 / tp, items));
        return std::max(1, std::min(k, items));
    };
    A.pairs = per_block(tpx, na);
    A.cols = per_block(tpy, nh);
    A.rows = per_block(tpx, nc);
    // interleaved buffers read by consecutive lanes start on different banks
    A.sa = fft::buf_stride(nx, 16 / std::min(A.pairs, 16));
    A.sb = fft::buf_stride(ny, 8);
    A.sc = fft::buf_stride(nx, 16 / std::min(A.rows, 16));
    const size_t ma = (size_t)A.pairs * A.sa * sizeof(float2);
    const size_t mb = (size_t)2 * A.cols * A.sb * sizeof(float2);
    const size_t mc = (size_t)A.rows * A.sc * sizeof(float2);
    const void *ka = nullptr, *kb = nullptr, *kc = nullptr;
    switch (A.lgx) {
#define PIC_SPEC_X(L)                                                                          \
    case L:                                                                                    \
        ka = adj ? (const void *)spec_rows_fwd_kernel<L, true>                                 \
                 : (const void *)spec_rows_fwd_kernel<L, false>;                               \
        kc = (const void *)spec_rows_inv_kernel<L>;                                            \
        break;
        PIC_SPEC_X(4) PIC_SPEC_X(5) PIC_SPEC_X(6) PIC_SPEC_X(7) PIC_SPEC_X(8) PIC_SPEC_X(9)
        PIC_SPEC_X(10) PIC_SPEC_X(11) PIC_SPEC_X(12)
#undef PIC_SPEC_X
    }
    switch (A.lgy) {
#define PIC_SPEC_Y(L)                                                                          \
    case L:                                                                                    \
        kb = adj ? (const void *)spec_cols_kernel<L, true> : (const void *)spec_cols_kernel<L, false>; \
        break;
        PIC_SPEC_Y(4) PIC_SPEC_Y(5) PIC_SPEC_Y(6) PIC_SPEC_Y(7) PIC_SPEC_Y(8) PIC_SPEC_Y(9)
        PIC_SPEC_Y(10) PIC_SPEC_Y(11) PIC_SPEC_Y(12)
#undef PIC_SPEC_Y
    }
    if (!ka || !kb || batch < 1) {
        set_error("spectral solve: grid side outside 16..4096");
        return PIC_ERR_INVALID_ARG;
    }
    PIC_TRY(allow_dynamic_smem(ka, ma));
    PIC_TRY(allow_dynamic_smem(kb, mb));
    PIC_TRY(allow_dynamic_smem(kc, mc));
    void *args[] = {&A};
    const unsigned nb = (unsigned)batch;
    PIC_CUDA(cudaLaunchKernel(ka, dim3(na / A.pairs, nb), dim3(A.pairs * tpx), args, ma, st));
    PIC_CUDA(cudaLaunchKernel(kb, dim3((nh + A.cols - 1) / A.cols, nb), dim3(A.cols * tpy), args,
                              mb, st));
    PIC_CUDA(cudaLaunchKernel(kc, dim3(nc / A.rows, nb), dim3(A.rows * tpx), args, mc, st));
    return PIC_OK;
}

pic_status launch_spectral(pic_handle *h)
{
    const Geometry &g = h->g;
    SpecArgs A;
    memset(&A, 0, sizeof A);
    A.rho_fix = h->rho_fix;
    A.rho = h->rho;
    A.S = h->rhohat;
    A.Tx = h->ehat;
    A.Ty = h->ehat + (size_t)g.nh * g.ny;
    A.ex = h->e;
    A.ey = h->e + (size_t)g.nx * g.ny;
    A.nx = g.nx;
    A.ny = g.ny;
    A.nh = g.nh;
    A.twx = h->tw;
    A.mean_fix = h->mean_fix;
    A.scale = (float)(h->q_unit / (4294967296.0 * g.dx * g.dy));
    A.kx1 = (float)(2.0 * 3.14159265358979323846 / g.Lx);
    A.ky1 = (float)(2.0 * 3.14159265358979323846 / g.Ly);
    A.inv_eps0_n = (float)(1.0 / (h->cfg.eps0 * (double)g.nx * (double)g.ny));
    A.tmx = h->track_mx;
    A.tmy = h->track_my;
    A.dev = h->dev;
    PIC_TRY(launch_kernels(A, 1, h->stream));
    PIC_CUDA(cudaMemsetAsync(h->rho_fix, 0, sizeof(unsigned long long) * (size_t)g.nx * g.ny,
                             h->stream));
    return PIC_OK;
}

pic_status launch_spectral_runs(const EnsRun *runs, int first, int count, int nx, int ny,
                                const unsigned long long *rho_fix, float *rho, float2 *rhohat,
                                float2 *ehat, float *e, const float2 *tw, DevState *devs,
                                cudaStream_t st)
{
    SpecArgs A;
    memset(&A, 0, sizeof A);
    A.rho_fix = rho_fix;
    A.rho = rho;
    A.S = rhohat;
    A.Tx = ehat;
    A.ex = e;
    A.nx = nx;
    A.ny = ny;
    A.nh = nx / 2 + 1;
    A.twx = tw;
    A.tmx = A.tmy = -1;
    A.dev = devs;
    A.runs = runs;
    // a grid's y dimension holds at most 65535 runs
    for (int b = 0; b < count; b += 65535) {
        A.first = first + b;
        PIC_TRY(launch_kernels(A, std::min(65535, count - b), st));
    }
    return PIC_OK;
}

// psi = S^T g on a power-of-two handle: gx, gy (ncell each) -> psi; gh
// (2 ny nh) and ph (ny nh) are scratch
pic_status launch_spectral_adjoint(pic_handle *h, const float *gx, const float *gy, float2 *gh,
                                   float2 *ph, float *psi)
{
    const Geometry &g = h->g;
    SpecArgs A;
    memset(&A, 0, sizeof A);
    A.gx = gx;
    A.gy = gy;
    A.S = gh;
    A.Sy = gh + (size_t)g.nh * g.ny;
    A.Tx = A.Ty = ph;
    A.ex = A.ey = psi;
    A.nx = g.nx;
    A.ny = g.ny;
    A.nh = g.nh;
    A.twx = h->tw;
    A.kx1 = (float)(2.0 * 3.14159265358979323846 / g.Lx);
    A.ky1 = (float)(2.0 * 3.14159265358979323846 / g.Ly);
    A.inv_eps0_n = (float)(1.0 / (h->cfg.eps0 * (double)g.nx * (double)g.ny));
    A.tmx = A.tmy = -1;
    A.dev = h->dev;
    return launch_kernels(A, 1, h->stream, true);
}

}  // namespace pic
