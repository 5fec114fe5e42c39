// pic_collide.cu -- collision operators: electron-neutral MCC (null-collision
// method) and neutral-neutral DSMC (Bird's no-time-counter scheme).
//
// Replace (taylorj5/msc-thesis, thesisCode/):
//   mccCollisions/src/particle.cc:112-127, mccCollisions/src/pic.cu:435-466
//     Bernoulli(0.8 / 0.22) resample v = 2(u1+u2+u3-1.5), no cross sections
//   dsmcCollisions/cellTrackerAdvanced/src/main.cc:288-350, src/pic.cu:791-870
//     nearest in-cell partner, fixed probability, +-(sum of uniforms)
// with the physical operators the configuration asks for.  Random numbers
// are Philox4x32-10 (pic_internal.cuh); MCC draws per particle id and
// collision pass, DSMC per cell, pass and candidate, so both are
// reproducible for a given particle or cell whatever the storage order.
#include <cuda_runtime.h>

#include "pic_internal.cuh"

namespace pic {

// ---------------------------------------------------------------- helpers
// orthonormal basis (e1, e2) perpendicular to unit u (Duff et al., "Building
// an orthonormal basis, revisited", JCGT 6(1), 2017)
__device__ __forceinline__ void perp_basis(float ux, float uy, float uz, float3 &e1, float3 &e2)
{
    const float sgn = copysignf(1.0f, uz);
    const float a = -1.0f / (sgn + uz);
    const float b = ux * uy * a;
    e1 = make_float3(1.0f + sgn * ux * ux * a, sgn * b, -sgn * ux);
    e2 = make_float3(b, sgn + uy * uy * a, -uy);
}

// unit vector at polar angle chi (cos chi = c) and azimuth 2 pi w about u
__device__ __forceinline__ float3 deflect(float ux, float uy, float uz, float c, float w)
{
    float3 e1, e2;
    perp_basis(ux, uy, uz, e1, e2);
    const float s = sqrtf(fmaxf(0.0f, 1.0f - c * c));
    float sp, cp;
    sincospif(2.0f * w, &sp, &cp);
    return make_float3(c * ux + s * (cp * e1.x + sp * e2.x), c * uy + s * (cp * e1.y + sp * e2.y),
                       c * uz + s * (cp * e1.z + sp * e2.z));
}

// ---------------------------------------------------------------- MCC
struct MccArgs {
    int32_t *ecell;
    float *eox, *eoy, *evx, *evy, *evz;
    uint32_t *epid;
    long long *d_ne;
    long long ecap;
    int32_t *icell;
    float *iox, *ioy, *ivx, *ivy, *ivz;
    uint32_t *ipid;
    long long *d_ni;
    long long icap;
    int has_ion;
    const float *tab;   // [energy | elastic | excitation | ionisation] x ntab
    int ntab;
    float ln_emin, inv_dln;
    float half_me_over_e;  // E[eV] = half_me_over_e * |v|^2
    float ng, nu_max, p_null, two_m_over_M;
    float e_exc, e_ion, vth_ion;
    uint32_t k0, k1;
    DevState *dev;
};

__device__ __forceinline__ void mcc_sigmas(const MccArgs &A, const float *tab, float E,
                                           float &sel, float &sexc, float &sion)
{
    const int nt = A.ntab;
    int k;
    float f;
    if (E <= tab[0]) {
        k = 0;
        f = 0.f;
    } else if (E >= tab[nt - 1]) {
        k = nt - 2;
        f = 1.f;
    } else {
        k = (int)((__logf(E) - A.ln_emin) * A.inv_dln);
        k = min(max(k, 0), nt - 2);
        // the log index can be off by one near a table point; fix it exactly
        if (E < tab[k]) k = max(k - 1, 0);
        if (E >= tab[k + 1]) k = min(k + 1, nt - 2);
        f = (E - tab[k]) / (tab[k + 1] - tab[k]);
    }
    const float *el = tab + nt, *ex = tab + 2 * nt, *io = tab + 3 * nt;
    sel = fmaf(f, el[k + 1] - el[k], el[k]);
    sexc = fmaf(f, ex[k + 1] - ex[k], ex[k]);
    sion = fmaf(f, io[k + 1] - io[k], io[k]);
}

constexpr int MCC_THREADS = 256;
constexpr int MCC_PER_THREAD = 8;
constexpr int MCC_CHUNK = MCC_THREADS * MCC_PER_THREAD;  // electrons tested per block pass

// Collision of candidate electron i (r: its first draw of this pass):
// real (elastic, excitation, ionisation with ion birth) or null.
__device__ __forceinline__ void mcc_collide(const MccArgs &A, const float *s_tab, long long i,
                                            uint32_t pid, unsigned long long pass, const U4 &r,
                                            unsigned &c_el, unsigned &c_exc, unsigned &c_ion,
                                            unsigned &c_null, bool &overflow)
{
    float vx = A.evx[i], vy = A.evy[i], vz = A.evz[i];
    const float v2 = vx * vx + vy * vy + vz * vz;
    const float v = sqrtf(v2);
    const float E = A.half_me_over_e * v2;
    float sel, sexc, sion;
    mcc_sigmas(A, s_tab, E, sel, sexc, sion);
    if (E < A.e_exc) sexc = 0.f;
    if (E < A.e_ion) sion = 0.f;
    const float nu_el = A.ng * sel * v, nu_exc = A.ng * sexc * v, nu_ion = A.ng * sion * v;
    const float R = u01f(r.y) * A.nu_max;
    const float ux = v > 0.f ? vx / v : 0.f, uy = v > 0.f ? vy / v : 0.f;
    const float uz = v > 0.f ? vz / v : 1.f;
    if (R < nu_el) {
        const float c = 1.f - 2.f * u01f(r.z);
        const float En = E * (1.f - A.two_m_over_M * (1.f - c));
        const float3 d = deflect(ux, uy, uz, c, u01f(r.w));
        const float vn = sqrtf(En / A.half_me_over_e);
        vx = vn * d.x;
        vy = vn * d.y;
        vz = vn * d.z;
        ++c_el;
    } else if (R < nu_el + nu_exc) {
        const float c = 1.f - 2.f * u01f(r.z);
        const float3 d = deflect(ux, uy, uz, c, u01f(r.w));
        const float vn = sqrtf(fmaxf(E - A.e_exc, 0.f) / A.half_me_over_e);
        vx = vn * d.x;
        vy = vn * d.y;
        vz = vn * d.z;
        ++c_exc;
    } else if (R < nu_el + nu_exc + nu_ion) {
        const U4 r2 = philox4x32_10(U4{pid, (uint32_t)pass, 1u, STREAM_MCC}, A.k0, A.k1);
        const float Er = fmaxf(E - A.e_ion, 0.f);
        const float Ej = u01f(r2.x) * Er, Es = Er - Ej;
        const float3 ds = deflect(ux, uy, uz, 1.f - 2.f * u01f(r.z), u01f(r.w));
        const float3 dj = deflect(ux, uy, uz, 1.f - 2.f * u01f(r2.y), u01f(r2.z));
        const float vs = sqrtf(Es / A.half_me_over_e), vj = sqrtf(Ej / A.half_me_over_e);
        vx = vs * ds.x;
        vy = vs * ds.y;
        vz = vs * ds.z;
        ++c_ion;
        if (A.has_ion) {
            // reserve the ion slot, then the electron slot; a reservation past
            // the capacity is given back, so the successful slots stay
            // contiguous from the old count
            const long long ji = (long long)atomicAdd((unsigned long long *)A.d_ni, 1ull);
            long long je = A.ecap;
            if (ji < A.icap) je = (long long)atomicAdd((unsigned long long *)A.d_ne, 1ull);
            if (ji < A.icap && je < A.ecap) {
                A.ecell[je] = A.ecell[i];
                A.eox[je] = A.eox[i];
                A.eoy[je] = A.eoy[i];
                A.evx[je] = vj * dj.x;
                A.evy[je] = vj * dj.y;
                A.evz[je] = vj * dj.z;
                A.epid[je] = (uint32_t)je;
                const U4 r3 = philox4x32_10(U4{pid, (uint32_t)pass, 2u, STREAM_MCC}, A.k0, A.k1);
                const float ra = sqrtf(-2.f * __logf(u01f(r3.x))), rb = sqrtf(-2.f * __logf(u01f(r3.z)));
                float sa, ca, sb, cb;
                sincospif(2.f * u01f(r3.y), &sa, &ca);
                sincospif(2.f * u01f(r3.w), &sb, &cb);
                A.icell[ji] = A.ecell[i];
                A.iox[ji] = A.eox[i];
                A.ioy[ji] = A.eoy[i];
                A.ivx[ji] = A.vth_ion * ra * ca;
                A.ivy[ji] = A.vth_ion * ra * sa;
                A.ivz[ji] = A.vth_ion * rb * cb;
                A.ipid[ji] = (uint32_t)ji;
            } else {
                // no room: give back what was reserved and report; an ion slot
                // whose electron did not fit stays empty (cell -1)
                if (ji >= A.icap) {
                    atomicAdd((unsigned long long *)A.d_ni, (unsigned long long)-1ll);
                } else {
                    atomicAdd((unsigned long long *)A.d_ne, (unsigned long long)-1ll);
                    A.icell[ji] = -1;
                    A.ipid[ji] = (uint32_t)ji;
                }
                overflow = true;
            }
        }
    } else {
        ++c_null;
        return;
    }
    A.evx[i] = vx;
    A.evy[i] = vy;
    A.evz[i] = vz;
}

// One null-collision pass over the electrons present at its start.  Each
// block takes MCC_CHUNK electrons at a time: first every electron draws its
// candidate test (one Philox draw keyed by particle id and pass) and the
// candidates (fraction P_null, a few percent) are queued in shared memory,
// then the block's threads work through the queue together, so the costly
// collision path runs in full warps instead of one lane per warp.  A thread
// loads the cells and ids of all its electrons of a chunk before the first
// draw, so that their DRAM reads overlap.
__global__ void __launch_bounds__(MCC_THREADS) mcc_kernel(MccArgs A)
{
    extern __shared__ float s_tab[];  // 4 ntab table floats, then the candidate queue
    int *s_q = reinterpret_cast<int *>(s_tab + 4 * A.ntab);
    for (int i = threadIdx.x; i < 4 * A.ntab; i += blockDim.x) s_tab[i] = A.tab[i];
    __shared__ unsigned long long s_cnt[4];
    __shared__ unsigned s_nq;
    if (threadIdx.x < 4) s_cnt[threadIdx.x] = 0ull;
    __syncthreads();
    // the count at the start of the pass: electrons born in this pass are not
    // candidates (blocks that start late would otherwise see them)
    const long long n = min(A.dev->mcc_n0, A.ecap);
    const unsigned long long pass = A.dev->mcc_pass;
    unsigned c_el = 0, c_exc = 0, c_ion = 0, c_null = 0;
    bool overflow = false;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    for (long long c0 = (long long)blockIdx.x * MCC_CHUNK; c0 < n;
         c0 += (long long)gridDim.x * MCC_CHUNK) {
        if (threadIdx.x == 0) s_nq = 0u;
        __syncthreads();
        int cellv[MCC_PER_THREAD];
        uint32_t pidv[MCC_PER_THREAD];
#pragma unroll
        for (int j = 0; j < MCC_PER_THREAD; ++j) {
            const long long i = c0 + threadIdx.x + j * MCC_THREADS;
            cellv[j] = i < n ? A.ecell[i] : -1;
            pidv[j] = i < n ? A.epid[i] : 0u;
        }
#pragma unroll
        for (int j = 0; j < MCC_PER_THREAD; ++j) {  // warp-uniform trip count
            const int k = threadIdx.x + j * MCC_THREADS;
            bool cand = false;
            if (cellv[j] >= 0) {
                const U4 r = philox4x32_10(U4{pidv[j], (uint32_t)pass, 0u, STREAM_MCC}, A.k0, A.k1);
                cand = u01f(r.x) < A.p_null;
            }
            const unsigned m = __ballot_sync(full, cand);
            if (m) {
                unsigned base = 0u;
                if (lane == 0) base = atomicAdd(&s_nq, (unsigned)__popc(m));
                base = __shfl_sync(full, base, 0);
                if (cand) s_q[base + __popc(m & ((1u << lane) - 1u))] = k;
            }
        }
        __syncthreads();
        const int nq = (int)s_nq;
        for (int j = threadIdx.x; j < nq; j += blockDim.x) {
            const long long i = c0 + s_q[j];
            const uint32_t pid = A.epid[i];
            const U4 r = philox4x32_10(U4{pid, (uint32_t)pass, 0u, STREAM_MCC}, A.k0, A.k1);
            mcc_collide(A, s_tab, i, pid, pass, r, c_el, c_exc, c_ion, c_null, overflow);
        }
        __syncthreads();  // the queue is reused by the next chunk
    }
    atomicAdd(&s_cnt[0], (unsigned long long)c_el);
    atomicAdd(&s_cnt[1], (unsigned long long)c_exc);
    atomicAdd(&s_cnt[2], (unsigned long long)c_ion);
    atomicAdd(&s_cnt[3], (unsigned long long)c_null);
    const int any_over = __syncthreads_or(overflow ? 1 : 0);
    if (threadIdx.x < 4) atomicAdd(&A.dev->coll[threadIdx.x][acc_slot()], s_cnt[threadIdx.x]);
    if (threadIdx.x == 0 && any_over) atomicOr(&A.dev->err, (unsigned)PIC_DEVERR_CAPACITY);
}

// ---------------------------------------------------------------- DSMC
struct NtcArgs {
    float *vx, *vy, *vz;      // the species' sorted buffer
    const uint32_t *offset;   // per key: particles [offset[k], offset[k+1])
    float *sgmax;             // per key (sigma g)_max
    long long nkeys;
    long long nslots;         // slots of the sorted buffer (bound of the offsets)
    float sigma;              // pi d^2
    float coef;               // F_N dt_c / (2 V_c)
    uint32_t k0, k1;
    DevState *dev;
};

__global__ void __launch_bounds__(256) ntc_kernel(NtcArgs A)
{
    __shared__ unsigned long long s_cnt[2];
    if (threadIdx.x < 2) s_cnt[threadIdx.x] = 0ull;
    __syncthreads();
    const unsigned long long pass = A.dev->dsmc_pass;
    unsigned ncoll = 0, ncand = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long key = (long long)blockIdx.x * blockDim.x + threadIdx.x; key < A.nkeys;
         key += stride) {
        const uint32_t o0 = A.offset[key], o1 = A.offset[key + 1];
        if (o1 < o0 || (long long)o1 > A.nslots) {  // offsets that do not fit the slots
            atomicOr(&A.dev->err, (unsigned)PIC_DEVERR_SORT);
            continue;
        }
        const uint32_t n = o1 - o0;
        if (n < 2) continue;
        float sgm = A.sgmax[key];
        const float want = A.coef * (float)n * (float)(n - 1) * sgm;
        const U4 r0 = philox4x32_10(U4{(uint32_t)key, (uint32_t)pass, 0u, STREAM_DSMC}, A.k0, A.k1);
        const float fl = floorf(want);
        const uint32_t nc = (uint32_t)fl + (u01f(r0.x) < want - fl ? 1u : 0u);
        for (uint32_t c = 0; c < nc; ++c) {
            const U4 r = philox4x32_10(U4{(uint32_t)key, (uint32_t)pass, 2u * c + 1u, STREAM_DSMC},
                                       A.k0, A.k1);
            uint32_t a = min((uint32_t)(u01f(r.x) * (float)n), n - 1);
            uint32_t b = min((uint32_t)(u01f(r.y) * (float)(n - 1)), n - 2);
            if (b >= a) ++b;
            const uint32_t i = o0 + a, j = o0 + b;
            const float gx = A.vx[i] - A.vx[j], gy = A.vy[i] - A.vy[j], gz = A.vz[i] - A.vz[j];
            const float g = sqrtf(gx * gx + gy * gy + gz * gz);
            const float sg = A.sigma * g;
            if (sg > sgm) sgm = sg;
            ++ncand;
            if (u01f(r.z) * sgm >= sg) continue;
            // hard spheres: isotropic post-collision relative velocity in the CM frame
            const U4 r2 = philox4x32_10(U4{(uint32_t)key, (uint32_t)pass, 2u * c + 2u, STREAM_DSMC},
                                        A.k0, A.k1);
            const float cx = 2.f * u01f(r.w) - 1.f;
            const float sx = sqrtf(fmaxf(0.f, 1.f - cx * cx));
            float sp, cp;
            sincospif(2.f * u01f(r2.x), &sp, &cp);
            const float hx = 0.5f * g * cx, hy = 0.5f * g * sx * cp, hz = 0.5f * g * sx * sp;
            const float mx = 0.5f * (A.vx[i] + A.vx[j]), my = 0.5f * (A.vy[i] + A.vy[j]);
            const float mz = 0.5f * (A.vz[i] + A.vz[j]);
            A.vx[i] = mx + hx;
            A.vy[i] = my + hy;
            A.vz[i] = mz + hz;
            A.vx[j] = mx - hx;
            A.vy[j] = my - hy;
            A.vz[j] = mz - hz;
            ++ncoll;
        }
        A.sgmax[key] = sgm;
    }
    atomicAdd(&s_cnt[0], (unsigned long long)ncoll);
    atomicAdd(&s_cnt[1], (unsigned long long)ncand);
    __syncthreads();
    if (threadIdx.x == 0) {
        atomicAdd(&A.dev->coll[4][acc_slot()], s_cnt[0]);
        atomicAdd(&A.dev->coll[5][acc_slot()], s_cnt[1]);
    }
}

__global__ void bump_kernel(unsigned long long *counter) { *counter += 1ull; }

// opens an MCC pass: new pass number and the electron count it works on
__global__ void mcc_prepare_kernel(DevState *d, int e)
{
    d->mcc_pass += 1ull;
    d->mcc_n0 = d->n[e];
}

// ---------------------------------------------------------------- launchers
pic_status launch_mcc(pic_handle *h)
{
    const MccState &M = h->mcc;
    SpeciesBuf &E = h->sp[M.e];
    MccArgs A;
    memset(&A, 0, sizeof A);
    A.ecell = E.cell[0];
    A.eox = E.ox[0];
    A.eoy = E.oy[0];
    A.evx = E.vx[0];
    A.evy = E.vy[0];
    A.evz = E.vz[0];
    A.epid = E.pid[0];
    A.d_ne = &h->dev->n[M.e];
    A.ecap = E.cap;
    if (M.i >= 0) {
        SpeciesBuf &I = h->sp[M.i];
        A.icell = I.cell[0];
        A.iox = I.ox[0];
        A.ioy = I.oy[0];
        A.ivx = I.vx[0];
        A.ivy = I.vy[0];
        A.ivz = I.vz[0];
        A.ipid = I.pid[0];
        A.d_ni = &h->dev->n[M.i];
        A.icap = I.cap;
        A.has_ion = 1;
    }
    A.tab = M.tab;
    A.ntab = M.ntab;
    A.ln_emin = M.ln_emin;
    A.inv_dln = M.inv_dln;
    A.half_me_over_e = M.half_me_over_e;
    A.ng = M.ng;
    A.nu_max = M.nu_max;
    A.p_null = M.p_null;
    A.two_m_over_M = M.two_m_over_M;
    A.e_exc = M.e_exc;
    A.e_ion = M.e_ion;
    A.vth_ion = M.vth_ion;
    A.k0 = (uint32_t)M.seed;
    A.k1 = (uint32_t)(M.seed >> 32);
    A.dev = h->dev;
    mcc_prepare_kernel<<<1, 1, 0, h->stream>>>(h->dev, M.e);
    PIC_CUDA(cudaGetLastError());
    mcc_kernel<<<grid_for(E.cap, MCC_CHUNK), MCC_THREADS,
                 4 * M.ntab * sizeof(float) + MCC_CHUNK * sizeof(int), h->stream>>>(A);
    PIC_CUDA(cudaGetLastError());
    return PIC_OK;
}

// DSMC pass on species D.s, which must have just been sorted (buffer 1, offsets)
pic_status launch_ntc(pic_handle *h)
{
    const DsmcState &D = h->dsmc;
    SpeciesBuf &B = h->sp[D.s];
    NtcArgs A;
    A.vx = B.vx[1];
    A.vy = B.vy[1];
    A.vz = B.vz[1];
    A.offset = h->offset;
    A.sgmax = D.sgmax;
    A.nkeys = (long long)h->g.nx * h->g.ny;
    A.nslots = B.cap;
    A.sigma = D.sigma;
    A.coef = D.coef;
    A.k0 = (uint32_t)D.seed;
    A.k1 = (uint32_t)(D.seed >> 32);
    A.dev = h->dev;
    ntc_kernel<<<grid_for(A.nkeys, 256), 256, 0, h->stream>>>(A);
    PIC_CUDA(cudaGetLastError());
    bump_kernel<<<1, 1, 0, h->stream>>>(&h->dev->dsmc_pass);
    PIC_CUDA(cudaGetLastError());
    return PIC_OK;
}

}  // namespace pic
