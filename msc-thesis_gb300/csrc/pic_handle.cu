// pic_handle.cu -- host side of libpic: configuration, device buffers,
// cuFFT plans, CUDA-graph capture of the step and the C ABI of the handle.
//
// The reference keeps everything inside one function (picFloatGpu,
// taylorj5/msc-thesis thesisCode/collisionless/double/src/pic.cu:429-611:
// allocate, copy in, loop, copy out, free).  Here a handle owns its stream and
// buffers across calls; the step's launches are captured once into CUDA
// graphs and replayed (see pic_step).
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "pic_internal.cuh"

namespace pic {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

pic_status cuda_fail(cudaError_t e, const char *what)
{
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    cudaGetLastError();  // clear a non-sticky error
    return (e == cudaErrorMemoryAllocation) ? PIC_ERR_OOM
           : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? PIC_ERR_NO_DEVICE
                                                                           : PIC_ERR_CUDA;
}

pic_status cufft_fail(cufftResult r, const char *what)
{
    char buf[64];
    snprintf(buf, sizeof buf, ": cufftResult %d", (int)r);
    set_error(std::string(what) + buf);
    return (r == CUFFT_ALLOC_FAILED) ? PIC_ERR_OOM : PIC_ERR_CUFFT;
}

int device_sms()
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            sms <= 0)
            sms = 152;
    }
    return sms;
}

int grid_for(long long n, int block)
{
    const int sms = device_sms();
    long long b = (n + block - 1) / block;
    const long long cap = (long long)sms * 8;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

int pick_divisor(int n, int target)
{
    if (target < 1) target = 1;
    if (target > n) target = n;
    int best = 1;
    for (int d = 1; d <= n; ++d)
        if (n % d == 0 && std::abs(d - target) < std::abs(best - target)) best = d;
    return best;
}

// Tile height for a tile of about `tcells` cells and width tw: the divisor
// of ny nearest to tcells / tw by ratio (so 6.4 gives 8, not 4: at 512^2 x
// 64 particles per cell in 8192-particle chunks, 16 x 8 tiles took 0.470 ms
// per step against 0.488 ms with 16 x 4).
int pick_tile_h(int ny, int tcells, int tw)
{
    const double target = std::max(1.0, (double)tcells / (double)tw);
    int best = 1;
    double bd = 1e300;
    for (int d = 1; d <= ny; ++d) {
        if (ny % d) continue;
        const double e = std::fabs(std::log((double)d / target));
        if (e < bd - 1e-12) {
            bd = e;
            best = d;
        }
    }
    return best;
}

static void free_handle_buffers(pic_handle *h)
{
    for (int s = 0; s < PIC_MAX_SPECIES; ++s) {
        SpeciesBuf &B = h->sp[s];
        for (int b = 0; b < 2; ++b) {
            cudaFree(B.cell[b]);
            cudaFree(B.ox[b]);
            cudaFree(B.oy[b]);
            cudaFree(B.vx[b]);
            cudaFree(B.vy[b]);
            cudaFree(B.vz[b]);
            cudaFree(B.pid[b]);
        }
        cudaFree(B.anchor);
        B = SpeciesBuf();
    }
    cudaFree(h->rho_fix);
    cudaFree(h->rho);
    cudaFree(h->rhohat);
    cudaFree(h->ehat);
    cudaFree(h->e);
    cudaFree(h->tw);
    cudaFree(h->count);
    cudaFree(h->offset);
    cudaFree(h->cursor);
    cudaFree(h->bsum);
    cudaFree(h->dev);
    cudaFree(h->hist);
    cudaFree(h->stage);
    cudaFree(h->mcc.tab);
    cudaFree(h->dsmc.sgmax);
    cudaFree(h->dsmc.count);
    if (h->plan_r2c) cufftDestroy(h->plan_r2c);
    if (h->plan_c2r2) cufftDestroy(h->plan_c2r2);
    if (h->plan_c2r1) cufftDestroy(h->plan_c2r1);
    if (h->g_period) cudaGraphExecDestroy(h->g_period);
    if (h->g_sortstep) cudaGraphExecDestroy(h->g_sortstep);
    if (h->g_one) cudaGraphExecDestroy(h->g_one);
    if (h->cub_temp) cudaFree(h->cub_temp);
    for (auto &e : h->field_ready)
        if (e) cudaEventDestroy(e);
    if (h->copies_done) cudaEventDestroy(h->copies_done);
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    if (h->stream) cudaStreamDestroy(h->stream);
}

template <class T> static pic_status dalloc(T **p, size_t n)
{
    *p = nullptr;
    if (n == 0) return PIC_OK;
    PIC_CUDA(cudaMalloc((void **)p, n * sizeof(T)));
    return PIC_OK;
}

static pic_status validate(const pic_config *c, pic_handle *h)
{
    auto bad = [](const char *m) {
        set_error(std::string("pic_create: ") + m);
        return PIC_ERR_INVALID_ARG;
    };
    if (c->nx < 2 || c->ny < 2 || c->nx > 32768 || c->ny > 32768)
        return bad("nx, ny must be in [2, 32768]");
    if ((long long)c->nx * c->ny > (1ll << 24) - 1) return bad("nx*ny must be < 2^24");
    if (!(c->Lx > 0) || !(c->Ly > 0) || !(c->dt > 0) || !(c->eps0 > 0))
        return bad("Lx, Ly, dt, eps0 must be positive");
    if (c->nspecies < 1 || c->nspecies > PIC_MAX_SPECIES) return bad("nspecies out of range");
    h->q_unit = 0.0;
    for (int s = 0; s < c->nspecies; ++s) {
        const pic_species_desc &S = c->species[s];
        if (S.capacity < 0 || S.capacity > (1ll << 31) - 4096) return bad("species capacity out of range");
        if (!(S.m > 0)) return bad("species mass must be positive");
        if ((S.q == 0.0) != (S.q_int == 0)) return bad("q == 0 exactly when q_int == 0");
        if (S.q_int != 0) {
            const double u = S.q / S.q_int;
            if (!(u > 0)) return bad("q and q_int must have the same sign");
            if (h->q_unit == 0.0)
                h->q_unit = u;
            else if (std::fabs(u - h->q_unit) > 1e-12 * h->q_unit)
                return bad("species charges are not integer multiples of one unit charge");
        }
    }
    if (h->q_unit == 0.0) h->q_unit = 1.0;
    if (c->chunk < 0 || (c->chunk % 4) != 0 || c->chunk > MAX_CHUNK)
        return bad("chunk must be a multiple of 4 and at most 32768");
    if (c->sort_every < 0 || c->halo < 0 || c->history < 0) return bad("negative tuning value");
    if (c->push_variant != 0 && c->push_variant != 1 && c->push_variant != 3)
        return bad("push_variant must be 0, 1 or 3");
    if (c->tile_w < 0 || c->tile_h < 0 || (c->tile_w && c->nx % c->tile_w) ||
        (c->tile_h && c->ny % c->tile_h))
        return bad("tile_w, tile_h must divide nx, ny");
    return PIC_OK;
}

static pic_status setup_geometry(pic_handle *h)
{
    const pic_config &c = h->cfg;
    Geometry &g = h->g;
    g.nx = c.nx;
    g.ny = c.ny;
    g.nh = c.nx / 2 + 1;
    g.Lx = c.Lx;
    g.Ly = c.Ly;
    g.dx = c.Lx / c.nx;
    g.dy = c.Ly / c.ny;
    g.chunk = c.chunk ? c.chunk : 8192;
    // default halo: the particles' drift between sorts grows with the cadence
    // (2048^2 x 32 ppc, sort every 40: 1.203 ms per step with 4 cells against
    // 1.234 with 2, 1.216 with 3, 1.211 with 5 or 6, 1.300 with 8; sort every
    // 20: 1.100 ms with 3 against 1.106 with 4), less where the window would
    // not fit
    const int every = c.sort_every ? c.sort_every : 20;
    g.halo = c.halo ? c.halo : (every <= 20 ? 3 : 4);
    long long maxcap = 0;
    for (int s = 0; s < c.nspecies; ++s) maxcap = std::max(maxcap, c.species[s].capacity);
    const double ppc = std::max(1.0, (double)maxcap / ((double)c.nx * c.ny));
    const int tcells = std::max(1, (int)std::lround(g.chunk / ppc));
    g.tw = c.tile_w ? c.tile_w : pick_divisor(c.nx, std::min(16, tcells));
    g.th = c.tile_h ? c.tile_h : pick_tile_h(c.ny, tcells, g.tw);
    g.ntx = c.nx / g.tw;
    g.nty = c.ny / g.th;
    auto window = [&] {
        g.wcx = 2 * g.tw + 2 * g.halo;
        g.wcy = g.th + 2 * g.halo;
        return window_bytes(g.wcx, g.wcy) + 32;
    };
    size_t smem = window();
    while (!c.halo && smem > WINDOW_SMEM_TARGET && g.halo > 1) {
        --g.halo;
        smem = window();
    }
    if (smem > WINDOW_SMEM_MAX) {
        set_error("pic_create: shared-memory window too large; use smaller tiles or halo");
        return PIC_ERR_INVALID_ARG;
    }
    return PIC_OK;
}

static pic_status reset_device_state(pic_handle *h)
{
    DevState z;
    memset(&z, 0, sizeof z);
    for (int s = 0; s < PIC_MAX_SPECIES; ++s) z.n[s] = h->sp[s].n;
    PIC_CUDA(cudaMemcpyAsync(h->dev, &z, sizeof z, cudaMemcpyHostToDevice, h->stream));
    PIC_CUDA(cudaMemsetAsync(h->hist, 0, sizeof(double) * 6 * (size_t)h->hist_cap, h->stream));
    PIC_CUDA(cudaStreamSynchronize(h->stream));  // z lives on this stack frame
    h->steps_host = 0;
    return PIC_OK;
}

// Background: mean fixed-point density per node, so that the float density
// carries only the deviation from it.  Exact integer arithmetic; the rest of
// a non-integer mean sits in the zero mode, which the solve removes.
static void update_mean(pic_handle *h)
{
    __int128 total = 0;
    for (int s = 0; s < h->cfg.nspecies; ++s)
        total += (__int128)h->cfg.species[s].q_int * h->sp[s].n * ((__int128)1 << 32);
    const __int128 nc = (__int128)h->g.nx * h->g.ny;
    h->mean_fix = (long long)(total / nc);
}

// ---------------------------------------------------------------- stages
// adv: the diagnostics folds to launch after the solve (ADV_FIELD, or
// ADV_PUSH | ADV_FIELD when the particle pass left its fold to this launch)
pic_status record_poisson(pic_handle *h, int adv)
{
    if (h->spectral) {
        PIC_TRY(launch_spectral(h));
    } else {
        PIC_TRY(launch_convert(h));
        PIC_CUFFT(cufftExecR2C(h->plan_r2c, h->rho, (cufftComplex *)h->rhohat));
        PIC_TRY(launch_kspace(h, false, nullptr));
        PIC_CUFFT(cufftExecC2R(h->plan_c2r2, (cufftComplex *)h->ehat, h->e));
    }
    PIC_TRY(launch_advance(h, adv));
    return PIC_OK;
}

// Particle pass of one step.  src = 1: every species was just sorted into
// buffer 1.  A DSMC species is sorted every step and collides on its sorted
// buffer before its push moves it back; MCC follows the push.
pic_status record_push_all(pic_handle *h, int src, bool deposit, bool fold)
{
    for (int s = 0; s < h->cfg.nspecies; ++s) {
        if (!h->sp[s].cap) continue;
        int from = src;
        if (h->dsmc.on && s == h->dsmc.s) {
            if (!src) PIC_TRY(launch_sort(h, s, true));  // counts kept by its last push
            PIC_TRY(launch_ntc(h));
            from = 1;
        }
        PIC_TRY(launch_push(h, s, from, deposit, 1.0f));
    }
    if (fold) PIC_TRY(launch_advance(h, ADV_PUSH));
    if (h->mcc.on) PIC_TRY(launch_mcc(h));
    return PIC_OK;
}

// One step.  Without MCC (whose pass starts from the folded counts) the
// particle pass's fold rides on the field's: one launch fewer per step.
static pic_status record_step(pic_handle *h, int src)
{
    const bool merge = !h->mcc.on;
    PIC_TRY(record_push_all(h, src, true, !merge));
    PIC_TRY(record_poisson(h, merge ? (ADV_PUSH | ADV_FIELD) : ADV_FIELD));
    return PIC_OK;
}

// Sort every species; the DSMC species goes last so that the cell offsets it
// collides on are the ones left in the shared sort buffers.
static pic_status record_sort_all(pic_handle *h)
{
    for (int s = 0; s < h->cfg.nspecies; ++s)
        if (h->sp[s].cap && !(h->dsmc.on && s == h->dsmc.s)) PIC_TRY(launch_sort(h, s));
    if (h->dsmc.on && h->sp[h->dsmc.s].cap) PIC_TRY(launch_sort(h, h->dsmc.s));
    return PIC_OK;
}

// Sorted data lives in buffer 1 after launch_sort; bring it back to 0.
static pic_status copy_back(pic_handle *h, int s)
{
    SpeciesBuf &B = h->sp[s];
    const size_t n = (size_t)B.cap;
    if (!n) return PIC_OK;
    cudaStream_t st = h->stream;
    PIC_CUDA(cudaMemcpyAsync(B.cell[0], B.cell[1], n * 4, cudaMemcpyDeviceToDevice, st));
    PIC_CUDA(cudaMemcpyAsync(B.ox[0], B.ox[1], n * 4, cudaMemcpyDeviceToDevice, st));
    PIC_CUDA(cudaMemcpyAsync(B.oy[0], B.oy[1], n * 4, cudaMemcpyDeviceToDevice, st));
    PIC_CUDA(cudaMemcpyAsync(B.vx[0], B.vx[1], n * 4, cudaMemcpyDeviceToDevice, st));
    PIC_CUDA(cudaMemcpyAsync(B.vy[0], B.vy[1], n * 4, cudaMemcpyDeviceToDevice, st));
    PIC_CUDA(cudaMemcpyAsync(B.pid[0], B.pid[1], n * 4, cudaMemcpyDeviceToDevice, st));
    if (B.vz[0]) PIC_CUDA(cudaMemcpyAsync(B.vz[0], B.vz[1], n * 4, cudaMemcpyDeviceToDevice, st));
    return PIC_OK;
}

// import: arbitrary order, radix sort of the keys (pic_import.cu);
// otherwise the periodic counting sort
static pic_status sort_now(pic_handle *h, bool import = false)
{
    // a species whose import records already sit in the stage goes first
    // (import_sort consumes the flag, so it is read once up front)
    bool first[PIC_MAX_SPECIES] = {};
    for (int s = 0; s < h->cfg.nspecies; ++s) first[s] = h->sp[s].records_ready;
    for (int pass = 0; pass < 2; ++pass)
        for (int s = 0; s < h->cfg.nspecies; ++s) {
            if (!h->sp[s].cap || first[s] != (pass == 0)) continue;
            bool in0 = false;
            if (import && h->sp[s].presorted) {  // in buffer 1, sorted range by range
                h->sp[s].presorted = false;
                in0 = true;
                PIC_TRY(launch_sort(h, s, false, 1));  // one counting sort into buffer 0
            } else {
                PIC_TRY(import ? import_sort(h, s, &in0) : launch_sort(h, s));
            }
            if (!in0) PIC_TRY(copy_back(h, s));
            if (import) PIC_TRY(launch_recount(h, s));  // the DSMC species' kept counts
        }
    h->since_sort = 0;
    return PIC_OK;
}

pic_status deposit_now(pic_handle *h)
{
    PIC_CUDA(cudaMemsetAsync(h->rho_fix, 0, sizeof(unsigned long long) * (size_t)h->g.nx * h->g.ny,
                             h->stream));
    for (int s = 0; s < h->cfg.nspecies; ++s)
        if (h->sp[s].cap) PIC_TRY(launch_deposit(h, s));
    return PIC_OK;
}

// After particles change from the host: sort, deposit, solve.
pic_status refresh(pic_handle *h)
{
    update_mean(h);
    PIC_TRY(sort_now(h, true));
    PIC_TRY(deposit_now(h));
    PIC_TRY(record_poisson(h));
    PIC_CUDA(cudaStreamSynchronize(h->stream));
    h->fields_valid = true;
    return PIC_OK;
}

static void drop_graphs(pic_handle *h)
{
    if (h->g_period) cudaGraphExecDestroy(h->g_period);
    if (h->g_sortstep) cudaGraphExecDestroy(h->g_sortstep);
    if (h->g_one) cudaGraphExecDestroy(h->g_one);
    h->g_period = h->g_sortstep = h->g_one = nullptr;
    h->graphs_valid = false;
}

template <class F> static pic_status capture(pic_handle *h, cudaGraphExec_t *out, F &&body)
{
    cudaGraph_t graph = nullptr;
    PIC_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    pic_status s = body();
    cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
    if (s != PIC_OK) {
        if (graph) cudaGraphDestroy(graph);
        return s;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    return PIC_OK;
}

static pic_status build_graphs(pic_handle *h)
{
    if (h->graphs_valid) return PIC_OK;
    drop_graphs(h);
    const int S = h->cfg.sort_every;
    PIC_TRY(capture(h, &h->g_one, [&] { return record_step(h, 0); }));
    PIC_TRY(capture(h, &h->g_sortstep, [&] {
        PIC_TRY(record_sort_all(h));
        return record_step(h, 1);
    }));
    PIC_TRY(capture(h, &h->g_period, [&] {
        PIC_TRY(record_sort_all(h));
        PIC_TRY(record_step(h, 1));
        for (int k = 1; k < S; ++k) PIC_TRY(record_step(h, 0));
        return PIC_OK;
    }));
    h->graphs_valid = true;
    return PIC_OK;
}

static pic_status need(pic_handle *h)
{
    if (!h) {
        set_error("null handle");
        return PIC_ERR_INVALID_ARG;
    }
    PIC_CUDA(cudaSetDevice(h->device));
    return PIC_OK;
}

static pic_status need_species(pic_handle *h, int s)
{
    PIC_TRY(need(h));
    if (s < 0 || s >= h->cfg.nspecies || h->sp[s].cap == 0) {
        set_error("species index out of range or species without capacity");
        return PIC_ERR_INVALID_ARG;
    }
    return PIC_OK;
}

// Device address of a page-locked host array (allocated or registered with
// the CUDA runtime), or null for other memory.
template <class T> static T *mapped(T *p)
{
    if (!p) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? (T *)a.devicePointer : nullptr;
}

// Whether the stage holds `bytes` now or can grow to it and leave 1 GiB of
// device memory free (callers fall back to a leaner layout otherwise).  The
// environment variable PIC_STAGE_MAX_BYTES caps the layouts chosen this way
// for callers that keep a device-memory budget.
bool stage_fits(pic_handle *h, size_t bytes)
{
    if (const char *cap = getenv("PIC_STAGE_MAX_BYTES")) {
        char *end = nullptr;
        const unsigned long long v = strtoull(cap, &end, 10);
        if (end != cap && bytes > v) return false;
    }
    if (h->stage_bytes >= bytes) return true;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return free_b + h->stage_bytes >= bytes + (1ull << 30);
}

pic_status ensure_stage(pic_handle *h, size_t bytes)
{
    if (h->stage_bytes >= bytes) return PIC_OK;
    cudaFree(h->stage);
    h->stage = nullptr;
    h->stage_bytes = 0;
    PIC_CUDA(cudaMalloc(&h->stage, bytes));
    h->stage_bytes = bytes;
    return PIC_OK;
}

static pic_status set_count(pic_handle *h, int s, long long n)
{
    SpeciesBuf &B = h->sp[s];
    const long long old4 = (B.n + 3) & ~3ll;
    B.n = n;
    const long long n4 = (n + 3) & ~3ll;
    PIC_CUDA(cudaMemcpyAsync(&h->dev->n[s], &B.n, sizeof(long long), cudaMemcpyHostToDevice,
                             h->stream));
    // slots past n up to the next multiple of 4 must read as empty
    PIC_TRY(launch_fill_padding(h, s, n, std::max(old4, n4)));
    PIC_CUDA(cudaStreamSynchronize(h->stream));
    return PIC_OK;
}

// After a state file was loaded into buffer 0: counts, padding, counters,
// then sort, deposit and solve (the field is a function of the positions).
pic_status handle_reload(pic_handle *h, const long long *n, long long step,
                         unsigned long long mcc_pass, unsigned long long dsmc_pass)
{
    for (int s = 0; s < h->cfg.nspecies; ++s)
        if (h->sp[s].cap) PIC_TRY(set_count(h, s, n[s]));
    PIC_TRY(reset_device_state(h));
    PIC_CUDA(cudaMemcpy(&h->dev->step, &step, sizeof step, cudaMemcpyHostToDevice));
    PIC_CUDA(cudaMemcpy(&h->dev->mcc_pass, &mcc_pass, sizeof mcc_pass, cudaMemcpyHostToDevice));
    PIC_CUDA(cudaMemcpy(&h->dev->dsmc_pass, &dsmc_pass, sizeof dsmc_pass, cudaMemcpyHostToDevice));
    h->steps_host = step;
    return refresh(h);
}

pic_status lattice_dims_for(int nx, int ny, long long n, int *lx, int *ly)
{
    const long long nc = (long long)nx * ny;
    if (n % nc) {
        set_error("lattice load needs a whole number of particles per cell");
        return PIC_ERR_INVALID_ARG;
    }
    const long long ppc = n / nc;
    long long a = (long long)std::ceil(std::sqrt((double)ppc));
    while (ppc % a) ++a;  // smallest divisor >= sqrt(ppc): more sites along x
    *lx = (int)(nx * a);
    *ly = (int)(ny * (ppc / a));
    return PIC_OK;
}

pic_status lattice_dims(pic_handle *h, long long n, int *lx, int *ly)
{
    return lattice_dims_for(h->g.nx, h->g.ny, n, lx, ly);
}

// The handle's second stream and its events (export copies, import ranges),
// created on first use.
pic_status ensure_copy_stream(pic_handle *h)
{
    if (h->copy_stream) return PIC_OK;
    PIC_CUDA(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
    for (auto &e : h->field_ready) PIC_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    PIC_CUDA(cudaEventCreateWithFlags(&h->copies_done, cudaEventDisableTiming));
    return PIC_OK;
}

}  // namespace pic

using namespace pic;

extern "C" {

const char *pic_status_string(pic_status s)
{
    switch (s) {
    case PIC_OK: return "ok";
    case PIC_ERR_INVALID_ARG: return "invalid argument";
    case PIC_ERR_OOM: return "out of memory";
    case PIC_ERR_CUDA: return "CUDA error";
    case PIC_ERR_CUFFT: return "cuFFT error";
    case PIC_ERR_OVERFLOW: return "capacity overflow";
    case PIC_ERR_NAN: return "non-finite particle state";
    case PIC_ERR_TIMEOUT: return "device wait timed out";
    case PIC_ERR_STATE: return "invalid state for this call";
    case PIC_ERR_NO_DEVICE: return "no CUDA device";
    }
    return "unknown status";
}

const char *pic_last_error(void) { return g_last_error.c_str(); }
const char *pic_version(void) { return "1.0.0"; }

pic_status pic_config_default(pic_config *c)
{
    if (!c) return PIC_ERR_INVALID_ARG;
    memset(c, 0, sizeof *c);
    c->nx = c->ny = 128;
    c->Lx = c->Ly = 1.0;
    c->dt = 0.1;
    c->eps0 = 1.0;
    c->nspecies = 1;
    c->species[0].capacity = 0;
    c->species[0].q = -1.0;
    c->species[0].m = 1.0;
    c->species[0].q_int = -1;
    return PIC_OK;
}

pic_status pic_create(const pic_config *cfg, pic_handle **out)
{
    if (!cfg || !out) {
        set_error("pic_create: null argument");
        return PIC_ERR_INVALID_ARG;
    }
    *out = nullptr;
    pic_handle *h = new pic_handle();
    h->cfg = *cfg;
    if (!h->cfg.sort_every) h->cfg.sort_every = 20;
    h->hist_cap = h->cfg.history ? h->cfg.history : 4096;
    pic_status s = validate(&h->cfg, h);
    if (s == PIC_OK) s = setup_geometry(h);
    if (s != PIC_OK) {
        delete h;
        return s;
    }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0 || cfg->device < 0 || cfg->device >= ndev) {
        delete h;
        set_error("pic_create: no usable CUDA device");
        return PIC_ERR_NO_DEVICE;
    }
    h->device = cfg->device;
    auto fail = [&](pic_status st) {
        free_handle_buffers(h);
        delete h;
        return st;
    };
#define H_TRY(call)                                                                            \
    do {                                                                                       \
        pic_status s_ = (call);                                                                \
        if (s_ != PIC_OK) return fail(s_);                                                     \
    } while (0)
#define H_CUDA(call)                                                                           \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) return fail(cuda_fail(e_, #call));                              \
    } while (0)
#define H_CUFFT(call)                                                                          \
    do {                                                                                       \
        cufftResult r_ = (call);                                                               \
        if (r_ != CUFFT_SUCCESS) return fail(cufft_fail(r_, #call));                           \
    } while (0)
    H_CUDA(cudaSetDevice(h->device));
    H_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    const Geometry &g = h->g;
    const size_t ncell = (size_t)g.nx * g.ny, nk = (size_t)g.ny * g.nh;
    for (int sp = 0; sp < h->cfg.nspecies; ++sp) {
        SpeciesBuf &B = h->sp[sp];
        const pic_species_desc &D = h->cfg.species[sp];
        B.cap = (D.capacity + 3) & ~3ll;
        if (!B.cap) continue;
        const size_t n = (size_t)B.cap;
        for (int b = 0; b < 2; ++b) {
            H_TRY(dalloc(&B.cell[b], n));
            H_TRY(dalloc(&B.ox[b], n));
            H_TRY(dalloc(&B.oy[b], n));
            H_TRY(dalloc(&B.vx[b], n));
            H_TRY(dalloc(&B.vy[b], n));
            H_TRY(dalloc(&B.pid[b], n));
            if (D.flags & PIC_SPECIES_HAS_VZ) H_TRY(dalloc(&B.vz[b], n));
            H_CUDA(cudaMemsetAsync(B.cell[b], 0xFF, n * 4, h->stream));  // all slots empty
            H_CUDA(cudaMemsetAsync(B.ox[b], 0, n * 4, h->stream));
            H_CUDA(cudaMemsetAsync(B.oy[b], 0, n * 4, h->stream));
            H_CUDA(cudaMemsetAsync(B.vx[b], 0, n * 4, h->stream));
            H_CUDA(cudaMemsetAsync(B.vy[b], 0, n * 4, h->stream));
            H_CUDA(cudaMemsetAsync(B.pid[b], 0, n * 4, h->stream));
            if (B.vz[b]) H_CUDA(cudaMemsetAsync(B.vz[b], 0, n * 4, h->stream));
        }
        B.nchunks = (B.cap + g.chunk - 1) / g.chunk;
        H_TRY(dalloc(&B.anchor, (size_t)B.nchunks));
        H_CUDA(cudaMemsetAsync(B.anchor, 0xFF, (size_t)B.nchunks * 4, h->stream));
    }
    H_TRY(dalloc(&h->rho_fix, ncell));
    H_TRY(dalloc(&h->rho, ncell));
    H_TRY(dalloc(&h->rhohat, nk));
    H_TRY(dalloc(&h->ehat, 2 * nk));
    H_TRY(dalloc(&h->e, 2 * ncell));
    H_TRY(dalloc(&h->count, ncell + 1));
    H_TRY(dalloc(&h->offset, ncell + 2));
    H_TRY(dalloc(&h->cursor, ncell + 1));
    h->scan_blocks = (int)((ncell + 1 + 4095) / 4096);
    H_TRY(dalloc(&h->bsum, (size_t)std::max(h->scan_blocks, 1)));
    H_TRY(dalloc(&h->dev, 1));
    H_TRY(dalloc(&h->hist, 6 * (size_t)h->hist_cap));
    H_CUDA(cudaMemsetAsync(h->rho_fix, 0, ncell * 8, h->stream));
    H_CUDA(cudaMemsetAsync(h->rho, 0, ncell * 4, h->stream));
    H_CUDA(cudaMemsetAsync(h->e, 0, 2 * ncell * 4, h->stream));
    // cuFFT: rows are y (slow), x contiguous; the half spectrum is along x
    H_CUFFT(cufftPlan2d(&h->plan_r2c, g.ny, g.nx, CUFFT_R2C));
    int dims[2] = {g.ny, g.nx};
    H_CUFFT(cufftPlanMany(&h->plan_c2r2, 2, dims, nullptr, 1, (int)nk, nullptr, 1, (int)ncell,
                          CUFFT_C2R, 2));
    H_CUFFT(cufftPlan2d(&h->plan_c2r1, g.ny, g.nx, CUFFT_C2R));
    H_CUFFT(cufftSetStream(h->plan_r2c, h->stream));
    H_CUFFT(cufftSetStream(h->plan_c2r2, h->stream));
    H_CUFFT(cufftSetStream(h->plan_c2r1, h->stream));
    // the step's solve: the spectral kernels on power-of-two grids, unless
    // PIC_FIELD_SOLVER=cufft asks for the library transforms
    h->spectral = spectral_wanted(g.nx, g.ny);
    if (h->spectral) H_TRY(spectral_twiddles(g.nx, g.ny, &h->tw));
    H_TRY(reset_device_state(h));
#undef H_TRY
#undef H_CUDA
#undef H_CUFFT
    *out = h;
    return PIC_OK;
}

pic_status pic_destroy(pic_handle *h)
{
    if (!h) return PIC_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_handle_buffers(h);
    delete h;
    return PIC_OK;
}

pic_status pic_get_stream(pic_handle *h, void **stream)
{
    PIC_TRY(need(h));
    if (!stream) return PIC_ERR_INVALID_ARG;
    *stream = (void *)h->stream;
    return PIC_OK;
}

static pic_status check_flags(pic_handle *h)
{
    unsigned int err = 0;
    PIC_CUDA(cudaMemcpy(&err, &h->dev->err, sizeof err, cudaMemcpyDeviceToHost));
    if (err & PIC_DEVERR_CELL) {
        set_error("device: a particle cell index outside the grid was found");
        return PIC_ERR_STATE;
    }
    if (err & PIC_DEVERR_SORT) {
        set_error("device: a sort destination fell outside the species' slots");
        return PIC_ERR_STATE;
    }
    if (err & PIC_DEVERR_TIMEOUT) {
        set_error("device: a bounded wait gave up");
        return PIC_ERR_TIMEOUT;
    }
    if (err & PIC_DEVERR_CAPACITY) {
        set_error("device: species capacity exceeded");
        return PIC_ERR_OVERFLOW;
    }
    if (err & PIC_DEVERR_NAN) {
        set_error("device: non-finite particle velocity");
        return PIC_ERR_NAN;
    }
    return PIC_OK;
}

pic_status pic_synchronize(pic_handle *h)
{
    PIC_TRY(need(h));
    PIC_CUDA(cudaStreamSynchronize(h->stream));
    return check_flags(h);
}

pic_status pic_init_particles(pic_handle *h, int s, const pic_init_spec *spec)
{
    PIC_TRY(need_species(h, s));
    if (!spec || spec->n < 0 || spec->n > h->cfg.species[s].capacity) {
        set_error("pic_init_particles: count exceeds capacity");
        return PIC_ERR_INVALID_ARG;
    }
    int lx = 0, ly = 0;
    if (spec->layout == PIC_LOAD_LATTICE) PIC_TRY(lattice_dims(h, spec->n, &lx, &ly));
    PIC_TRY(set_count(h, s, spec->n));
    PIC_TRY(launch_init(h, s, spec, lx, ly));
    PIC_TRY(reset_device_state(h));
    return refresh(h);
}

pic_status pic_set_particles(pic_handle *h, int s, long long n, const double *x, const double *y,
                             const double *vx, const double *vy, const double *vz)
{
    PIC_TRY(need_species(h, s));
    if (n < 0 || n > h->cfg.species[s].capacity || (n && (!x || !y || !vx || !vy))) {
        set_error("pic_set_particles: bad count or null array");
        return PIC_ERR_INVALID_ARG;
    }
    const size_t nn = (size_t)n;
    PIC_TRY(set_count(h, s, n));
    const double *dx = mapped(x), *dy = mapped(y), *dvx = mapped(vx), *dvy = mapped(vy);
    const double *dvz = vz ? mapped(vz) : nullptr;
    if (n && dx && dy && dvx && dvy && (!vz || dvz)) {
        // page-locked host arrays: the conversion kernel reads them in place
        // over the CPU-GPU link (coalesced, in particle order), straight
        // into the import sort's keys and records when the stage holds them
        const size_t rec_bytes = (size_t)h->sp[s].cap * 48;
        if (stage_fits(h, rec_bytes)) {
            PIC_TRY(ensure_stage(h, rec_bytes));
            if (h->sp[s].cap >= IMPORT_SPLIT_MIN) {
                PIC_TRY(import_records_in_parts(h, s, n, dx, dy, dvx, dvy, dvz));
            } else {
                PIC_TRY(launch_from_global_records(h, s, n, dx, dy, dvx, dvy, dvz));
                h->sp[s].records_ready = true;
            }
        } else {
            PIC_TRY(launch_from_global(h, s, n, dx, dy, dvx, dvy, dvz));
        }
    } else {
        PIC_TRY(ensure_stage(h, std::max<size_t>(1, nn) * 5 * sizeof(double)));
        double *d = (double *)h->stage;
        if (n) {
            PIC_CUDA(cudaMemcpyAsync(d, x, nn * 8, cudaMemcpyHostToDevice, h->stream));
            PIC_CUDA(cudaMemcpyAsync(d + nn, y, nn * 8, cudaMemcpyHostToDevice, h->stream));
            PIC_CUDA(cudaMemcpyAsync(d + 2 * nn, vx, nn * 8, cudaMemcpyHostToDevice, h->stream));
            PIC_CUDA(cudaMemcpyAsync(d + 3 * nn, vy, nn * 8, cudaMemcpyHostToDevice, h->stream));
            if (vz) PIC_CUDA(cudaMemcpyAsync(d + 4 * nn, vz, nn * 8, cudaMemcpyHostToDevice, h->stream));
        }
        PIC_TRY(launch_from_global(h, s, n, d, d + nn, d + 2 * nn, d + 3 * nn,
                                   vz ? d + 4 * nn : nullptr));
    }
    pic_status rc = reset_device_state(h);
    if (rc == PIC_OK) rc = refresh(h);
    h->sp[s].records_ready = false;  // consumed by the import sort, or stale after an error
    h->sp[s].presorted = false;
    return rc;
}

pic_status pic_get_particles(pic_handle *h, int s, long long *n, double *x, double *y, double *vx,
                             double *vy, double *vz)
{
    PIC_TRY(need_species(h, s));
    PIC_CUDA(cudaStreamSynchronize(h->stream));
    long long cnt = 0;
    PIC_CUDA(cudaMemcpy(&cnt, &h->dev->n[s], sizeof cnt, cudaMemcpyDeviceToHost));
    h->sp[s].n = cnt;
    if (n) *n = cnt;
    const size_t nn = (size_t)cnt;
    if (!nn) return PIC_OK;
    // id order: the slots' fields scattered as one 32-byte record per id,
    // EXPORT_PARTS id ranges at a time for large counts (or, when the stage
    // cannot hold the records, through the inverse of the id permutation);
    // each field is converted with coalesced writes and copied to the host
    // on the copy stream while the next one is prepared
    double *host[5] = {x, y, vx, vy, vz};
    int nreq = 0;
    for (double *p : host) nreq += p != nullptr;
    const size_t cap = (size_t)h->sp[s].cap;
    const int parts = (long long)nn >= EXPORT_SPLIT_MIN ? EXPORT_PARTS : 1;
    const size_t part_max = (nn + parts - 1) / parts;
    const size_t packed_bytes = part_max * 32 + nn * nreq * sizeof(double);
    const bool packed = stage_fits(h, packed_bytes);
    PIC_TRY(ensure_stage(h, packed ? packed_bytes : nn * nreq * sizeof(double) + cap * sizeof(uint32_t)));
    // packed: records (16-byte aligned) then the doubles; else the doubles
    // then the inverse permutation
    uint4 *rec = (uint4 *)h->stage;
    double *d = packed ? (double *)(rec + 2 * part_max) : (double *)h->stage;
    uint32_t *inv = (uint32_t *)(d + nreq * nn);
    PIC_TRY(ensure_copy_stream(h));
    double *dev[5];
    for (int k = 0, j = 0; k < 5; ++k) dev[k] = host[k] ? d + (j++) * nn : nullptr;
    if (packed) {
        for (int r = 0; r < parts; ++r) {
            const long long lo = (long long)(nn * r / parts), hi = (long long)(nn * (r + 1) / parts);
            cudaEvent_t *ready = h->field_ready + 5 * r;
            PIC_TRY(launch_to_global_by_record(h, s, lo, hi, dev, rec, ready));
            for (int k = 0; k < 5; ++k) {
                if (!host[k] || hi <= lo) continue;
                PIC_CUDA(cudaStreamWaitEvent(h->copy_stream, ready[k], 0));
                PIC_CUDA(cudaMemcpyAsync(host[k] + lo, dev[k] + lo, (size_t)(hi - lo) * 8,
                                         cudaMemcpyDeviceToHost, h->copy_stream));
            }
        }
    } else {
        PIC_TRY(launch_to_global_by_id(h, s, dev, inv, h->field_ready));
        for (int k = 0; k < 5; ++k) {
            if (!host[k]) continue;
            PIC_CUDA(cudaStreamWaitEvent(h->copy_stream, h->field_ready[k], 0));
            PIC_CUDA(cudaMemcpyAsync(host[k], dev[k], nn * 8, cudaMemcpyDeviceToHost, h->copy_stream));
        }
    }
    PIC_CUDA(cudaEventRecord(h->copies_done, h->copy_stream));
    PIC_CUDA(cudaStreamWaitEvent(h->stream, h->copies_done, 0));
    PIC_CUDA(cudaStreamSynchronize(h->stream));
    return PIC_OK;
}

pic_status pic_get_particles_raw(pic_handle *h, int s, long long *n, int32_t *cell, float *ox,
                                 float *oy, float *vx, float *vy, uint32_t *pid)
{
    PIC_TRY(need_species(h, s));
    PIC_CUDA(cudaStreamSynchronize(h->stream));
    long long cnt = 0;
    PIC_CUDA(cudaMemcpy(&cnt, &h->dev->n[s], sizeof cnt, cudaMemcpyDeviceToHost));
    if (n) *n = cnt;
    const SpeciesBuf &B = h->sp[s];
    const size_t b = (size_t)cnt * 4;
    if (cell) PIC_CUDA(cudaMemcpy(cell, B.cell[0], b, cudaMemcpyDeviceToHost));
    if (ox) PIC_CUDA(cudaMemcpy(ox, B.ox[0], b, cudaMemcpyDeviceToHost));
    if (oy) PIC_CUDA(cudaMemcpy(oy, B.oy[0], b, cudaMemcpyDeviceToHost));
    if (vx) PIC_CUDA(cudaMemcpy(vx, B.vx[0], b, cudaMemcpyDeviceToHost));
    if (vy) PIC_CUDA(cudaMemcpy(vy, B.vy[0], b, cudaMemcpyDeviceToHost));
    if (pid) PIC_CUDA(cudaMemcpy(pid, B.pid[0], b, cudaMemcpyDeviceToHost));
    return PIC_OK;
}

pic_status pic_particles_device(pic_handle *h, int s, pic_particles_view *v)
{
    PIC_TRY(need_species(h, s));
    if (!v) return PIC_ERR_INVALID_ARG;
    const SpeciesBuf &B = h->sp[s];
    v->n = B.n;
    v->cell_dev = B.cell[0];
    v->ox_dev = B.ox[0];
    v->oy_dev = B.oy[0];
    v->vx_dev = B.vx[0];
    v->vy_dev = B.vy[0];
    v->vz_dev = B.vz[0];
    v->pid_dev = B.pid[0];
    return PIC_OK;
}

pic_status pic_prime_leapfrog(pic_handle *h)
{
    PIC_TRY(need(h));
    if (!h->fields_valid) {
        set_error("pic_prime_leapfrog: no field yet");
        return PIC_ERR_STATE;
    }
    for (int s = 0; s < h->cfg.nspecies; ++s)
        if (h->sp[s].cap && h->cfg.species[s].q != 0.0)
            PIC_TRY(launch_push(h, s, 0, false, -0.5f));
    return PIC_OK;
}

pic_status pic_sort(pic_handle *h)
{
    PIC_TRY(need(h));
    return sort_now(h);
}

pic_status pic_deposit(pic_handle *h)
{
    PIC_TRY(need(h));
    return deposit_now(h);
}

pic_status pic_poisson(pic_handle *h)
{
    PIC_TRY(need(h));
    PIC_TRY(record_poisson(h));
    h->fields_valid = true;
    return PIC_OK;
}

pic_status pic_gather_push(pic_handle *h, int deposit)
{
    PIC_TRY(need(h));
    if (!h->fields_valid) {
        set_error("pic_gather_push: no field yet");
        return PIC_ERR_STATE;
    }
    if (deposit)
        PIC_CUDA(cudaMemsetAsync(h->rho_fix, 0,
                                 sizeof(unsigned long long) * (size_t)h->g.nx * h->g.ny, h->stream));
    PIC_TRY(record_push_all(h, 0, deposit != 0));
    h->since_sort++;
    h->steps_host++;
    return PIC_OK;
}

pic_status pic_step(pic_handle *h, long long nsteps)
{
    PIC_TRY(need(h));
    if (nsteps < 0) return PIC_ERR_INVALID_ARG;
    if (!h->fields_valid) {
        set_error("pic_step: initialise particles first");
        return PIC_ERR_STATE;
    }
    PIC_TRY(build_graphs(h));
    const int S = h->cfg.sort_every;
    long long n = nsteps;
    while (n > 0) {
        if (h->since_sort >= S) {
            if (n >= S) {
                PIC_CUDA(cudaGraphLaunch(h->g_period, h->stream));
                n -= S;
                h->since_sort = S;
            } else {
                PIC_CUDA(cudaGraphLaunch(h->g_sortstep, h->stream));
                n -= 1;
                h->since_sort = 1;
            }
        } else {
            PIC_CUDA(cudaGraphLaunch(h->g_one, h->stream));
            n -= 1;
            h->since_sort += 1;
        }
    }
    h->steps_host += nsteps;
    return PIC_OK;
}

pic_status pic_run_host(pic_handle *h, long long n, const double *x, const double *y,
                        const double *vx, const double *vy, long long nsteps, int prime,
                        double *x_out, double *y_out, double *vx_out, double *vy_out)
{
    PIC_TRY(pic_set_particles(h, 0, n, x, y, vx, vy, nullptr));
    if (prime) PIC_TRY(pic_prime_leapfrog(h));
    PIC_TRY(pic_step(h, nsteps));
    PIC_TRY(check_flags(h));
    return pic_get_particles(h, 0, nullptr, x_out, y_out, vx_out, vy_out, nullptr);
}

pic_status pic_diagnostics(pic_handle *h, pic_diag *d)
{
    PIC_TRY(need(h));
    if (!d) return PIC_ERR_INVALID_ARG;
    PIC_CUDA(cudaStreamSynchronize(h->stream));
    DevState st;
    PIC_CUDA(cudaMemcpy(&st, h->dev, sizeof st, cudaMemcpyDeviceToHost));
    memset(d, 0, sizeof *d);
    d->step = st.step;
    const int cap = h->hist_cap;
    double v = 0.0;
    PIC_CUDA(cudaMemcpy(&v, h->hist + 0 * (size_t)cap + st.step % cap, 8, cudaMemcpyDeviceToHost));
    d->field_energy = v;
    double c = 0.0;
    PIC_CUDA(cudaMemcpy(&c, h->hist + 4 * (size_t)cap + st.step % cap, 8, cudaMemcpyDeviceToHost));
    if (st.step > 0) {
        const long long k = (st.step - 1) % cap;
        PIC_CUDA(cudaMemcpy(&d->kinetic_energy, h->hist + 1 * (size_t)cap + k, 8, cudaMemcpyDeviceToHost));
        PIC_CUDA(cudaMemcpy(&d->momentum[0], h->hist + 2 * (size_t)cap + k, 8, cudaMemcpyDeviceToHost));
        PIC_CUDA(cudaMemcpy(&d->momentum[1], h->hist + 3 * (size_t)cap + k, 8, cudaMemcpyDeviceToHost));
    }
    d->total_charge_fixed = (long long)c;
    unsigned long long expect = 0;
    for (int s = 0; s < PIC_MAX_SPECIES; ++s) {
        d->n[s] = st.n[s];
        if (s < h->cfg.nspecies)
            expect += (unsigned long long)(long long)h->cfg.species[s].q_int *
                      ((unsigned long long)st.n[s] << 32);
    }
    d->expected_charge_fixed = (long long)expect;
    d->error_flags = st.err;
    return PIC_OK;
}

pic_status pic_get_history(pic_handle *h, int which, long long first, long long count, double *out)
{
    PIC_TRY(need(h));
    if (which < 0 || which > 5 || first < 0 || count < 0 || (count && !out)) return PIC_ERR_INVALID_ARG;
    PIC_CUDA(cudaStreamSynchronize(h->stream));
    long long step = 0;
    PIC_CUDA(cudaMemcpy(&step, &h->dev->step, sizeof step, cudaMemcpyDeviceToHost));
    const bool per_push = (which >= 1 && which <= 3);
    const long long last = per_push ? step - 1 : step;  // newest valid index
    const int cap = h->hist_cap;
    if (count && (first + count - 1 > last || first < last - cap + 1)) {
        set_error("pic_get_history: range outside the kept history");
        return PIC_ERR_INVALID_ARG;
    }
    std::vector<double> ring((size_t)cap);
    PIC_CUDA(cudaMemcpy(ring.data(), h->hist + (size_t)which * cap, sizeof(double) * cap,
                        cudaMemcpyDeviceToHost));
    for (long long i = 0; i < count; ++i) out[i] = ring[(size_t)((first + i) % cap)];
    return PIC_OK;
}

pic_status pic_track_mode(pic_handle *h, int mx, int my)
{
    PIC_TRY(need(h));
    if (mx < 0 || mx >= h->g.nh || my < 0 || my >= h->g.ny) return PIC_ERR_INVALID_ARG;
    h->track_mx = mx;
    h->track_my = my;
    drop_graphs(h);  // the kernel arguments are baked into the graphs
    return PIC_OK;
}

pic_status pic_get_grid(pic_handle *h, int which, double *out)
{
    PIC_TRY(need(h));
    if (!out || which < 0 || which > 3) return PIC_ERR_INVALID_ARG;
    if (!h->fields_valid) {
        set_error("pic_get_grid: no field yet");
        return PIC_ERR_STATE;
    }
    const size_t ncell = (size_t)h->g.nx * h->g.ny;
    std::vector<float> tmp(ncell);
    const float *src = nullptr;
    if (which == PIC_GRID_RHO) {
        src = h->rho;
    } else if (which == PIC_GRID_EX) {
        src = h->e;
    } else if (which == PIC_GRID_EY) {
        src = h->e + ncell;
    } else {
        // phi^ into the first half of ehat, C2R into the second half (the
        // spectral solve leaves no full spectrum: transform rho first)
        const size_t nk = (size_t)h->g.ny * h->g.nh;
        if (h->spectral)
            PIC_CUFFT(cufftExecR2C(h->plan_r2c, h->rho, (cufftComplex *)h->rhohat));
        PIC_TRY(launch_kspace(h, true, h->ehat));
        PIC_CUFFT(cufftExecC2R(h->plan_c2r1, (cufftComplex *)h->ehat, (cufftReal *)(h->ehat + nk)));
        src = (const float *)(h->ehat + nk);
    }
    PIC_CUDA(cudaMemcpyAsync(tmp.data(), src, ncell * 4, cudaMemcpyDeviceToHost, h->stream));
    PIC_CUDA(cudaStreamSynchronize(h->stream));
    for (size_t i = 0; i < ncell; ++i) out[i] = tmp[i];
    return PIC_OK;
}

pic_status pic_get_rho_fixed(pic_handle *h, int64_t *out)
{
    PIC_TRY(need(h));
    if (!out) return PIC_ERR_INVALID_ARG;
    const size_t ncell = (size_t)h->g.nx * h->g.ny;
    PIC_TRY(deposit_now(h));
    PIC_CUDA(cudaMemcpyAsync(out, h->rho_fix, ncell * 8, cudaMemcpyDeviceToHost, h->stream));
    PIC_CUDA(cudaMemsetAsync(h->rho_fix, 0, ncell * 8, h->stream));
    PIC_CUDA(cudaStreamSynchronize(h->stream));
    return PIC_OK;
}

}  // extern "C"

extern "C" pic_status pic_set_mcc(pic_handle *h, const pic_mcc_params *p)
{
    PIC_TRY(need(h));
    const pic_config &c = h->cfg;
    auto bad = [](const char *m) {
        set_error(std::string("pic_set_mcc: ") + m);
        return PIC_ERR_INVALID_ARG;
    };
    if (!p) return bad("null parameters");
    if (p->electron_species < 0 || p->electron_species >= c.nspecies ||
        !h->sp[p->electron_species].vz[0])
        return bad("electron species must exist and carry vz");
    if (p->ion_species >= c.nspecies ||
        (p->ion_species >= 0 && (!h->sp[p->ion_species].vz[0] || p->ion_species == p->electron_species)))
        return bad("ion species must carry vz and differ from the electrons");
    if (p->ntab < 2 || p->ntab > 4096 || !(p->e_min_eV > 0) || !(p->e_max_eV > p->e_min_eV) ||
        !p->sigma_elastic || !p->sigma_excitation || !p->sigma_ionization)
        return bad("cross-section table");
    if (!(p->neutral_density > 0) || !(p->electron_mass > 0) || !(p->ion_mass > 0) ||
        !(p->unit_charge > 0) || p->neutral_temp_eV < 0 || p->e_exc_eV < 0 || p->e_ion_eV < 0)
        return bad("physical constants");
    const int nt = p->ntab;
    std::vector<float> tab(4 * (size_t)nt);
    const double lr = std::log(p->e_max_eV / p->e_min_eV) / (nt - 1);
    double nu_max = 0.0;
    auto vel = [&](double e) { return std::sqrt(2.0 * e * p->unit_charge / p->electron_mass); };
    for (int k = 0; k < nt; ++k) {
        const double e = p->e_min_eV * std::exp(lr * k);
        tab[k] = (float)e;
        tab[nt + k] = (float)p->sigma_elastic[k];
        tab[2 * nt + k] = (float)p->sigma_excitation[k];
        tab[3 * nt + k] = (float)p->sigma_ionization[k];
        if (p->sigma_elastic[k] < 0 || p->sigma_excitation[k] < 0 || p->sigma_ionization[k] < 0)
            return bad("negative cross section");
    }
    // upper bound of n_g sigma_T(E) v(E) with sigma linear between table
    // points: the larger endpoint cross section at the segment's top speed
    for (int k = 0; k + 1 < nt; ++k) {
        const double s0 = p->sigma_elastic[k] + p->sigma_excitation[k] + p->sigma_ionization[k];
        const double s1 = p->sigma_elastic[k + 1] + p->sigma_excitation[k + 1] + p->sigma_ionization[k + 1];
        nu_max = std::max(nu_max, std::max(s0, s1) * vel(p->e_min_eV * std::exp(lr * (k + 1))));
    }
    nu_max *= p->neutral_density * 1.0001;
    MccState &M = h->mcc;
    if (!M.tab || M.ntab != nt) {
        cudaFree(M.tab);
        M.tab = nullptr;
        PIC_CUDA(cudaMalloc(&M.tab, tab.size() * sizeof(float)));
    }
    PIC_CUDA(cudaMemcpy(M.tab, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice));
    M.ntab = nt;
    M.e = p->electron_species;
    M.i = p->ion_species;
    M.ln_emin = (float)std::log(p->e_min_eV);
    M.inv_dln = (float)(1.0 / lr);
    M.half_me_over_e = (float)(0.5 * p->electron_mass / p->unit_charge);
    M.ng = (float)p->neutral_density;
    M.nu_max = (float)nu_max;
    M.p_null = (float)(1.0 - std::exp(-nu_max * c.dt));
    M.two_m_over_M = (float)(2.0 * p->electron_mass / p->ion_mass);
    M.e_exc = (float)p->e_exc_eV;
    M.e_ion = (float)p->e_ion_eV;
    M.vth_ion = (float)std::sqrt(p->neutral_temp_eV * p->unit_charge / p->ion_mass);
    M.seed = p->seed;
    M.on = true;
    drop_graphs(h);
    return PIC_OK;
}

extern "C" pic_status pic_set_dsmc(pic_handle *h, const pic_dsmc_params *p)
{
    PIC_TRY(need(h));
    if (!p || p->species < 0 || p->species >= h->cfg.nspecies || !h->sp[p->species].vz[0] ||
        h->cfg.species[p->species].q != 0.0 || !(p->diameter > 0) || !(p->weight > 0) ||
        !(p->depth > 0) || !(p->sigma_g_max0 > 0)) {
        set_error("pic_set_dsmc: the species must be neutral and carry vz; diameter, weight, "
                  "depth and sigma_g_max0 must be positive");
        return PIC_ERR_INVALID_ARG;
    }
    DsmcState &D = h->dsmc;
    const size_t ncell = (size_t)h->g.nx * h->g.ny;
    if (!D.sgmax) PIC_CUDA(cudaMalloc(&D.sgmax, ncell * sizeof(float)));
    std::vector<float> init(ncell, (float)p->sigma_g_max0);
    PIC_CUDA(cudaMemcpy(D.sgmax, init.data(), ncell * sizeof(float), cudaMemcpyHostToDevice));
    D.s = p->species;
    D.sigma = (float)(3.14159265358979323846 * p->diameter * p->diameter);
    D.coef = (float)(p->weight * h->cfg.dt / (2.0 * h->g.dx * h->g.dy * p->depth));
    D.seed = p->seed;
    if (!D.count) PIC_CUDA(cudaMalloc(&D.count, (ncell + 1) * sizeof(uint32_t)));
    D.on = true;
    drop_graphs(h);
    // a full sort counts the species into D.count, which its pushes then keep
    PIC_TRY(launch_sort(h, D.s));
    return copy_back(h, D.s);
}

extern "C" pic_status pic_collide(pic_handle *h, int kind)
{
    PIC_TRY(need(h));
    if (kind == PIC_COLLIDE_MCC) {
        if (!h->mcc.on) {
            set_error("pic_collide: MCC not configured (pic_set_mcc)");
            return PIC_ERR_STATE;
        }
        return launch_mcc(h);
    }
    if (kind == PIC_COLLIDE_DSMC) {
        if (!h->dsmc.on) {
            set_error("pic_collide: DSMC not configured (pic_set_dsmc)");
            return PIC_ERR_STATE;
        }
        PIC_TRY(launch_sort(h, h->dsmc.s, true));
        PIC_TRY(launch_ntc(h));
        return copy_back(h, h->dsmc.s);
    }
    set_error("pic_collide: unknown collision kind");
    return PIC_ERR_INVALID_ARG;
}

extern "C" pic_status pic_collision_counts(pic_handle *h, long long counts[6])
{
    PIC_TRY(need(h));
    if (!counts) return PIC_ERR_INVALID_ARG;
    PIC_CUDA(cudaStreamSynchronize(h->stream));
    unsigned long long c[6][ACC_SLOTS];
    PIC_CUDA(cudaMemcpy(c, h->dev->coll, sizeof c, cudaMemcpyDeviceToHost));
    for (int k = 0; k < 6; ++k) {
        unsigned long long t = 0;
        for (int l = 0; l < ACC_SLOTS; ++l) t += c[k][l];
        counts[k] = (long long)t;
    }
    return PIC_OK;
}
