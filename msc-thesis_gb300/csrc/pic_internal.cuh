// pic_internal.cuh -- shared declarations of libpic's translation units.
//
// Device data layout (physics mode), per species, structure of arrays:
//   cell  int32  cx | (cy << 16); -1 marks an empty (padding) slot
//   ox,oy float  in-cell offsets in [0,1), in cell units
//   vx,vy float  velocity (vz when PIC_SPECIES_HAS_VZ)
//   pid   uint32 particle id (moved only by the sort)
// Two copies (buffer 0 = live, buffer 1 = sort target).  Grids are row-major
// [iy][ix]: the fixed-point density rho_fix (uint64, two's complement,
// 2^-32 charge units), the float density rho (background removed), and the
// field planes e[0] = Ex, e[1] = Ey.
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>

#include <string>

#include "pic.h"

namespace pic {

// ------------------------------------------------------------------ errors
void set_error(const std::string &msg);
pic_status cuda_fail(cudaError_t e, const char *what);
pic_status cufft_fail(cufftResult r, const char *what);

#define PIC_CUDA(call)                                                                         \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) return ::pic::cuda_fail(e_, #call);                             \
    } while (0)
#define PIC_CUFFT(call)                                                                        \
    do {                                                                                       \
        cufftResult r_ = (call);                                                               \
        if (r_ != CUFFT_SUCCESS) return ::pic::cufft_fail(r_, #call);                          \
    } while (0)
#define PIC_TRY(call)                                                                          \
    do {                                                                                       \
        pic_status s_ = (call);                                                                \
        if (s_ != PIC_OK) return s_;                                                           \
    } while (0)

// ------------------------------------------------------------------ Philox
// Philox4x32-10 (Salmon et al., SC'11): published multipliers and Weyl
// key increments; 10 rounds.
struct U4 {
    uint32_t x, y, z, w;
};
__host__ __device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c.x;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c.z;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    }
    return c;
}
// (0,1) open interval from 32 random bits
__host__ __device__ __forceinline__ float u01f(uint32_t r)
{
    return ((float)(r >> 8) + 0.5f) * (1.0f / 16777216.0f);
}
__host__ __device__ __forceinline__ double u01d(uint32_t r)
{
    return ((double)r + 0.5) * (1.0 / 4294967296.0);
}

// Shared-memory window of a push block covering wcx x wcy cells: E (float2)
// at its (wcx + 1)(wcy + 1) nodes, then the deposit area: five 32-bit
// moment planes of its cells (count, sum fx, sum fy, and the low 16 and the
// high bits of sum fx*fy), with room also for two float planes of its nodes
// (the ensemble adjoint kick's scatter sums); a multiple of 16 bytes.
__host__ __device__ __forceinline__ size_t window_dep_words(int wcx, int wcy)
{
    const size_t nw = (size_t)(wcx + 1) * (wcy + 1), nc = (size_t)wcx * wcy;
    return 5 * nc > 2 * nw ? 5 * nc : 2 * nw;
}

__host__ __device__ __forceinline__ size_t window_bytes(int wcx, int wcy)
{
    return ((size_t)(wcx + 1) * (wcy + 1) * 8 + window_dep_words(wcx, wcy) * 4 + 15) & ~(size_t)15;
}

// Largest push chunk: every per-cell moment sum of a block stays at most 2^31,
// inside its unsigned 32-bit word.
constexpr int MAX_CHUNK = 32768;
// Push windows: halos shrink until a block's shared memory fits four blocks
// per SM (WINDOW_SMEM_TARGET); a window above WINDOW_SMEM_MAX even with
// 1-cell halos is refused (smaller tiles).
constexpr size_t WINDOW_SMEM_TARGET = 56 * 1024;
constexpr size_t WINDOW_SMEM_MAX = 112 * 1024;

// Philox stream identifiers (counter word 3)
enum : uint32_t {
    STREAM_INIT = 0x696e6974u,   // "init"
    STREAM_MCC = 0x6d636321u,    // "mcc!"
    STREAM_DSMC = 0x64736d63u    // "dsmc"
};

// ------------------------------------------------------------------ handle
struct SpeciesBuf {
    int32_t *cell[2] = {nullptr, nullptr};
    float *ox[2] = {nullptr, nullptr}, *oy[2] = {nullptr, nullptr};
    float *vx[2] = {nullptr, nullptr}, *vy[2] = {nullptr, nullptr};
    float *vz[2] = {nullptr, nullptr};
    uint32_t *pid[2] = {nullptr, nullptr};
    int32_t *anchor = nullptr;  // per push chunk: tile (tx | ty << 16) or -1
    long long cap = 0;          // allocated slots (multiple of 4)
    long long n = 0;            // host mirror of the count
    long long nchunks = 0;      // push grid size for this species
    bool records_ready = false; // import keys and records already in the stage
    bool presorted = false;     // imported already sorted, range by range
};

// An import from page-locked host arrays of at least IMPORT_SPLIT_MIN slots
// is converted and radix-sorted in IMPORT_PARTS slot ranges, each range
// sorted on the copy stream while the next one crosses the link.
constexpr int IMPORT_PARTS = 8;
constexpr long long IMPORT_SPLIT_MIN = 1ll << 22;

// An export of at least EXPORT_SPLIT_MIN particles is done in EXPORT_PARTS
// id ranges, each copied to the host while the next one is prepared.
constexpr int EXPORT_PARTS = 8;
constexpr long long EXPORT_SPLIT_MIN = 1ll << 22;

// Device-side accumulators and counters (one struct in device memory).
// Block-level partial sums go to one of ACC_SLOTS copies (block index mod
// ACC_SLOTS) so that the blocks of a kernel, which finish together, do not
// serialise on one address; the advance kernel folds the slots.
constexpr int ACC_SLOTS = 32;
struct DevState {
    double ke[ACC_SLOTS], px[ACC_SLOTS], py[ACC_SLOTS];  // push of the current step
    double fe[ACC_SLOTS];                               // k-space kernel
    unsigned long long q[ACC_SLOTS];                    // convert kernel (fixed-point charge)
    unsigned long long coll[6][ACC_SLOTS];  // elastic, excitation, ionisation, null, DSMC collisions, pairs
    double mode_amp;          // |rho^| of the tracked mode
    long long step;           // completed steps
    long long n[PIC_MAX_SPECIES];
    unsigned int err;         // PIC_DEVERR_* bits
    unsigned int pad;
    unsigned long long mcc_pass, dsmc_pass;  // collision pass counters (Philox counters)
    long long mcc_n0;         // electron count at the start of the current MCC pass
};
__device__ __forceinline__ int acc_slot() { return (int)(blockIdx.x & (ACC_SLOTS - 1)); }

// MCC configuration resolved for the device
struct MccState {
    bool on = false;
    int e = 0, i = -1;        // electron / ion species
    float *tab = nullptr;     // device [energy | elastic | excitation | ionisation] x ntab
    int ntab = 0;
    float ln_emin = 0, inv_dln = 0, half_me_over_e = 0, ng = 0, nu_max = 0, p_null = 0;
    float two_m_over_M = 0, e_exc = 0, e_ion = 0, vth_ion = 0;
    unsigned long long seed = 0;
};

struct DsmcState {
    bool on = false;
    int s = 0;
    float *sgmax = nullptr;   // per cell key
    uint32_t *count = nullptr;  // the species' particles per cell key (and the empty bin),
                                // recounted by every full sort, kept by its push
    float sigma = 0, coef = 0;
    unsigned long long seed = 0;
};

struct Geometry {
    int nx, ny, nh;           // nh = nx/2 + 1 (half spectrum along x)
    double Lx, Ly, dx, dy;
    int tw, th, ntx, nty;     // sort tiles
    int halo, chunk;
    int wcx, wcy;             // cell window of a push block: (2 tw + 2 halo) x (th + 2 halo)
};

}  // namespace pic

struct pic_handle {
    pic_config cfg;
    pic::Geometry g;
    int device = 0;
    cudaStream_t stream = nullptr;
    pic::SpeciesBuf sp[PIC_MAX_SPECIES];
    double q_unit = 0.0;       // charge of one deposit unit (q = q_int * q_unit)
    long long mean_fix = 0;    // background: mean fixed-point density per node
    // grids
    unsigned long long *rho_fix = nullptr;  // nx*ny
    float *rho = nullptr;                    // nx*ny
    float2 *rhohat = nullptr;                // ny*nh
    float2 *ehat = nullptr;                  // 2*ny*nh
    float *e = nullptr;                      // 2*nx*ny: Ex plane then Ey plane
    cufftHandle plan_r2c = 0, plan_c2r2 = 0, plan_c2r1 = 0;
    // power-of-two grids: the step's solve runs in pic_spectral.cu's kernels
    // (rhohat and ehat then hold their column-major intermediates)
    bool spectral = false;
    float2 *tw = nullptr;  // twiddles: nx entries, then ny
    // sort
    uint32_t *count = nullptr, *offset = nullptr, *cursor = nullptr, *bsum = nullptr;
    int scan_blocks = 0;
    // diagnostics
    pic::DevState *dev = nullptr;
    double *hist = nullptr;  // 6 * hist_cap doubles, see pic_history
    int hist_cap = 0;
    int track_mx = -1, track_my = -1;
    // graphs
    cudaGraphExec_t g_period = nullptr, g_sortstep = nullptr, g_one = nullptr;
    int since_sort = 0;
    bool graphs_valid = false;
    bool fields_valid = false;
    long long steps_host = 0;
    // host<->device staging for imports and exports (grown on demand)
    void *stage = nullptr;
    size_t stage_bytes = 0;
    // collision operators
    pic::MccState mcc;
    pic::DsmcState dsmc;
    // radix sort temporary storage of the import sort
    void *cub_temp = nullptr;
    size_t cub_temp_bytes = 0;
    // export: copies to the host on their own stream, field by field
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t field_ready[5 * pic::EXPORT_PARTS] = {};
    cudaEvent_t copies_done = nullptr;
};

namespace pic {

// ------------------------------------------------------------------ launchers
// pic_push.cu
pic_status launch_push(pic_handle *h, int s, int src, bool deposit, float dt_scale);
// lets `kernel` take `bytes` of dynamic shared memory (above the default 48 KB)
pic_status allow_dynamic_smem(const void *kernel, size_t bytes);
pic_status launch_deposit(pic_handle *h, int s);
// pic_field.cu
pic_status launch_convert(pic_handle *h);
pic_status launch_kspace(pic_handle *h, bool phi_only, float2 *phihat);
enum AdvanceKind { ADV_PUSH = 1, ADV_FIELD = 2 };
pic_status launch_advance(pic_handle *h, int kind);
// pic_spectral.cu
bool spectral_size_ok(int nx, int ny);
// spectral_size_ok, unless the environment variable PIC_FIELD_SOLVER=cufft
bool spectral_wanted(int nx, int ny);
pic_status spectral_twiddles(int nx, int ny, float2 **tw);  // cudaMalloc'd tables
pic_status launch_spectral(pic_handle *h);  // convert + solve, rho_fix cleared
// the adjoint solve psi = S^T g (gx, gy -> psi) on a handle with h->spectral;
// gh (2 ny nh) and ph (ny nh) are scratch
pic_status launch_spectral_adjoint(pic_handle *h, const float *gx, const float *gy, float2 *gh,
                                   float2 *ph, float *psi);
struct EnsRun;
// convert + solve of runs [first, first + count) of an ensemble's run table
// (one grid size; grids at each run's offsets); rho_fix is not cleared
pic_status launch_spectral_runs(const EnsRun *runs, int first, int count, int nx, int ny,
                                const unsigned long long *rho_fix, float *rho, float2 *rhohat,
                                float2 *ehat, float *e, const float2 *tw, DevState *devs,
                                cudaStream_t st);
// pic_sort.cu
pic_status launch_sort(pic_handle *h, int s, bool counts_kept = false, int from = 0);
pic_status launch_recount(pic_handle *h, int s);
void sort_sizes_for(double density, int *wk, int *hb);
pic_status scatter_smem_attr(const void *kernel);
pic_status launch_anchors(pic_handle *h, int s, int buf = 1);
// pic_import.cu: arbitrary order in buffer 0 -> key order in buffer 0 (records)
// or buffer 1 (per-field gather), with the anchors
pic_status import_sort(pic_handle *h, int s, bool *in_buffer0);
pic_status import_records_in_parts(pic_handle *h, int s, long long n, const double *x_dev,
                                   const double *y_dev, const double *vx_dev,
                                   const double *vy_dev, const double *vz_dev);
pic_status ensure_copy_stream(pic_handle *h);
// exclusive scan of count[0, nkeys) into offset and cursor, offset[nkeys] =
// *d_total; bsum, bsum_s: ceil(nkeys / 4096) entries, bsum2: ceil(that / 4096)
pic_status launch_key_scan(const uint32_t *count, uint32_t *offset, uint32_t *cursor,
                           long long nkeys, uint32_t *bsum, uint32_t *bsum_s, uint32_t *bsum2,
                           const long long *d_total, cudaStream_t st);
// pic_collide.cu
pic_status launch_mcc(pic_handle *h);
pic_status launch_ntc(pic_handle *h);
// pic_init.cu
pic_status launch_init(pic_handle *h, int s, const pic_init_spec *spec, int lat_nx, int lat_ny);
pic_status launch_from_global(pic_handle *h, int s, long long n, const double *x_dev,
                              const double *y_dev, const double *vx_dev, const double *vy_dev,
                              const double *vz_dev);
// the same conversion straight into the import sort's stage layout (keys,
// slots and packed records of all cap slots; see import_sort)
// (at most max_blocks blocks of 256 threads when max_blocks > 0, leaving the
// rest of the GPU to kernels on other streams)
pic_status launch_from_global_records_range(pic_handle *h, int s, long long n, long long lo,
                                            long long hi, const double *x_dev, const double *y_dev,
                                            const double *vx_dev, const double *vy_dev,
                                            const double *vz_dev, int max_blocks);
pic_status launch_from_global_records(pic_handle *h, int s, long long n, const double *x_dev,
                                      const double *y_dev, const double *vx_dev,
                                      const double *vy_dev, const double *vz_dev);
pic_status launch_to_global_by_id(pic_handle *h, int s, double *const *out, uint32_t *inv,
                                  cudaEvent_t *ready);
// ids [lo, hi) of an export through packed records (rec holds hi - lo)
pic_status launch_to_global_by_record(pic_handle *h, int s, long long lo, long long hi,
                                      double *const *out, uint4 *rec, cudaEvent_t *ready);
pic_status launch_fill_padding(pic_handle *h, int s, long long from, long long to);
pic_status launch_init_dA(pic_handle *h, const pic_init_spec *spec, int lat_nx, int lat_ny,
                          double *dxdA, double *dydA);
// particle arrays (buffer 0) and grid of one run, for callers without a handle
struct InitTarget {
    int32_t *cell;
    float *ox, *oy, *vx, *vy, *vz;
    uint32_t *pid;
    int nx, ny;
    double Lx, Ly;
};
InitTarget target_of(pic_handle *h, int s);
pic_status launch_init_target(const InitTarget &T, const pic_init_spec *spec, int lat_nx,
                              int lat_ny, cudaStream_t st);
pic_status launch_init_dA_target(const InitTarget &T, const pic_init_spec *spec, int lat_nx,
                                 int lat_ny, double *dxdA, double *dydA, cudaStream_t st);
pic_status launch_to_global_target(const InitTarget &T, const long long *d_n, long long cap,
                                   double *x_dev, double *y_dev, double *vx_dev, double *vy_dev,
                                   cudaStream_t st);

// grid-stride launch size for `n` items on the current device
int grid_for(long long n, int block);
int device_sms();  // multiprocessors of the current device (cached; 152 if unknown)
unsigned sort_grid(long long chunks, int per_sm);  // sort blocks: at most the resident ones

// pic_handle.cu stages used by other host files
pic_status record_poisson(pic_handle *h, int adv = ADV_FIELD);
pic_status record_push_all(pic_handle *h, int src, bool deposit, bool fold = true);
pic_status deposit_now(pic_handle *h);
pic_status refresh(pic_handle *h);
pic_status ensure_stage(pic_handle *h, size_t bytes);
bool stage_fits(pic_handle *h, size_t bytes);
pic_status lattice_dims(pic_handle *h, long long n, int *lx, int *ly);
pic_status lattice_dims_for(int nx, int ny, long long n, int *lx, int *ly);
int pick_divisor(int n, int target);
int pick_tile_h(int ny, int tcells, int tw);

}  // namespace pic
