// pic_ensemble.cuh -- the ensemble's run table, work tables and state,
// shared by pic_ensemble.cu (stepping) and pic_ensemble_adjoint.cu.
#pragma once
#include <cuda_runtime.h>
#include <cufft.h>

#include <string>
#include <vector>

#include "pic_internal.cuh"
#include "pic_sort_dev.cuh"

namespace pic {

// One run of an ensemble: its grid, sort tiles and push window, its offsets
// in the pools (particle slots, grid nodes, spectrum, sort keys) and its
// step coefficients.
struct EnsRun {
    int nx, ny, nh, tw, th, ntx, nty, wcx, wcy, hx, hy;
    int key_off;
    long long n, cap4, poff, goff, ncp, khoff, nk;
    float qm_dt, dtdx, dtdy, rho_scale;
    float kx1, ky1, inv_eps0_n;
    float dt, inv_dx, inv_dy, q_dA, eps0_dA;  // adjoint: dt, 1/dx, 1/dy, q/(dx dy), eps0 dx dy
    unsigned long long qmul;
    double ke_scale, p_scale, fe_scale;
    long long mean_fix;
    double dx, dy;
};

struct SegBlock {
    long long base;
    int count;
    int run;
};

constexpr int ENS_NODES_PER_BLOCK = 2048;

}  // namespace pic

struct pic_ensemble {
    int device = 0;
    cudaStream_t stream = nullptr;
    int nruns = 0;
    std::vector<pic_config> cfg;     // caller order
    std::vector<int> slot_of, run_of;
    std::vector<pic::EnsRun> runs;        // slot order
    pic::EnsRun *d_runs = nullptr;
    long long nslots = 0, nnodes = 0, nmodes = 0, nkeys = 0;
    int chunk = 8192, halo = 2, sort_every = 20, hist_cap = 4096;
    // particles, two buffers
    int32_t *cell[2] = {nullptr, nullptr};
    float *ox[2] = {nullptr, nullptr}, *oy[2] = {nullptr, nullptr};
    float *vx[2] = {nullptr, nullptr}, *vy[2] = {nullptr, nullptr};
    uint32_t *pid[2] = {nullptr, nullptr};
    // grids
    unsigned long long *rho_fix = nullptr;
    float *rho = nullptr, *e = nullptr;
    float2 *rhohat = nullptr, *ehat = nullptr;
    // sort
    uint32_t *count = nullptr, *offset = nullptr, *cursor = nullptr;
    uint32_t *bsum = nullptr, *bsum_s = nullptr, *bsum2 = nullptr;
    long long *d_total = nullptr;
    // work tables
    pic::SegBlock *push_blk = nullptr, *sort_blk = nullptr, *node_blk = nullptr, *mode_blk = nullptr;
    pic::SegBlock *hist_blk = nullptr;  // histogram blocks: four sort chunks of one run
    int npush = 0, nsort = 0, nnode_blk = 0, nmode_blk = 0, nhist = 0;
    int32_t *anchor = nullptr;
    size_t push_smem = 0;
    // diagnostics
    pic::DevState *dev = nullptr;
    double *hist = nullptr;
    // FFT groups: runs of one grid size, adjacent slots
    struct Group {
        int nx, ny, first, count;
        cufftHandle r2c = 0, c2r = 0;
        cufftHandle r2c2 = 0, c2r1 = 0;  // adjoint solve (made on first use)
        float2 *tw = nullptr;            // spectral solve's twiddle tables
    };
    std::vector<Group> groups;
    // every group's side lengths are powers of two (16..4096): the step's
    // solve runs in the spectral kernels, one launch of each per group
    bool spectral = false;
    // graphs
    cudaGraphExec_t g_one = nullptr, g_period = nullptr, g_sortstep = nullptr;
    int since_sort = 0;
    bool ready = false;
    // export staging
    double *stage = nullptr;
    size_t stage_n = 0;
};

namespace pic {

pic_status ens_need(pic_ensemble *E, int run);
template <class T> pic_status ens_alloc(T **p, size_t n)
{
    *p = nullptr;
    PIC_CUDA(cudaMalloc((void **)p, (n ? n : 1) * sizeof(T)));
    return PIC_OK;
}
// particle pass over every run: kind 0 step (gather, drift, deposit), 1 prime
// (kick -1/2, no drift, no deposit), 2 deposit only, 3 drift back by one step
// (x -= dt v) and deposit
pic_status ens_launch_push(pic_ensemble *E, int src, int kind);
pic_status ens_advance(pic_ensemble *E, int kind);
pic_status ens_poisson(pic_ensemble *E);
// sort every run from buffer 0 into buffer 1 (and the four extra per-particle
// arrays xin -> xout when given), push-block anchors
pic_status ens_sort(pic_ensemble *E, const float *const *xin = nullptr, float *const *xout = nullptr);
pic_status ens_graphs(pic_ensemble *E);
// pic_import.cu: every run, arbitrary order in buffer 0 -> key order in
// buffer 1; scratch holds 4 words per slot (12 with packed records), CUB
// temporary storage grows in temp
pic_status ens_import_sort(pic_ensemble *E, uint32_t *scratch, bool packed, void **temp,
                           size_t *temp_bytes);

}  // namespace pic
