// pic_tune.cu -- autotuner for the push chunk, sort tile and sort cadence.
//
// The fastest settings depend on the workload: particles per cell set how
// many cells a push chunk covers, and particle speeds set how quickly the
// cell order decays between sorts.  pic_autotune times candidate settings on
// the caller's own configuration and initial load (coordinate search: chunk
// first, then cadence) and keeps the fastest.
#include <cuda_runtime.h>

#include <cstring>

#include "pic_internal.cuh"

namespace {

pic_status time_candidate(const pic_config &c, int species, const pic_init_spec *spec,
                          int trial_steps, double *ms, int *tw, int *th)
{
    pic_handle *h = nullptr;
    PIC_TRY(pic_create(&c, &h));
    pic_status st = pic_init_particles(h, species, spec);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const int S = h->cfg.sort_every;
    const long long steps = ((long long)(trial_steps + S - 1) / S) * S;
    if (st == PIC_OK) st = pic_prime_leapfrog(h);
    if (st == PIC_OK) st = pic_step(h, S);  // warm-up period (graphs built, sort done)
    if (st == PIC_OK) st = pic_synchronize(h);
    if (st == PIC_OK && cudaEventCreate(&e0) != cudaSuccess) st = PIC_ERR_CUDA;
    if (st == PIC_OK && cudaEventCreate(&e1) != cudaSuccess) st = PIC_ERR_CUDA;
    if (st == PIC_OK) {
        cudaEventRecord(e0, h->stream);
        st = pic_step(h, steps);
        cudaEventRecord(e1, h->stream);
        if (st == PIC_OK) st = pic_synchronize(h);
        float t = 0.f;
        if (st == PIC_OK && cudaEventElapsedTime(&t, e0, e1) == cudaSuccess)
            *ms = t / (double)steps;
        else if (st == PIC_OK)
            st = PIC_ERR_CUDA;
    }
    *tw = h->g.tw;
    *th = h->g.th;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    pic_destroy(h);
    return st;
}

}  // namespace

extern "C" pic_status pic_autotune(pic_config *cfg, int species, const pic_init_spec *spec,
                                   int trial_steps, pic_tune_result *out)
{
    if (!cfg || !spec || trial_steps < 1) {
        pic::set_error("pic_autotune: null argument or trial_steps < 1");
        return PIC_ERR_INVALID_ARG;
    }
    pic_config best = *cfg;
    best.tile_w = best.tile_h = 0;  // tiles follow the chunk
    if (!best.sort_every) best.sort_every = 20;
    double best_ms = 1e300;
    int best_tw = 0, best_th = 0, tried = 0;
    const int chunks[] = {4096, 8192, 16384};
    pic_config base = best;
    for (int c : chunks) {
        pic_config t = base;
        t.chunk = c;
        double ms = 0.0;
        int tw = 0, th = 0;
        const pic_status st = time_candidate(t, species, spec, trial_steps, &ms, &tw, &th);
        if (st == PIC_ERR_INVALID_ARG) continue;  // e.g. window too large for this chunk
        if (st != PIC_OK) return st;
        ++tried;
        if (ms < best_ms) {
            best_ms = ms;
            best = t;
            best_tw = tw;
            best_th = th;
        }
    }
    const int cadences[] = {2, 5, 10, 20, 40, 80};
    base = best;
    for (int se : cadences) {
        if (se == base.sort_every) continue;
        pic_config t = base;
        t.sort_every = se;
        double ms = 0.0;
        int tw = 0, th = 0;
        const pic_status st = time_candidate(t, species, spec, trial_steps, &ms, &tw, &th);
        if (st != PIC_OK) return st;
        ++tried;
        if (ms < best_ms) {
            best_ms = ms;
            best = t;
            best_tw = tw;
            best_th = th;
        }
    }
    if (tried == 0) {
        pic::set_error("pic_autotune: no candidate could be created");
        return PIC_ERR_INVALID_ARG;
    }
    best.tile_w = best_tw;
    best.tile_h = best_th;
    *cfg = best;
    if (out) {
        out->chunk = best.chunk;
        out->tile_w = best_tw;
        out->tile_h = best_th;
        out->sort_every = best.sort_every;
        out->ms_per_step = best_ms;
        out->tried = tried;
    }
    return PIC_OK;
}
