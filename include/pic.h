/*
 * pic.h -- C ABI of libpic, a GB300-native (sm_103a) 2-D electrostatic
 * particle-in-cell step: particle/grid init, charge deposit, Poisson solve,
 * field gather + push, collisions and diagnostics.
 *
 * Every call returns a pic_status; nothing calls exit().  Pointers are plain
 * host pointers unless a name says "_dev".  A handle owns its CUDA stream and
 * all device buffers; one handle per host thread makes the library re-entrant.
 *
 * Reference interfaces replaced (paths inside taylorj5/msc-thesis,
 * thesisCode/collisionless/double/ unless stated):
 *   pic_compat_run        <- picFloatGpu              inc/pic.h:5-7, src/pic.cu:429-611
 *   pic_compat_run_steps  <- the CPU step loop body   src/main.cc:137-172
 *   pic_init_particles    <- initialiseParticles      src/main.cc:201-244
 *   pic_set_particles     <- Particle::Particle       src/particle.cc:21-29
 *   pic_deposit           <- Grid::chargeAssignment   src/grid.cc:46-76
 *   pic_deposit_grid      <- Grid::chargeAssignment   src/grid.cc:46-76 (stateless form)
 *   pic_poisson           <- fftPoissonSolver + Grid::computeElectricField
 *                                                     src/fourier.cc:15-126, src/grid.cc:85-96
 *   pic_gather_push       <- Particle::forceCalculation + Particle::positionUpdate
 *                                                     src/particle.cc:37-106
 *   pic_collide           <- Particle::collision (mccCollisions/src/particle.cc:112-127),
 *                            collisions (dsmcCollisions/cellTrackerAdvanced/src/main.cc:288-350)
 *   pic_sort              <- cellTracking (dsmcCollisions/cellTrackerAdvanced/src/main.cc:269-278)
 *   pic_diagnostics       <- checkResults / checkError (src/main.cc:254-267;
 *                            dsmcCollisions/cellTrackerAdvanced/src/main.cc:380-408)
 *   pic_get_particles, pic_get_grid <- the D2H copies at src/pic.cu:583-584 and the
 *                            public Grid arrays (inc/grid.h:27-29)
 */
#ifndef PIC_H
#define PIC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* status                                                              */
/* ------------------------------------------------------------------ */
typedef enum pic_status {
    PIC_OK = 0,
    PIC_ERR_INVALID_ARG = 1, /* bad config or argument                     */
    PIC_ERR_OOM = 2,         /* device or host allocation failed           */
    PIC_ERR_CUDA = 3,        /* a CUDA runtime call failed                 */
    PIC_ERR_CUFFT = 4,       /* a cuFFT call failed                        */
    PIC_ERR_OVERFLOW = 5,    /* capacity exceeded (particles, cells)       */
    PIC_ERR_NAN = 6,         /* non-finite particle state detected         */
    PIC_ERR_TIMEOUT = 7,     /* a bounded device wait gave up (no kernel of
                                this library waits on another)             */
    PIC_ERR_STATE = 8,       /* call not valid in the handle's state       */
    PIC_ERR_NO_DEVICE = 9    /* no CUDA device visible                     */
} pic_status;

/* Static English text for a status. */
const char *pic_status_string(pic_status s);
/* Detail of the last failure on the calling thread ("" if none). */
const char *pic_last_error(void);
/* Library version, e.g. "1.0.0". */
const char *pic_version(void);

/* ------------------------------------------------------------------ */
/* reference drop-in: the reference's conventions, FP64 on the GPU    */
/* ------------------------------------------------------------------ */
/* The fields of the reference's struct Params that its step reads
 * (inc/params.h:21-47), as plain data.  xDim/yDim are int there too. */
typedef struct pic_ref_params {
    int xDim, yDim;      /* domain size                                   */
    int nx, ny;          /* cells per direction                           */
    int npx, npy;        /* particles = npx * npy                         */
    double dt, tmax;     /* step count = iterations of while (t < tmax)   */
    double charge, mass; /* macro-particle charge and mass                */
    double vtx, vty, vdx, vdy;
} pic_ref_params;

/* Drop-in for picFloatGpu (inc/pic.h:6): copies the four initial particle
 * arrays to the device, runs the reference's step (src/main.cc:137-172 with
 * the CPU conventions of grid.cc, fourier.cc, particle.cc) for as many
 * steps as `while (t < tmax) t += dt` iterates, and copies the final
 * positions back.  *seconds (may be NULL) receives the elapsed time of the
 * whole call, as picFloatGpu returns it.  Unlike picFloatGpu the deposit
 * is atomic, the density is zeroed each step and forceOld starts at zero for
 * every particle, so the result follows the reference's CPU path. */
pic_status pic_compat_run(const pic_ref_params *p, const double *posX, const double *posY,
                          const double *velX, const double *velY, double *xOut, double *yOut,
                          double *seconds);

/* Same step for an explicit number of steps, returning the final particle
 * arrays and the ghost-padded (nx+2)*(ny+2) grids rho, phi, Ex, Ey (row
 * index = x cell, as in the reference's Grid).  Any output may be NULL. */
pic_status pic_compat_run_steps(const pic_ref_params *p, const double *x0, const double *y0,
                                const double *vx0, const double *vy0, long long nsteps,
                                double *x, double *y, double *vx, double *vy, double *rho,
                                double *phi, double *ex, double *ey);

/* ------------------------------------------------------------------ */
/* physics-mode handle                                                 */
/* ------------------------------------------------------------------ */
#define PIC_MAX_SPECIES 4

enum pic_species_flags {
    PIC_SPECIES_HAS_VZ = 1 /* carry a third velocity component (collisions) */
};

typedef struct pic_species_desc {
    long long capacity; /* maximum particle count held on the device           */
    double q;           /* macro-particle charge (0 for a neutral species)     */
    double m;           /* macro-particle mass                                 */
    int q_int;          /* charge in deposit units: q = q_int * unit charge    */
    int flags;          /* pic_species_flags                                   */
} pic_species_desc;

typedef struct pic_config {
    int nx, ny;          /* cells; periodic in both directions                */
    double Lx, Ly;       /* domain lengths                                    */
    double dt;           /* time step                                         */
    double eps0;         /* vacuum permittivity in the chosen units           */
    int nspecies;
    pic_species_desc species[PIC_MAX_SPECIES];
    int sort_every;      /* steps between counting sorts (0: 20)              */
    int tile_w, tile_h;  /* sort tile in cells (0: chosen from the density)   */
    int chunk;           /* particles per push block, multiple of 4, at most
                            32768 (0: 8192)                                   */
    int halo;            /* shared-memory window halo in cells (0: 4, or less
                            where the window would exceed 56 KB; windows over
                            112 KB are refused)                               */
    int history;         /* diagnostic history length in steps (0: 4096)      */
    int device;          /* CUDA device ordinal                               */
    int push_variant;    /* 0: auto (1), 1: direct 128-bit loads, 3: direct
                            loads with deposit groups summed across the warp
                            (2 and 4, bulk-copy pipelines measured slower
                            than 1, were removed and are refused)             */
} pic_config;

typedef struct pic_handle pic_handle;

pic_status pic_config_default(pic_config *cfg);
/* Power-of-two grids of 16..4096 cells a side solve the field with the
 * library's spectral kernels, other sizes with cuFFT; the environment
 * variable PIC_FIELD_SOLVER=cufft, read here, selects cuFFT for any size. */
pic_status pic_create(const pic_config *cfg, pic_handle **out);
pic_status pic_destroy(pic_handle *h);
/* The CUDA stream all of the handle's work runs on (cudaStream_t). */
pic_status pic_get_stream(pic_handle *h, void **stream);
/* Wait for the handle's stream; reports device error flags. */
pic_status pic_synchronize(pic_handle *h);

enum pic_load { PIC_LOAD_RANDOM = 0, PIC_LOAD_LATTICE = 1 };
enum pic_pert {
    PIC_PERT_NONE = 0,
    PIC_PERT_XDISP = 1,   /* x += amp cos(kx x)                                  */
    PIC_PERT_DENSITY = 2, /* n ~ 1 + amp cos(k.x), by displacement along k        */
    PIC_PERT_BEAM_MODE = 3 /* per beam b: x += Re(xi_b e^{i kx x}), vx += Re(u_b e^{i kx x}) */
};

typedef struct pic_init_spec {
    long long n;        /* particles to create                                */
    int layout;         /* pic_load                                           */
    int pert_kind;      /* pic_pert                                           */
    double vth[3];      /* thermal speeds (Gaussian sigma) per component      */
    double vdrift[2];   /* drift velocity                                     */
    double beam_v;      /* != 0: two beams, +beam_v (even id) / -beam_v (odd) */
    double pert_amp;    /* XDISP: x += amp cos(kx x); DENSITY: n ~ 1+amp cos(k.x) */
    int pert_mx, pert_my; /* perturbation mode numbers (k = 2 pi m / L)       */
    unsigned long long seed;
    /* PIC_PERT_BEAM_MODE: complex amplitudes (re, im) per beam, beam 0 = even
     * ids (+beam_v), beam 1 = odd ids; lets a caller load a linear eigenmode */
    double beam_xi[2][2];
    double beam_u[2][2];
} pic_init_spec;

/* Create spec->n particles of a species on the device (Philox streams keyed
 * by seed and particle id), sort them, deposit and solve for E. */
pic_status pic_init_particles(pic_handle *h, int species, const pic_init_spec *spec);
/* Replace a species' particles from host arrays: positions in [0, L)
 * (global coordinates), velocities; vz may be NULL.  Particle ids are the
 * array indices.  Sorts, deposits and solves for E afterwards.  Page-locked
 * arrays are read in place by the GPU; the sort borrows up to 48 bytes of
 * device memory per slot (16 when less is free or the environment variable
 * PIC_STAGE_MAX_BYTES caps it; the result is the same). */
pic_status pic_set_particles(pic_handle *h, int species, long long n, const double *x,
                             const double *y, const double *vx, const double *vy,
                             const double *vz);
/* Copy a species to host arrays in particle-id order (id i -> index i).
 * *n receives the count; any array may be NULL.  Borrows 8 bytes of device
 * memory per particle and requested array plus 8 per particle for the
 * reordering (4 per slot under PIC_STAGE_MAX_BYTES or low memory). */
pic_status pic_get_particles(pic_handle *h, int species, long long *n, double *x, double *y,
                             double *vx, double *vy, double *vz);

/* Copy a species' raw device storage to host arrays in storage order, not
 * id order: after a sort the DSMC species is ordered by cell, every other
 * species by tile and, within a tile, by cell row (tile-major cell index /
 * tile_w); any array may be NULL. */
pic_status pic_get_particles_raw(pic_handle *h, int species, long long *n, int32_t *cell,
                                 float *ox, float *oy, float *vx, float *vy, uint32_t *pid);

/* Borrowed device views of a species' SoA storage (valid until the next
 * call that sorts or resizes): cell = cx | (cy << 16) (int32), in-cell
 * offsets ox, oy in [0,1) (float), velocities (float), particle id (uint32). */
typedef struct pic_particles_view {
    long long n;
    int32_t *cell_dev;
    float *ox_dev, *oy_dev, *vx_dev, *vy_dev, *vz_dev;
    uint32_t *pid_dev;
} pic_particles_view;
pic_status pic_particles_device(pic_handle *h, int species, pic_particles_view *v);

/* Time-leapfrog priming: v <- v - (q/m) E(x) dt/2 for every charged
 * species, using the current field. */
pic_status pic_prime_leapfrog(pic_handle *h);

/* ---- the step stages ---- */
pic_status pic_sort(pic_handle *h);    /* counting sort of every species: by tile row,
                                          the DSMC species by cell */
pic_status pic_deposit(pic_handle *h); /* fixed-point rho from the current positions  */
pic_status pic_poisson(pic_handle *h); /* rho -> E (spectral solve, see pic_create)    */
/* Gather E, push every species one step; with deposit != 0 the new charge
 * density is deposited in the same pass (then pic_poisson gives E). */
pic_status pic_gather_push(pic_handle *h, int deposit);

enum pic_collide_kind { PIC_COLLIDE_MCC = 1, PIC_COLLIDE_DSMC = 2 };

/* Electron-neutral Monte Carlo collisions against a uniform background gas,
 * by the null-collision method (Vahedi & Surendra, Comput. Phys. Commun. 87
 * (1995) 179): each step every electron is a candidate with probability
 * P = 1 - exp(-nu_max dt), nu_max = n_g max_E sigma_T(E) v(E); a candidate's
 * process follows from one uniform number against nu_j(E)/nu_max.
 * Processes: elastic (isotropic, energy loss 2 m/M (1 - cos chi) E),
 * excitation (E -= e_exc, isotropic), ionisation (E -= e_ion, the rest
 * split uniformly between scattered and ejected electron, each isotropic; a
 * new ion from the neutral Maxwellian at the same position).  Velocities
 * are 3-D (species need PIC_SPECIES_HAS_VZ).  Random numbers: Philox4x32-10
 * keyed by seed, counter (particle id, collision pass, stream).  Replaces
 * the reference's constant-probability velocity resample
 * (mccCollisions/src/particle.cc:112-127, mccCollisions/src/pic.cu:435-466). */
typedef struct pic_mcc_params {
    int electron_species;     /* species index of the electrons                 */
    int ion_species;          /* species receiving ionisation ions (-1: none)   */
    double neutral_density;   /* n_g, m^-3                                      */
    double neutral_temp_eV;   /* background temperature (ion birth velocities)  */
    double electron_mass;     /* physical electron mass, kg (energies)          */
    double ion_mass;          /* physical ion / neutral mass, kg                */
    double unit_charge;       /* C per eV                                       */
    int ntab;                 /* table points, log-spaced in [e_min, e_max] eV  */
    double e_min_eV, e_max_eV;
    const double *sigma_elastic;    /* ntab cross sections, m^2 (copied)        */
    const double *sigma_excitation;
    const double *sigma_ionization;
    double e_exc_eV, e_ion_eV; /* thresholds = energy losses                    */
    unsigned long long seed;
} pic_mcc_params;
/* Configure MCC (once; the tables are copied).  pic_step then runs one MCC
 * pass after each push; pic_collide(h, PIC_COLLIDE_MCC) runs one pass now. */
pic_status pic_set_mcc(pic_handle *h, const pic_mcc_params *p);

/* Neutral-neutral DSMC with Bird's no-time-counter scheme (Bird, Molecular
 * Gas Dynamics and the Direct Simulation of Gas Flows, 1994), hard spheres:
 * per cell of the cell-sorted array, N = 1/2 n (n-1) F_N (sigma g)_max dt_c
 * / V_c candidate pairs (fraction by randomised rounding), each accepted
 * with probability sigma g / (sigma g)_max, isotropic scattering in the
 * centre-of-mass frame.  (sigma g)_max is kept per cell and raised when
 * exceeded.  Replaces the reference's nearest-neighbour toy
 * (dsmcCollisions/cellTrackerAdvanced/src/main.cc:288-350, src/pic.cu:791-870). */
typedef struct pic_dsmc_params {
    int species;              /* neutral species (q = 0, PIC_SPECIES_HAS_VZ)    */
    double diameter;          /* hard-sphere diameter, m                        */
    double weight;            /* F_N: real atoms per macro-particle             */
    double depth;             /* cell depth for the 2-D cell volume, m          */
    double sigma_g_max0;      /* initial (sigma g)_max per cell, m^3/s          */
    int every;                /* collide every `every` steps, dt_c = every*dt (0: 1) */
    unsigned long long seed;
} pic_dsmc_params;
pic_status pic_set_dsmc(pic_handle *h, const pic_dsmc_params *p);

/* One collision pass now (MCC: on the live arrays; DSMC: sorts the neutral
 * species by cell first). */
pic_status pic_collide(pic_handle *h, int kind);

/* Cumulative collision counts since init: [0] elastic, [1] excitation,
 * [2] ionisation, [3] null candidates, [4] DSMC collisions,
 * [5] DSMC candidate pairs. */
pic_status pic_collision_counts(pic_handle *h, long long counts[6]);

/* nsteps full steps (push+deposit, Poisson, sort every sort_every), replayed
 * from CUDA graphs.  Asynchronous: returns once the work is queued. */
pic_status pic_step(pic_handle *h, long long nsteps);

/* Whole run from and to host memory through one call, as the reference's
 * GPU driver is used: copy species 0 in (global coordinates), deposit,
 * solve, prime the leapfrog when prime != 0, step nsteps times and copy the
 * final state back (in id order).  Outputs may alias inputs. */
pic_status pic_run_host(pic_handle *h, long long n, const double *x, const double *y,
                        const double *vx, const double *vy, long long nsteps, int prime,
                        double *x_out, double *y_out, double *vx_out, double *vy_out);

/* ---- checkpoints ----
 * A state file holds the grid geometry, the step and collision-pass
 * counters and every species' particles (cell, offsets, velocities, ids) in
 * storage order: little-endian, magic "PICSTATE", version 1.  A
 * collisionless run resumed from a file continues bit for bit as the
 * uninterrupted run; collision operators continue their random streams
 * (keyed by particle id and pass counter).  Collision settings are not in
 * the file: set them on the loading handle.  No counterpart in the
 * reference (it keeps no state between runs). */
pic_status pic_save(pic_handle *h, const char *path);
/* Load a state file into a handle created with the same nx, ny, Lx, Ly, dt,
 * eps0 and species (same count, flags, q_int, q and m), each species'
 * capacity at least the saved count; the field is recomputed from the
 * loaded positions.  The
 * whole file is read and checked first (cells on the grid or -1, offsets in
 * [0, 1), finite velocities, ids a permutation, no trailing bytes): a bad
 * file returns PIC_ERR_INVALID_ARG and leaves the handle unchanged. */
pic_status pic_load(pic_handle *h, const char *path);

/* ---- adjoint of the collisionless step ----
 * Gradients of J = final field energy (1/2 eps0 sum |E|^2 dA after nsteps)
 * by the discrete adjoint of the GPU step, for a handle with one charged
 * species (species 0) and no collision operator.  The map differentiated
 * is: v(-1/2) = v0 - (q/m) E(x0) dt/2, then nsteps leapfrog steps.
 * Backward: a_v += dt a_x; a_x += [dt (q/m) dF/dx]^T a_v, where the transpose
 * is the local CIC-gradient term, the scatter of mu = dt (q/m) a_v to the
 * grid (the adjoint of the gather), the k-space solve psi^ = i k.g^ /
 * (eps0 k^2) (the Poisson-gradient operator transposed) and the CIC-gradient
 * gather of psi (the adjoint of the deposit).  Checkpoints of (x, v) every
 * `every` steps; each segment is recomputed forward into a ring of positions
 * and fields and walked backwards.  The run does not re-sort particles.
 * The initial state is spec's load (spec != NULL) or the particles already
 * loaded and not yet primed, as pic_set_particles leaves them (spec ==
 * NULL).  Gradient arrays are in particle-id order (may be NULL).  With
 * spec, dJ/d(beam_v) and dJ/d(pert_amp) follow from the initial gradients
 * and the load's derivatives (pert_amp: PIC_PERT_XDISP and
 * PIC_PERT_DENSITY; 0 for the other kinds).  The 2^-16 quantisation of the
 * deposit weights is not differentiated.  Device memory: 20 bytes per
 * particle slot per checkpoint plus `every` x (12 bytes per slot + 8 bytes
 * per cell) for the ring.  Leaves the handle at step nsteps, with the
 * history of the forward run.  No counterpart in the reference. */
typedef struct pic_adjoint_result {
    double J;           /* final field energy                                 */
    double dJ_dbeam_v;  /* d J / d(spec->beam_v)   (spec given)               */
    double dJ_damp;     /* d J / d(spec->pert_amp) (spec given)               */
} pic_adjoint_result;
pic_status pic_adjoint_run(pic_handle *h, const pic_init_spec *spec, long long nsteps, int every,
                           double *dJ_dx0, double *dJ_dy0, double *dJ_dvx0, double *dJ_dvy0,
                           pic_adjoint_result *out);

/* ---- autotuning ---- */
typedef struct pic_tune_result {
    int chunk;            /* particles per push block                        */
    int tile_w, tile_h;   /* sort tile (cells)                               */
    int sort_every;       /* steps between counting sorts                    */
    double ms_per_step;   /* measured with the chosen values                 */
    int tried;            /* candidates timed                                */
} pic_tune_result;
/* Pick the push chunk (and with it the sort tile) and the sort cadence for a
 * workload by timing short runs: for each candidate a handle is created from
 * *cfg, species `species` is loaded from *spec, the leapfrog primed and
 * `trial_steps` steps (rounded up to whole sort periods) timed with CUDA
 * events after one warm-up period.  Chunk is searched first (4096, 8192,
 * 16384) at the configured cadence, then the cadence (2, 5, 10, 20, 40, 80).  The
 * chosen values are written into *cfg.  Needs the memory of one handle at a
 * time. */
pic_status pic_autotune(pic_config *cfg, int species, const pic_init_spec *spec,
                        int trial_steps, pic_tune_result *out);

/* ---- diagnostics ---- */
typedef struct pic_diag {
    long long step;              /* completed steps                           */
    double field_energy;         /* 1/2 eps0 sum |E|^2 dA at `step`           */
    double kinetic_energy;       /* at step-1 (time-centred), all species     */
    double momentum[2];          /* at step-1, all species                    */
    long long total_charge_fixed; /* sum of the fixed-point density (2^-32 q units) */
    long long expected_charge_fixed; /* sum over species of q_int * n * 2^32  */
    long long n[PIC_MAX_SPECIES];
    unsigned int error_flags;    /* PIC_DEVERR_* bits                         */
} pic_diag;

enum pic_device_errors {
    PIC_DEVERR_NAN = 1,       /* a particle had a non-finite velocity          */
    PIC_DEVERR_CAPACITY = 2,  /* a species ran out of capacity (ionisation)    */
    PIC_DEVERR_CELL = 4,      /* a cell index outside the grid was seen        */
    PIC_DEVERR_TIMEOUT = 8,   /* a bounded device wait gave up (unused: no
                                 kernel of this library waits on another)     */
    PIC_DEVERR_SORT = 16      /* a sort destination fell outside the slots
                                 (cell counts inconsistent with the particles;
                                 the particle was left unmoved)               */
};

pic_status pic_diagnostics(pic_handle *h, pic_diag *d);

enum pic_history {
    PIC_HIST_FIELD_ENERGY = 0, /* indexed by step (0 = initial field)          */
    PIC_HIST_KINETIC = 1,      /* indexed by step of the push                  */
    PIC_HIST_MOMENTUM_X = 2,
    PIC_HIST_MOMENTUM_Y = 3,
    PIC_HIST_CHARGE = 4,       /* total fixed-point charge, as a double        */
    PIC_HIST_MODE_AMP = 5      /* |rho^(mx,my)| of the tracked mode (pic_track_mode) */
};
/* Copy history entries [first, first+count) (steps) to host. */
pic_status pic_get_history(pic_handle *h, int which, long long first, long long count,
                           double *out);

/* ---- ensembles of independent runs ----
 * Many independent collisionless runs, each with its own grid, particle
 * count and load, advanced together: every stage of a step is one launch
 * over all runs (push, sort, density conversion, k-space kernel, diagnostics
 * fold), the FFTs are batched over the runs of each grid size, and steps are
 * replayed from CUDA graphs.  A per-run offset table (particle slots, grid
 * nodes, spectrum, sort keys) and per-block work tables drive the kernels.
 * Run r follows runs[r]: nx, ny, Lx, Ly, dt, eps0 and species[0] (one
 * charged species: capacity, q, m, q_int); its sort tiles are chosen from
 * its particles per cell.  chunk, halo, sort_every, history and device are
 * taken from runs[0] (0: the handle defaults).  A run gives the same
 * particles as a handle created from runs[r] and stepped alike.  No
 * counterpart in the reference (it runs one simulation per process). */
typedef struct pic_ensemble pic_ensemble;
pic_status pic_ensemble_create(const pic_config *runs, int nruns, pic_ensemble **out);
pic_status pic_ensemble_destroy(pic_ensemble *e);
pic_status pic_ensemble_get_stream(pic_ensemble *e, void **stream);
pic_status pic_ensemble_synchronize(pic_ensemble *e);
/* Load run r from specs[r] (specs[r].n <= its capacity), sort, deposit,
 * solve, and prime the leapfrog (v to t = -dt/2) of every run. */
pic_status pic_ensemble_init(pic_ensemble *e, const pic_init_spec *specs);
pic_status pic_ensemble_step(pic_ensemble *e, long long nsteps);
pic_status pic_ensemble_diagnostics(pic_ensemble *e, int run, pic_diag *d);
pic_status pic_ensemble_get_history(pic_ensemble *e, int run, int which, long long first,
                                    long long count, double *out);
pic_status pic_ensemble_get_particles(pic_ensemble *e, int run, long long *n, double *x, double *y,
                                      double *vx, double *vy);
/* Discrete adjoint of every run of the ensemble (see pic_adjoint_run): each
 * run is loaded from specs[r], primed and stepped nsteps times, and the
 * gradients of its final field energy J_r with respect to its initial state
 * are computed.  Memory: instead of a ring of recomputed positions, each
 * segment of `every` steps is walked backwards by reversing the leapfrog
 * (x -= dt v, field of the reversed positions, v -= dt (q/m) F) from an
 * exact checkpoint of its end state, so the ensemble keeps one checkpoint
 * (24 bytes per particle slot) per segment and no per-step storage;
 * checkpoints go to pinned host memory when device memory runs out.  The
 * adjoint arrays travel with the particles through the sorts.  out[r]
 * (nruns entries) receives J_r, dJ_r/d(beam_v) and dJ_r/d(pert_amp) of
 * specs[r]; gradient arrays (may be NULL) are the runs' arrays in run order,
 * each in particle-id order (run r starts after the particles of runs
 * 0..r-1).  Leaves the ensemble at step nsteps.  No counterpart in the
 * reference. */
pic_status pic_ensemble_adjoint(pic_ensemble *e, const pic_init_spec *specs, long long nsteps,
                                int every, double *dJ_dx0, double *dJ_dy0, double *dJ_dvx0,
                                double *dJ_dvy0, pic_adjoint_result *out);
/* Pick the push chunk (and with it every run's sort tile) and the sort
 * cadence of an ensemble by timing short runs of it, as pic_autotune does
 * for one handle: chunk from (2048, 4096, 8192, 16384), then cadence from
 * (1, 2, 3, 5, 10, 20).  The chosen chunk and sort_every are written into
 * runs[0]; out->tile_w/tile_h are 0 (tiles differ per run).  Needs the
 * memory of one ensemble at a time. */
pic_status pic_ensemble_autotune(pic_config *runs, int nruns, const pic_init_spec *specs,
                                 int trial_steps, pic_tune_result *out);

/* Track |rho^| of one Fourier mode each step (PIC_HIST_MODE_AMP). */
pic_status pic_track_mode(pic_handle *h, int mx, int my);

enum pic_grid_kind { PIC_GRID_RHO = 0, PIC_GRID_PHI = 1, PIC_GRID_EX = 2, PIC_GRID_EY = 3 };
/* Copy a grid (row-major [iy][ix], nx*ny doubles) to host.  RHO is the net
 * charge density of the last field solve, i.e. the particles' density plus
 * the uniform neutralising background (its mean is zero); PHI is computed
 * on request from that density. */
pic_status pic_get_grid(pic_handle *h, int which, double *out);
/* The raw fixed-point density of the last deposit (int64, 2^-32 charge
 * units, before the background is removed). */
pic_status pic_get_rho_fixed(pic_handle *h, int64_t *out);

/* ------------------------------------------------------------------ */
/* stateless deposit of device particle arrays                         */
/* ------------------------------------------------------------------ */
/* CIC deposit of n particles (cell = cx | (cy << 16), offsets in [0,1))
 * into rho_dev (nx*ny doubles, row-major [iy][ix]), which is overwritten
 * with q_int * scale * (fixed-point density / 2^32).  Accumulates in an
 * int64 scratch grid that this call allocates on the device and frees.
 * stream may be NULL (legacy default stream).  Entries with cell < 0 and
 * cells off the grid are skipped without a report (the handle's kernels
 * report off-grid cells as PIC_DEVERR_CELL).  Returns after the deposit has
 * finished (it synchronises the stream). */
pic_status pic_deposit_grid(int nx, int ny, long long n, const int32_t *cell_dev,
                            const float *ox_dev, const float *oy_dev, int q_int, double scale,
                            double *rho_dev, void *stream);

/* The same deposit without any device allocation, for callers that cannot
 * call cudaMalloc: a framework that owns the GPU's memory through its own
 * pool, a process held to a fixed device-memory budget, or a loop that must
 * not pay cudaFree's device-wide synchronisation.  No counterpart in the
 * reference.  The int64 scratch grid is a static device array of
 * PIC_NOALLOC_MAX_CELLS cells (8 MiB held on every GPU that loads the
 * library); nx*ny above that is rejected with PIC_ERR_INVALID_ARG.  Unlike
 * pic_deposit_grid the call only enqueues work on `stream` (NULL: legacy
 * default stream) and returns: synchronise the stream before reading rho_dev
 * or reusing the particle arrays; kernel faults surface at that sync.
 * All calls share the scratch grid: calls whose work overlaps on the GPU
 * race.  Every call looks up the scratch address on the current device; the
 * first call on a device also loads the library's device code there, so make
 * it before any stream capture on that device.  Cells off the grid are
 * skipped without a report, as in pic_deposit_grid. */
#define PIC_NOALLOC_MAX_CELLS (1 << 20)
pic_status pic_deposit_grid_noalloc(int nx, int ny, long long n, const int32_t *cell_dev,
                                    const float *ox_dev, const float *oy_dev, int q_int,
                                    double scale, double *rho_dev, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* PIC_H */
