/*
 * pic_oracle.h -- CPU oracle for the 2-D electrostatic PIC step.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline / reference legs of bench.py may load this library; the
 * product (libpic) never links or calls it.
 *
 * Three parts:
 *  1. compat  -- a plain-C restatement of the reference's serial CPU step
 *                (taylorj5/msc-thesis thesisCode/collisionless/double/src/
 *                grid.cc, fourier.cc, particle.cc), FP64, with every
 *                convention of that code kept.  Pinned bit-for-bit against
 *                the reference itself (oracle/_ref) by the golden tests.
 *  2. physics -- a standard FP64 PIC step (CIC to cell-corner nodes,
 *                spectral Poisson with k = 2 pi m / L, E = -i k phi,
 *                leapfrog), the checker for the GPU's physics mode.
 *  3. exact integer restatements of GPU work: Philox4x32-10 and the
 *                fixed-point (2^-32 charge units) CIC deposit.
 */
#ifndef PIC_ORACLE_H
#define PIC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Fields of the reference's struct Params (collisionless/double/inc/params.h:21-47)
 * that the step reads.  Same layout as ref_params in ref_harness.cc. */
typedef struct orc_ref_params {
    int xDim, yDim, nx, ny, npx, npy;
    double dt, tmax, charge, mass, vtx, vty, vdx, vdy;
} orc_ref_params;

long orc_count_steps(double dt, double tmax);

/* Reference-convention lattice positions (main.cc:207-217); velocities are
 * drawn from Philox normals (the reference's libstdc++ engine is not
 * restated), then the reference's mean/drift correction (main.cc:226-243)
 * is applied. */
void orc_compat_init(const orc_ref_params *p, uint64_t seed, double *x, double *y, double *vx,
                     double *vy);

/* nsteps of the reference step from the given state.  Outputs as in
 * ref_run (ref_harness.cc); any may be NULL.  nthreads > 1 parallelises the
 * particle loops and the deposit (the deposit then sums in a different
 * order, so only nthreads == 1 is bit-identical to the reference). */
int orc_compat_run(const orc_ref_params *p, const double *x0, const double *y0, const double *vx0,
                   const double *vy0, long nsteps, double *x, double *y, double *vx, double *vy,
                   double *rho, double *phi, double *ex, double *ey, int nthreads);

/* ---------------- physics mode ---------------- */
typedef struct orc_phys_cfg {
    int nx, ny;
    double Lx, Ly, dt, eps0;
    int nspecies;
} orc_phys_cfg;

typedef struct orc_species {
    long n;
    double q, m;            /* macro-particle charge and mass */
    double *x, *y, *vx, *vy; /* in/out: positions in [0,L), velocities at half steps */
} orc_species;

/* Solve for E from the current positions (deposit + spectral Poisson) and
 * return the field energy 1/2 eps0 sum |E|^2 dA.  Grids are row-major
 * [iy][ix], nx*ny doubles, any may be NULL. */
double orc_phys_fields(const orc_phys_cfg *c, const orc_species *sp, double *rho, double *phi,
                       double *ex, double *ey, int nthreads);

/* Half step back: v -= (q/m) E(x) dt/2 for every species (leapfrog priming). */
void orc_phys_prime(const orc_phys_cfg *c, orc_species *sp, int nthreads);

/* nsteps leapfrog steps.  Histories (NULL to skip):
 *   fe[0..nsteps]   field energy after each field solve (fe[0] = initial)
 *   ke[0..nsteps-1] kinetic energy at integer time, 1/2 m (|v-|^2+|v+|^2)/2
 *   px, py[0..nsteps-1] momentum m (v- + v+)/2
 * Final grids as in orc_phys_fields. */
int orc_phys_run(const orc_phys_cfg *c, orc_species *sp, long nsteps, double *fe, double *ke,
                 double *px, double *py, double *rho, double *phi, double *ex, double *ey,
                 int nthreads);

/* ---------------- exact integer restatements ---------------- */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Fixed-point CIC deposit, as the GPU computes it: cell = cx | (cy << 16)
 * (cell < 0 marks an empty slot); per particle
 * fx = rint(ox * 2^16), fy = rint(oy * 2^16) (ties to even), node weights
 * (2^16-fx)(2^16-fy), fx(2^16-fy), (2^16-fx)fy, fx fy at the cell's four
 * corner nodes, times q_int, added into rho (int64, row-major [iy][ix]). */
void orc_deposit_fixed(int nx, int ny, long n, const int32_t *cell, const float *ox,
                       const float *oy, int64_t q_int, int64_t *rho);

/* ---------------- collision operators (restatements of pic_collide.cu) ----
 * Same algorithms, same Philox counters and the same 24-bit uniform
 * conversion as the GPU, in double precision.  MCC draws are keyed by
 * (particle id, pass, stream); the i-th candidate's decisions therefore
 * match the GPU's except where a float comparison lands on the other side. */
typedef struct orc_mcc {
    int ntab;
    double e_min, e_max;
    const double *sel, *sexc, *sion;
    double ng, half_me_over_e, two_m_over_M, e_exc, e_ion, vth_ion;
    double nu_max, p_null; /* as the GPU uses them (float-rounded by the caller) */
    uint64_t seed;
} orc_mcc;

/* One MCC pass over n electrons (velocities in/out).  Ionisations append
 * the ejected electron's velocity to new_e[3*k..] and the ion's to
 * new_i[3*k..] (k < cap_new) and the parent's index to parent[k].
 * counts: elastic, excitation, ionisation, null.  Returns new pairs. */
long orc_mcc_pass(const orc_mcc *m, long n, const uint32_t *pid, double *vx, double *vy,
                  double *vz, uint64_t pass, long cap_new, double *new_e, double *new_i,
                  long *parent, long counts[4]);

/* npasses MCC passes (first_pass, first_pass + 1, ...) over n electrons
 * whose ids and velocities persist between passes (velocities in/out), with
 * no field between passes; ionisations scatter the parent but their new
 * particles are not kept.  counts accumulate as for orc_mcc_pass. */
void orc_mcc_passes(const orc_mcc *m, long n, const uint32_t *pid, double *vx, double *vy,
                    double *vz, uint64_t first_pass, long npasses, long counts[4], int nthreads);

/* DSMC (hard spheres, Bird's NTC) of one neutral species with free
 * streaming, nsteps steps: each step groups particles by cell (cx + cy*nx),
 * collides per cell, then moves x += v dt (periodic).  sgmax: per cell,
 * in/out.  T_even / T_odd (may be NULL): temperature (kelvin, 3-D) of the
 * particles with even / odd id after each step, kB T = m <|v - <v>|^2> / 3.
 * counts[0] collisions, counts[1] candidate pairs. */
typedef struct orc_dsmc {
    int nx, ny;
    double Lx, Ly, dt, sigma, coef; /* coef = F_N dt / (2 V_c) */
    double mass;                    /* physical mass (temperatures) */
    uint64_t seed;
} orc_dsmc;
void orc_dsmc_run(const orc_dsmc *d, long n, double *x, double *y, double *vx, double *vy,
                  double *vz, double *sgmax, long nsteps, uint64_t first_pass, double *T_even,
                  double *T_odd, long counts[2]);

/* ---------------- adjoint of the physics step (FP64) ----------------
 * One species on the physics-mode step: v(-1/2) = v0 - (q/m) E(x0) dt/2,
 * then nsteps leapfrog steps; J = 1/2 eps0 dA sum |E(x_N)|^2.  Stores the
 * whole trajectory (test sizes only) and runs the discrete adjoint
 * backwards: a_v += dt a_x; a_x += [dt (q/m) dF/dx]^T a_v, the transpose made
 * of the local CIC-gradient term, the scatter of mu = dt (q/m) a_v to the
 * grid, psi = S^T g (psi^ = i k.g^ / (eps0 k^2)) and the CIC-gradient gather
 * of psi.  Returns J; writes dJ/dx0, dJ/dy0, dJ/dvx0, dJ/dvy0 (n each, may be
 * NULL).  x0.. are not modified. */
double orc_adjoint(const orc_phys_cfg *c, long n, double q, double m, const double *x0,
                   const double *y0, const double *vx0, const double *vy0, long nsteps,
                   double *gx0, double *gy0, double *gvx0, double *gvy0, int nthreads);
/* Forward only, same map: J for the given initial state. */
double orc_forward_J(const orc_phys_cfg *c, long n, double q, double m, const double *x0,
                     const double *y0, const double *vx0, const double *vy0, long nsteps,
                     int nthreads);

#ifdef __cplusplus
}
#endif
#endif
