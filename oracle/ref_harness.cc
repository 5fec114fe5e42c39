/*
 * ref_harness.cc -- C entry points around the reference's UNMODIFIED serial
 * CPU step, compiled from the reference tree by oracle/Makefile into
 * oracle/_ref/libpicref.so.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  Used by tests/golden/make_golden.py
 * to produce golden vectors and, on machines where it was built, as a CPU
 * timing point.  Nothing in the product links it.
 *
 * What it drives (reference paths within taylorj5/msc-thesis, thesisCode/):
 *   collisionless/double/src/main.cc:201-244  initialiseParticles
 *   collisionless/double/src/main.cc:137-172  the step loop body, i.e.
 *     grid.cc:46-76   Grid::chargeAssignment
 *     fourier.cc:15-126 fftPoissonSolver
 *     grid.cc:85-96   Grid::computeElectricField
 *     particle.cc:37-60 Particle::forceCalculation
 *     particle.cc:69-106 Particle::positionUpdate
 * main.cc is compiled with -Dmain=thesis_reference_main so that its
 * initialiseParticles can be called; its GPU entry point is stubbed below.
 */
#include <cstring>
#include <memory>
#include <vector>

#include "fourier.h"
#include "grid.h"
#include "params.h"
#include "particle.h"

void initialiseParticles(std::vector<Particle> &particles, std::shared_ptr<Params> p);

extern "C" {

/* The reference's main.cc references its GPU driver; the oracle never calls
 * it, so a stub satisfies the linker. */
double picFloatGpu(double *, double *, double *, double *, double *, double *, std::shared_ptr<Params>)
{
    return -1.0;
}

/* Plain-old-data mirror of the fields of struct Params
 * (collisionless/double/inc/params.h:21-47) that the step reads. */
typedef struct ref_params {
    int xDim, yDim, nx, ny, npx, npy;
    double dt, tmax, charge, mass, vtx, vty, vdx, vdy;
} ref_params;

static std::shared_ptr<Params> make_params(const ref_params *rp)
{
    auto p = std::make_shared<Params>();
    p->xDim = rp->xDim;
    p->yDim = rp->yDim;
    p->nx = rp->nx;
    p->ny = rp->ny;
    p->numParticlesX = rp->npx;
    p->numParticlesY = rp->npy;
    p->dt = rp->dt;
    p->tmax = rp->tmax;
    p->electronCharge = rp->charge;
    p->mass = rp->mass;
    p->vtx = rp->vtx;
    p->vty = rp->vty;
    p->vdx = rp->vdx;
    p->vdy = rp->vdy;
    /* derived values exactly as main.cc:75-78 computes them */
    p->dx = (double)p->xDim / p->nx;
    p->dy = (double)p->yDim / p->ny;
    p->area = p->dx * p->dy;
    p->numParticles = p->numParticlesX * p->numParticlesY;
    return p;
}

/* Number of iterations of `while (t < tmax) { ...; t += dt; }`
 * (collisionless/double/src/main.cc:137,170). */
long ref_count_steps(double dt, double tmax)
{
    long n = 0;
    double t = 0.0;
    while (t < tmax) {
        t += dt;
        ++n;
    }
    return n;
}

/* The reference's own initial particle arrays (main.cc:201-244). */
int ref_init(const ref_params *rp, double *x, double *y, double *vx, double *vy)
{
    auto p = make_params(rp);
    std::vector<Particle> particles;
    initialiseParticles(particles, p);
    for (size_t i = 0; i < particles.size(); ++i) {
        Point pos = particles[i].getPosition();
        Point vel = particles[i].getVelocity();
        x[i] = pos.x;
        y[i] = pos.y;
        vx[i] = vel.x;
        vy[i] = vel.y;
    }
    return 0;
}

/*
 * Run `nsteps` iterations of the reference step.  Initial state comes from
 * the given arrays (x0 != NULL) or from the reference's initialiseParticles.
 * Outputs (each may be NULL): final particle arrays (numParticles doubles),
 * and the (nx+2)*(ny+2) ghost-padded grids as they stand after the last
 * step: rho, phi, Ex, Ey.
 */
int ref_run(const ref_params *rp, const double *x0, const double *y0, const double *vx0,
            const double *vy0, long nsteps, double *x, double *y, double *vx, double *vy,
            double *rho, double *phi, double *ex, double *ey)
{
    auto p = make_params(rp);
    Grid grid(p->nx, p->ny, p->numParticles, p);
    std::vector<Particle> particles;
    if (x0) {
        particles.reserve(p->numParticles);
        for (int i = 0; i < p->numParticles; ++i) {
            particles.emplace_back(Point{x0[i], y0[i]}, p);
            particles.back().setVelocity(Point{vx0[i], vy0[i]});
        }
    } else {
        initialiseParticles(particles, p);
    }
    for (long s = 0; s < nsteps; ++s) {
        grid.chargeAssignment(particles);
        fftPoissonSolver(grid, p);
        grid.computeElectricField();
        for (auto it = particles.begin(); it != particles.end(); ++it) it->forceCalculation(grid, p);
        for (auto it = particles.begin(); it != particles.end(); ++it) it->positionUpdate(p);
    }
    for (size_t i = 0; i < particles.size(); ++i) {
        Point pos = particles[i].getPosition();
        Point vel = particles[i].getVelocity();
        if (x) x[i] = pos.x;
        if (y) y[i] = pos.y;
        if (vx) vx[i] = vel.x;
        if (vy) vy[i] = vel.y;
    }
    const size_t ng = (size_t)(p->nx + 2) * (p->ny + 2);
    for (size_t k = 0; k < ng; ++k) {
        if (rho) rho[k] = grid.chargeDensity[k];
        if (phi) phi[k] = grid.electricPotential[k];
        if (ex) ex[k] = grid.electricField[k].x;
        if (ey) ey[k] = grid.electricField[k].y;
    }
    return 0;
}

} /* extern "C" */
