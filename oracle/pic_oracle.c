/*
 * pic_oracle.c -- CPU oracle for the 2-D electrostatic PIC step.
 *
 * TEST INFRASTRUCTURE ONLY (see pic_oracle.h).  Compiled with
 * -ffp-contract=off so that no multiply-add is fused and the compat part
 * reproduces the reference's IEEE double arithmetic operation for operation.
 *
 * Reference files cited below are paths inside taylorj5/msc-thesis,
 * thesisCode/collisionless/double/.
 */
#include "pic_oracle.h"
#include "orc_fft.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

static int clamp_threads(int n)
{
#ifdef _OPENMP
    if (n <= 0) n = omp_get_max_threads();
    return n;
#else
    (void)n;
    return 1;
#endif
}

/* ===================================================================== */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers:  */
/* as easy as 1, 2, 3", SC'11): 10 rounds of the 4x32 Philox S-box with  */
/* the published multipliers and Weyl key increments.                    */
/* ===================================================================== */
#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += PHILOX_W0;
            k1 += PHILOX_W1;
        }
        uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
        uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

static double u01_open(uint32_t r) { return ((double)r + 0.5) * (1.0 / 4294967296.0); }

/* ===================================================================== */
/* Part 1: compat -- the reference's serial CPU step, restated.          */
/* ===================================================================== */

/* main.cc:137,170 -- the loop `while (t < tmax) { ...; t += dt; }` */
long orc_count_steps(double dt, double tmax)
{
    long n = 0;
    double t = 0.0;
    while (t < tmax) {
        t += dt;
        ++n;
    }
    return n;
}

typedef struct compat_state {
    const orc_ref_params *p;
    double dx, dy, area;
    long np;
    int X, Y; /* ghost-padded grid extents (grid.cc:18: x = nx+2, y = ny+2) */
    double *px, *py, *cx, *cy, *vx, *vy, *fx, *fy, *fox, *foy;
    double *rho, *phi, *efx, *efy;
} compat_state;

/* main.cc:75-78 */
static void compat_derived(const orc_ref_params *p, double *dx, double *dy, double *area)
{
    *dx = (double)p->xDim / p->nx;
    *dy = (double)p->yDim / p->ny;
    *area = *dx * *dy;
}

void orc_compat_init(const orc_ref_params *p, uint64_t seed, double *x, double *y, double *vx,
                     double *vy)
{
    /* lattice positions: main.cc:207-217 (note the integer division in the
     * offset, main.cc:208-209) */
    double xOffset = 0.5 * (double)(p->xDim / p->nx);
    double yOffset = 0.5 * (double)(p->yDim / p->ny);
    long np = (long)p->npx * p->npy;
    for (int i = 0; i < p->npy; ++i) {
        double yc = ((double)p->yDim / p->npy) * (double)i + yOffset;
        for (int j = 0; j < p->npx; ++j) {
            long k = (long)i * p->npx + j;
            x[k] = ((double)p->xDim / p->npx) * (double)j + xOffset;
            y[k] = yc;
            /* Box-Muller from one Philox block per particle */
            uint32_t ctr[4] = {(uint32_t)k, (uint32_t)((uint64_t)k >> 32), 0u, 0x636f6d70u};
            uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
            uint32_t r[4];
            orc_philox4x32_10(ctr, key, r);
            double rad = sqrt(-2.0 * log(u01_open(r[0])));
            double th = 2.0 * M_PI * u01_open(r[1]);
            vx[k] = p->vtx * rad * cos(th);
            vy[k] = p->vty * rad * sin(th);
        }
    }
    /* drift correction: main.cc:226-243 */
    double sx = 0.0, sy = 0.0;
    for (long k = 0; k < np; ++k) {
        sx += vx[k];
        sy += vy[k];
    }
    double var = 1.0 / (double)np;
    sx = var * sx - p->vdx;
    sy = var * sy - p->vdy;
    for (long k = 0; k < np; ++k) {
        vx[k] -= sx;
        vy[k] -= sy;
    }
}

/* grid.cc:46-76 Grid::chargeAssignment (resetGrid at grid.cc:30-37) */
static void compat_charge_assignment(compat_state *s, int nthreads)
{
    const orc_ref_params *p = s->p;
    const int Y = s->Y;
    const size_t ng = (size_t)s->X * s->Y;
    memset(s->rho, 0, sizeof(double) * ng);
    const double totalArea = s->area;
    const double dx = s->dx, dy = s->dy, q = p->charge;

#define COMPAT_DEPOSIT_ONE(RHO, k)                                                              \
    do {                                                                                        \
        double X_ = s->px[k], Y_ = s->py[k], cx_ = s->cx[k], cy_ = s->cy[k];                    \
        double area1 = (X_ - cx_ * dx) * (Y_ - cy_ * dy) / totalArea;                           \
        double area2 = ((cx_ * dx + dx) - X_) * (Y_ - cy_ * dy) / totalArea;                    \
        double area3 = (X_ - cx_ * dx) * ((cy_ * dy + dy) - Y_) / totalArea;                    \
        double area4 = ((cx_ * dx + dx) - X_) * ((cy_ * dy + dy) - Y_) / totalArea;             \
        RHO[(size_t)((1 + cx_) * Y + (1 + cy_))] += (area1 * q);                                \
        RHO[(1 + (int)(cx_ + 1) % p->nx) * Y + (1 + (int)cy_)] += (area2 * q);                 \
        RHO[(1 + (int)cx_) * Y + (1 + (int)(cy_ + 1) % p->ny)] += (area3 * q);                 \
        RHO[(1 + (int)(cx_ + 1) % p->nx) * Y + (1 + (int)(cy_ + 1) % p->ny)] += (area4 * q);   \
    } while (0)

    if (nthreads <= 1) {
        for (long k = 0; k < s->np; ++k) COMPAT_DEPOSIT_ONE(s->rho, k);
    } else {
        double *priv = (double *)calloc((size_t)nthreads * ng, sizeof(double));
#pragma omp parallel num_threads(nthreads)
        {
            int t = 0;
#ifdef _OPENMP
            t = omp_get_thread_num();
#endif
            double *r = priv + (size_t)t * ng;
#pragma omp for schedule(static)
            for (long k = 0; k < s->np; ++k) COMPAT_DEPOSIT_ONE(r, k);
        }
        for (int t = 0; t < nthreads; ++t) {
            const double *r = priv + (size_t)t * ng;
            for (size_t i = 0; i < ng; ++i) s->rho[i] += r[i];
        }
        free(priv);
    }
#undef COMPAT_DEPOSIT_ONE

    /* periodic ghost copy, grid.cc:66-75 */
    const int nxe = p->nx + 2, nye = p->ny + 2;
    for (int i = 0; i < nye; i++) {
        s->rho[i] = s->rho[p->nx * Y + i];
        s->rho[(nxe - 1) * Y + i] = s->rho[Y + i];
    }
    for (int i = 1; i < nxe - 1; i++) {
        s->rho[i * Y] = s->rho[i * Y + p->ny];
        s->rho[i * Y + (nye - 1)] = s->rho[i * Y + 1];
    }
}

/* fourier.cc:15-126 fftPoissonSolver */
static void compat_poisson(compat_state *s)
{
    const orc_ref_params *p = s->p;
    const double pi = M_PI;
    const int nx = p->nx, ny = p->ny, nyh = p->ny / 2 + 1;
    const double norm = 1.0 / (p->nx * p->ny);
    const int Y = s->Y;
    double *in = (double *)malloc(sizeof(double) * (size_t)nx * ny);
    double *out = (double *)malloc(sizeof(double) * 2 * (size_t)nx * nyh);
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++) in[i * ny + j] = s->rho[(i + 1) * Y + (j + 1)];
    orc_fft2d_r2c(nx, ny, in, out);
    /* k-space scaling with the reference's index maps (fourier.cc:46-77) */
    for (int i = 0; i < nx; i++) {
        int II = (2 * i < nx) ? i : i - nx;
        double k1 = 2 * pi * II;
        for (int j = 0; j < nyh; j++) {
            int JJ = (2 * j < nyh) ? j : j - ny;
            double k2 = 2 * pi * JJ;
            double fact = k1 * k1 + k2 * k2;
            double *o = out + 2 * ((size_t)i * nyh + j);
            if (fabs(fact) < 1e-14) {
                o[0] = 0.0;
                o[1] = 0.0;
            } else {
                o[0] /= -fact;
                o[1] /= -fact;
            }
        }
    }
    orc_fft2d_c2r(nx, ny, out, in);
    /* the normalisation is applied twice (fourier.cc:84-93) */
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++) {
            in[i * ny + j] *= norm;
            in[i * ny + j] *= norm;
        }
    const int nxe = p->nx + 2, nye = p->ny + 2;
    for (int i = 1; i < nxe - 1; i++)
        for (int j = 1; j < nye - 1; j++) s->phi[i * Y + j] = in[(i - 1) * ny + (j - 1)];
    /* ghost copy, fourier.cc:108-115 (corners are never written) */
    for (int i = 1; i < nye - 1; i++) {
        s->phi[i] = s->phi[p->nx * Y + i];
        s->phi[(nxe - 1) * Y + i] = s->phi[Y + i];
    }
    for (int i = 1; i < nxe - 1; i++) {
        s->phi[i * Y] = s->phi[i * Y + p->ny];
        s->phi[i * Y + (nye - 1)] = s->phi[i * Y + 1];
    }
    free(in);
    free(out);
}

/* grid.cc:85-96 computeElectricField (interior only; x and y differences
 * taken along the second and first index respectively) */
static void compat_efield(compat_state *s)
{
    const orc_ref_params *p = s->p;
    const int Y = s->Y, nxe = p->nx + 2, nye = p->ny + 2;
    for (int i = 1; i < nxe - 1; i++)
        for (int j = 1; j < nye - 1; j++) {
            s->efx[i * Y + j] = (s->phi[i * Y + (j - 1)] - s->phi[i * Y + (j + 1)]) / (2 * s->dx);
            s->efy[i * Y + j] = (s->phi[(i - 1) * Y + j] - s->phi[(i + 1) * Y + j]) / (2 * s->dy);
        }
}

/* particle.cc:37-60 forceCalculation followed by particle.cc:69-106
 * positionUpdate, for particle k. */
static void compat_force_push(compat_state *s, long k)
{
    const orc_ref_params *p = s->p;
    const int Y = s->Y;
    const double dx = s->dx, dy = s->dy, totalArea = s->area;
    double X = s->px[k], Yp = s->py[k], cx = s->cx[k], cy = s->cy[k];
    double area1 = ((X - cx * dx) * (Yp - cy * dy)) / totalArea;
    double area2 = (((cx * dx + dx) - X) * (Yp - cy * dy)) / totalArea;
    double area3 = ((X - cx * dx) * ((cy * dy + dy) - Yp)) / totalArea;
    double area4 = (((cx * dx + dx) - X) * ((cy * dy + dy) - Yp)) / totalArea;
    double qm = p->charge / p->mass;
    size_t i1 = (size_t)(cx * Y + cy);
    size_t i2 = (size_t)(((int)(cx + 1) % p->nx) * Y + cy);
    size_t i3 = (size_t)(cx * Y + (int)(cy + 1) % p->ny);
    size_t i4 = (size_t)(((int)(cx + 1) % p->nx) * Y + (int)(cy + 1) % p->ny);
    double fxv = 0.0;
    fxv += area1 * s->efx[i1];
    fxv += area2 * s->efx[i2];
    fxv += area3 * s->efx[i3];
    fxv += area4 * s->efx[i4];
    fxv *= qm;
    double fyv = 0.0;
    fyv += area1 * s->efy[i1];
    fyv += area2 * s->efy[i2];
    fyv += area3 * s->efy[i3];
    fyv += area4 * s->efy[i4];
    fyv *= qm;
    s->fx[k] = fxv;
    s->fy[k] = fyv;

    double dt = p->dt;
    double vxh = s->vx[k] + 0.5 * dt * s->fox[k];
    double vyh = s->vy[k] + 0.5 * dt * s->foy[k];
    X += vxh * dt;
    Yp += vyh * dt;
    if (X > p->xDim)
        X -= p->xDim;
    else if (X < 0)
        X += p->xDim;
    if (Yp > p->yDim)
        Yp -= p->yDim;
    else if (Yp < 0)
        Yp += p->yDim;
    s->vx[k] = vxh + 0.5 * dt * fxv;
    s->vy[k] = vyh + 0.5 * dt * fyv;
    s->fox[k] = fxv;
    s->foy[k] = fyv;
    s->px[k] = X;
    s->py[k] = Yp;
    s->cx[k] = (int)(X / dx);
    s->cy[k] = (int)(Yp / dy);
}

int orc_compat_run(const orc_ref_params *p, const double *x0, const double *y0, const double *vx0,
                   const double *vy0, long nsteps, double *x, double *y, double *vx, double *vy,
                   double *rho, double *phi, double *ex, double *ey, int nthreads)
{
    nthreads = clamp_threads(nthreads);
    compat_state s;
    memset(&s, 0, sizeof(s));
    s.p = p;
    compat_derived(p, &s.dx, &s.dy, &s.area);
    s.np = (long)p->npx * p->npy;
    s.X = p->nx + 2;
    s.Y = p->ny + 2;
    const size_t ng = (size_t)s.X * s.Y;
    double *pool = (double *)calloc((size_t)10 * s.np + 4 * ng, sizeof(double));
    if (!pool) return -1;
    s.px = pool;
    s.py = s.px + s.np;
    s.cx = s.py + s.np;
    s.cy = s.cx + s.np;
    s.vx = s.cy + s.np;
    s.vy = s.vx + s.np;
    s.fx = s.vy + s.np;
    s.fy = s.fx + s.np;
    s.fox = s.fy + s.np;
    s.foy = s.fox + s.np;
    s.rho = s.foy + s.np;
    s.phi = s.rho + ng;
    s.efx = s.phi + ng;
    s.efy = s.efx + ng;
    /* Particle::Particle, particle.cc:21-29 */
    for (long k = 0; k < s.np; ++k) {
        s.px[k] = x0[k];
        s.py[k] = y0[k];
        s.vx[k] = vx0[k];
        s.vy[k] = vy0[k];
        s.cx[k] = (int)(s.px[k] / s.dx);
        s.cy[k] = (int)(s.py[k] / s.dy);
    }
    for (long st = 0; st < nsteps; ++st) {
        compat_charge_assignment(&s, nthreads);
        compat_poisson(&s);
        compat_efield(&s);
#pragma omp parallel for num_threads(nthreads) schedule(static)
        for (long k = 0; k < s.np; ++k) compat_force_push(&s, k);
    }
    for (long k = 0; k < s.np; ++k) {
        if (x) x[k] = s.px[k];
        if (y) y[k] = s.py[k];
        if (vx) vx[k] = s.vx[k];
        if (vy) vy[k] = s.vy[k];
    }
    for (size_t i = 0; i < ng; ++i) {
        if (rho) rho[i] = s.rho[i];
        if (phi) phi[i] = s.phi[i];
        if (ex) ex[i] = s.efx[i];
        if (ey) ey[i] = s.efy[i];
    }
    free(pool);
    return 0;
}

/* ===================================================================== */
/* Part 2: physics mode (FP64), the checker for the GPU physics path.    */
/* ===================================================================== */

static inline void cic_locate(double x, double d, int n, int *i0, double *f)
{
    double g = x / d;
    double fl = floor(g);
    int i = (int)fl;
    double fr = g - fl;
    if (fr >= 1.0) {
        fr = 0.0;
        i += 1;
    }
    i %= n;
    if (i < 0) i += n;
    *i0 = i;
    *f = fr;
}

static void phys_deposit(const orc_phys_cfg *c, const orc_species *sp, double *rho, int nthreads)
{
    const int nx = c->nx, ny = c->ny;
    const double dx = c->Lx / nx, dy = c->Ly / ny, inv_area = 1.0 / (dx * dy);
    const size_t ng = (size_t)nx * ny;
    double *priv = (double *)calloc((size_t)nthreads * ng, sizeof(double));
    for (int s = 0; s < c->nspecies; ++s) {
        const orc_species *S = &sp[s];
        const double qa = S->q * inv_area;
#pragma omp parallel num_threads(nthreads)
        {
            int t = 0;
#ifdef _OPENMP
            t = omp_get_thread_num();
#endif
            double *r = priv + (size_t)t * ng;
#pragma omp for schedule(static)
            for (long k = 0; k < S->n; ++k) {
                int ix, iy;
                double fx, fy;
                cic_locate(S->x[k], dx, nx, &ix, &fx);
                cic_locate(S->y[k], dy, ny, &iy, &fy);
                int ix1 = (ix + 1) % nx, iy1 = (iy + 1) % ny;
                r[(size_t)iy * nx + ix] += qa * (1.0 - fx) * (1.0 - fy);
                r[(size_t)iy * nx + ix1] += qa * fx * (1.0 - fy);
                r[(size_t)iy1 * nx + ix] += qa * (1.0 - fx) * fy;
                r[(size_t)iy1 * nx + ix1] += qa * fx * fy;
            }
        }
    }
    memset(rho, 0, sizeof(double) * ng);
    for (int t = 0; t < nthreads; ++t)
        for (size_t i = 0; i < ng; ++i) rho[i] += priv[(size_t)t * ng + i];
    free(priv);
    /* immobile neutralising background: remove the mean */
    double mean = 0.0;
    for (size_t i = 0; i < ng; ++i) mean += rho[i];
    mean /= (double)ng;
    for (size_t i = 0; i < ng; ++i) rho[i] -= mean;
}

/* spectral Poisson: phi^ = rho^/(eps0 k^2), E^ = -i k phi^, Nyquist
 * components of the derivative set to zero, zero mode removed. */
static double phys_solve(const orc_phys_cfg *c, const double *rho, double *phi, double *ex,
                         double *ey)
{
    const int nx = c->nx, ny = c->ny, nh = nx / 2 + 1;
    const double dx = c->Lx / nx, dy = c->Ly / ny;
    const size_t ng = (size_t)nx * ny, nk = (size_t)ny * nh;
    double *rh = (double *)malloc(sizeof(double) * 2 * nk);
    double *ph = (double *)malloc(sizeof(double) * 2 * nk);
    double *exh = (double *)malloc(sizeof(double) * 2 * nk);
    double *eyh = (double *)malloc(sizeof(double) * 2 * nk);
    orc_fft2d_r2c(ny, nx, rho, rh);
    for (int my = 0; my < ny; ++my) {
        int sy = (my <= ny / 2) ? my : my - ny;
        double ky = 2.0 * M_PI * sy / c->Ly;
        for (int mx = 0; mx < nh; ++mx) {
            double kx = 2.0 * M_PI * mx / c->Lx;
            size_t q = (size_t)my * nh + mx;
            double k2 = kx * kx + ky * ky;
            double a = 0.0, b = 0.0;
            if (mx != 0 || my != 0) {
                a = rh[2 * q] / (c->eps0 * k2);
                b = rh[2 * q + 1] / (c->eps0 * k2);
            }
            ph[2 * q] = a;
            ph[2 * q + 1] = b;
            double kxe = ((nx % 2 == 0) && mx == nx / 2) ? 0.0 : kx;
            double kye = ((ny % 2 == 0) && my == ny / 2) ? 0.0 : ky;
            /* -i k (a + i b) = k b - i k a */
            exh[2 * q] = kxe * b;
            exh[2 * q + 1] = -kxe * a;
            eyh[2 * q] = kye * b;
            eyh[2 * q + 1] = -kye * a;
        }
    }
    double *tmp = (double *)malloc(sizeof(double) * ng);
    const double inv_n = 1.0 / (double)ng;
    double fe = 0.0;
    orc_fft2d_c2r(ny, nx, exh, tmp);
    for (size_t i = 0; i < ng; ++i) {
        tmp[i] *= inv_n;
        fe += tmp[i] * tmp[i];
        if (ex) ex[i] = tmp[i];
    }
    orc_fft2d_c2r(ny, nx, eyh, tmp);
    for (size_t i = 0; i < ng; ++i) {
        tmp[i] *= inv_n;
        fe += tmp[i] * tmp[i];
        if (ey) ey[i] = tmp[i];
    }
    if (phi) {
        orc_fft2d_c2r(ny, nx, ph, tmp);
        for (size_t i = 0; i < ng; ++i) phi[i] = tmp[i] * inv_n;
    }
    free(tmp);
    free(rh);
    free(ph);
    free(exh);
    free(eyh);
    return 0.5 * c->eps0 * fe * dx * dy;
}

double orc_phys_fields(const orc_phys_cfg *c, const orc_species *sp, double *rho, double *phi,
                       double *ex, double *ey, int nthreads)
{
    nthreads = clamp_threads(nthreads);
    const size_t ng = (size_t)c->nx * c->ny;
    double *r = rho ? rho : (double *)malloc(sizeof(double) * ng);
    phys_deposit(c, sp, r, nthreads);
    double fe = phys_solve(c, r, phi, ex, ey);
    if (!rho) free(r);
    return fe;
}

static void phys_push(const orc_phys_cfg *c, orc_species *sp, const double *ex, const double *ey,
                      double dt_v, double dt_x, double *ke, double *px, double *py, int nthreads)
{
    const int nx = c->nx, ny = c->ny;
    const double dx = c->Lx / nx, dy = c->Ly / ny;
    double KE = 0.0, PX = 0.0, PY = 0.0;
    for (int s = 0; s < c->nspecies; ++s) {
        orc_species *S = &sp[s];
        const double qm = S->q / S->m, m = S->m;
        double ke_s = 0.0, px_s = 0.0, py_s = 0.0;
#pragma omp parallel for num_threads(nthreads) schedule(static) reduction(+ : ke_s, px_s, py_s)
        for (long k = 0; k < S->n; ++k) {
            int ix, iy;
            double fx, fy;
            cic_locate(S->x[k], dx, nx, &ix, &fx);
            cic_locate(S->y[k], dy, ny, &iy, &fy);
            int ix1 = (ix + 1) % nx, iy1 = (iy + 1) % ny;
            size_t n00 = (size_t)iy * nx + ix, n10 = (size_t)iy * nx + ix1;
            size_t n01 = (size_t)iy1 * nx + ix, n11 = (size_t)iy1 * nx + ix1;
            double w00 = (1.0 - fx) * (1.0 - fy), w10 = fx * (1.0 - fy);
            double w01 = (1.0 - fx) * fy, w11 = fx * fy;
            double Ex = w00 * ex[n00] + w10 * ex[n10] + w01 * ex[n01] + w11 * ex[n11];
            double Ey = w00 * ey[n00] + w10 * ey[n10] + w01 * ey[n01] + w11 * ey[n11];
            double vx0 = S->vx[k], vy0 = S->vy[k];
            double vx1 = vx0 + qm * Ex * dt_v, vy1 = vy0 + qm * Ey * dt_v;
            ke_s += 0.25 * m * (vx0 * vx0 + vy0 * vy0 + vx1 * vx1 + vy1 * vy1);
            px_s += 0.5 * m * (vx0 + vx1);
            py_s += 0.5 * m * (vy0 + vy1);
            S->vx[k] = vx1;
            S->vy[k] = vy1;
            if (dt_x != 0.0) {
                double x = S->x[k] + vx1 * dt_x, y = S->y[k] + vy1 * dt_x;
                x -= c->Lx * floor(x / c->Lx);
                y -= c->Ly * floor(y / c->Ly);
                if (x >= c->Lx) x -= c->Lx;
                if (y >= c->Ly) y -= c->Ly;
                if (x < 0.0) x = 0.0;
                if (y < 0.0) y = 0.0;
                S->x[k] = x;
                S->y[k] = y;
            }
        }
        KE += ke_s;
        PX += px_s;
        PY += py_s;
    }
    if (ke) *ke = KE;
    if (px) *px = PX;
    if (py) *py = PY;
}

void orc_phys_prime(const orc_phys_cfg *c, orc_species *sp, int nthreads)
{
    nthreads = clamp_threads(nthreads);
    const size_t ng = (size_t)c->nx * c->ny;
    double *ex = (double *)malloc(sizeof(double) * ng), *ey = (double *)malloc(sizeof(double) * ng);
    orc_phys_fields(c, sp, NULL, NULL, ex, ey, nthreads);
    phys_push(c, sp, ex, ey, -0.5 * c->dt, 0.0, NULL, NULL, NULL, nthreads);
    free(ex);
    free(ey);
}

int orc_phys_run(const orc_phys_cfg *c, orc_species *sp, long nsteps, double *fe, double *ke,
                 double *px, double *py, double *rho, double *phi, double *ex, double *ey,
                 int nthreads)
{
    nthreads = clamp_threads(nthreads);
    const size_t ng = (size_t)c->nx * c->ny;
    double *r = (double *)malloc(sizeof(double) * ng);
    double *gx = (double *)malloc(sizeof(double) * ng), *gy = (double *)malloc(sizeof(double) * ng);
    double f = orc_phys_fields(c, sp, r, NULL, gx, gy, nthreads);
    if (fe) fe[0] = f;
    for (long st = 0; st < nsteps; ++st) {
        double k_, x_, y_;
        phys_push(c, sp, gx, gy, c->dt, c->dt, &k_, &x_, &y_, nthreads);
        if (ke) ke[st] = k_;
        if (px) px[st] = x_;
        if (py) py[st] = y_;
        f = orc_phys_fields(c, sp, r, NULL, gx, gy, nthreads);
        if (fe) fe[st + 1] = f;
    }
    if (rho) memcpy(rho, r, sizeof(double) * ng);
    if (ex) memcpy(ex, gx, sizeof(double) * ng);
    if (ey) memcpy(ey, gy, sizeof(double) * ng);
    if (phi) {
        double *tmp = (double *)malloc(sizeof(double) * ng);
        phys_solve(c, r, phi, tmp, NULL);
        free(tmp);
    }
    free(r);
    free(gx);
    free(gy);
    return 0;
}

/* ===================================================================== */
/* Part 3: the GPU's fixed-point deposit, restated exactly.              */
/* ===================================================================== */
void orc_deposit_fixed(int nx, int ny, long n, const int32_t *cell, const float *ox,
                       const float *oy, int64_t q_int, int64_t *rho)
{
    for (long k = 0; k < n; ++k) {
        int32_t c = cell[k];
        if (c < 0) continue; /* empty slot */
        int ix = c & 0xFFFF, iy = c >> 16; /* cell = cx | (cy << 16) */
        int ix1 = (ix + 1 == nx) ? 0 : ix + 1;
        int iy1 = (iy + 1 == ny) ? 0 : iy + 1;
        /* ox * 65536 is exact in binary32; rintf rounds half to even */
        uint64_t fx = (uint64_t)rintf(ox[k] * 65536.0f);
        uint64_t fy = (uint64_t)rintf(oy[k] * 65536.0f);
        uint64_t gx = 65536u - fx, gy = 65536u - fy;
        rho[(size_t)iy * nx + ix] += q_int * (int64_t)(gx * gy);
        rho[(size_t)iy * nx + ix1] += q_int * (int64_t)(fx * gy);
        rho[(size_t)iy1 * nx + ix] += q_int * (int64_t)(gx * fy);
        rho[(size_t)iy1 * nx + ix1] += q_int * (int64_t)(fx * fy);
    }
}

/* ===================================================================== */
/* Part 4: collision operators, restated from pic_collide.cu.            */
/* ===================================================================== */
#define STREAM_MCC 0x6d636321u
#define STREAM_DSMC 0x64736d63u

static double u24(uint32_t r) { return ((double)(r >> 8) + 0.5) * (1.0 / 16777216.0); }

static void philox_u4(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint64_t seed, uint32_t o[4])
{
    uint32_t c[4] = {c0, c1, c2, c3};
    uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    orc_philox4x32_10(c, k, o);
}

/* orthonormal basis perpendicular to u (Duff et al., JCGT 6(1), 2017) */
static void deflect(double ux, double uy, double uz, double c, double w, double out[3])
{
    double sgn = uz >= 0.0 ? 1.0 : -1.0;
    double a = -1.0 / (sgn + uz);
    double b = ux * uy * a;
    double e1[3] = {1.0 + sgn * ux * ux * a, sgn * b, -sgn * ux};
    double e2[3] = {b, sgn + uy * uy * a, -uy};
    double s = sqrt(fmax(0.0, 1.0 - c * c));
    double cp = cos(2.0 * M_PI * w), sp = sin(2.0 * M_PI * w);
    for (int i = 0; i < 3; ++i) out[i] = c * (i == 0 ? ux : i == 1 ? uy : uz) + s * (cp * e1[i] + sp * e2[i]);
}

static void mcc_sigmas(const orc_mcc *m, double E, double *sel, double *sexc, double *sion)
{
    int nt = m->ntab;
    double lr = log(m->e_max / m->e_min) / (nt - 1);
    int k;
    double f, e0, e1;
    if (E <= m->e_min) {
        k = 0;
        f = 0.0;
    } else if (E >= m->e_max) {
        k = nt - 2;
        f = 1.0;
    } else {
        k = (int)(log(E / m->e_min) / lr);
        if (k < 0) k = 0;
        if (k > nt - 2) k = nt - 2;
        e0 = m->e_min * exp(lr * k);
        e1 = m->e_min * exp(lr * (k + 1));
        if (E < e0 && k > 0) {
            --k;
            e1 = e0;
            e0 = m->e_min * exp(lr * k);
        }
        if (E >= e1 && k < nt - 2) {
            ++k;
            e0 = e1;
            e1 = m->e_min * exp(lr * (k + 1));
        }
        f = (E - e0) / (e1 - e0);
    }
    *sel = m->sel[k] + f * (m->sel[k + 1] - m->sel[k]);
    *sexc = m->sexc[k] + f * (m->sexc[k + 1] - m->sexc[k]);
    *sion = m->sion[k] + f * (m->sion[k + 1] - m->sion[k]);
}

/* One electron's null-collision test and collision in pass `pass`
 * (velocity in/out).  Returns the process (0 elastic, 1 excitation,
 * 2 ionisation, 3 null, -1 not a candidate); for an ionisation with ej
 * and ion non-NULL, the ejected electron's and the ion's velocities. */
static int mcc_one(const orc_mcc *m, uint32_t pid, uint64_t pass, double *pvx, double *pvy,
                   double *pvz, double ej[3], double ion[3])
{
    uint32_t r[4];
    philox_u4(pid, (uint32_t)pass, 0u, STREAM_MCC, m->seed, r);
    if (u24(r[0]) >= m->p_null) return -1;
    double vx = *pvx, vy = *pvy, vz = *pvz;
    double v2 = vx * vx + vy * vy + vz * vz;
    double v = sqrt(v2), E = m->half_me_over_e * v2;
    double sel, sexc, sion;
    mcc_sigmas(m, E, &sel, &sexc, &sion);
    if (E < m->e_exc) sexc = 0.0;
    if (E < m->e_ion) sion = 0.0;
    double nel = m->ng * sel * v, nexc = m->ng * sexc * v, nion = m->ng * sion * v;
    double R = u24(r[1]) * m->nu_max;
    double ux = v > 0 ? vx / v : 0.0, uy = v > 0 ? vy / v : 0.0, uz = v > 0 ? vz / v : 1.0;
    double d[3], vn;
    int proc;
    if (R < nel) {
        double c = 1.0 - 2.0 * u24(r[2]);
        double En = E * (1.0 - m->two_m_over_M * (1.0 - c));
        deflect(ux, uy, uz, c, u24(r[3]), d);
        vn = sqrt(En / m->half_me_over_e);
        proc = 0;
    } else if (R < nel + nexc) {
        deflect(ux, uy, uz, 1.0 - 2.0 * u24(r[2]), u24(r[3]), d);
        vn = sqrt(fmax(E - m->e_exc, 0.0) / m->half_me_over_e);
        proc = 1;
    } else if (R < nel + nexc + nion) {
        uint32_t r2[4], r3[4];
        philox_u4(pid, (uint32_t)pass, 1u, STREAM_MCC, m->seed, r2);
        double Er = fmax(E - m->e_ion, 0.0), Ej = u24(r2[0]) * Er, Es = Er - Ej;
        double dj[3];
        deflect(ux, uy, uz, 1.0 - 2.0 * u24(r[2]), u24(r[3]), d);
        deflect(ux, uy, uz, 1.0 - 2.0 * u24(r2[1]), u24(r2[2]), dj);
        vn = sqrt(Es / m->half_me_over_e);
        double vj = sqrt(Ej / m->half_me_over_e);
        if (ej && ion) {
            philox_u4(pid, (uint32_t)pass, 2u, STREAM_MCC, m->seed, r3);
            double ra = sqrt(-2.0 * log(u24(r3[0]))), rb = sqrt(-2.0 * log(u24(r3[2])));
            for (int k = 0; k < 3; ++k) ej[k] = vj * dj[k];
            ion[0] = m->vth_ion * ra * cos(2.0 * M_PI * u24(r3[1]));
            ion[1] = m->vth_ion * ra * sin(2.0 * M_PI * u24(r3[1]));
            ion[2] = m->vth_ion * rb * cos(2.0 * M_PI * u24(r3[3]));
        }
        proc = 2;
    } else {
        return 3;
    }
    *pvx = vn * d[0];
    *pvy = vn * d[1];
    *pvz = vn * d[2];
    return proc;
}

long orc_mcc_pass(const orc_mcc *m, long n, const uint32_t *pid, double *vx, double *vy,
                  double *vz, uint64_t pass, long cap_new, double *new_e, double *new_i,
                  long *parent, long counts[4])
{
    long born = 0;
    for (long i = 0; i < n; ++i) {
        double ej[3], ion[3];
        int keep = born < cap_new;
        int proc = mcc_one(m, pid[i], pass, &vx[i], &vy[i], &vz[i], keep ? ej : NULL,
                           keep ? ion : NULL);
        if (proc < 0) continue;
        counts[proc]++;
        if (proc == 2 && keep) {
            for (int k = 0; k < 3; ++k) {
                new_e[3 * born + k] = ej[k];
                new_i[3 * born + k] = ion[k];
            }
            parent[born] = i;
            born++;
        }
    }
    return born;
}

void orc_mcc_passes(const orc_mcc *m, long n, const uint32_t *pid, double *vx, double *vy,
                    double *vz, uint64_t first_pass, long npasses, long counts[4], int nthreads)
{
    long c0 = 0, c1 = 0, c2 = 0, c3 = 0;
    nthreads = clamp_threads(nthreads);
#pragma omp parallel for num_threads(nthreads) schedule(static) reduction(+ : c0, c1, c2, c3)
    for (long i = 0; i < n; ++i) {
        for (long p = 0; p < npasses; ++p) {
            switch (mcc_one(m, pid[i], first_pass + (uint64_t)p, &vx[i], &vy[i], &vz[i], NULL,
                            NULL)) {
            case 0: c0++; break;
            case 1: c1++; break;
            case 2: c2++; break;
            case 3: c3++; break;
            default: break;
            }
        }
    }
    counts[0] += c0;
    counts[1] += c1;
    counts[2] += c2;
    counts[3] += c3;
}

static void group_temps(long n, const double *vx, const double *vy, const double *vz, double mass,
                        double *te, double *to)
{
    double s[2][3] = {{0}}, q[2] = {0}, c[2] = {0};
    for (long i = 0; i < n; ++i) {
        int g = (int)(i & 1);
        s[g][0] += vx[i];
        s[g][1] += vy[i];
        s[g][2] += vz[i];
        q[g] += vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i];
        c[g] += 1.0;
    }
    const double kB = 1.380649e-23;
    for (int g = 0; g < 2; ++g) {
        double m2 = 0.0;
        for (int k = 0; k < 3; ++k) m2 += (s[g][k] / c[g]) * (s[g][k] / c[g]);
        double T = mass * (q[g] / c[g] - m2) / (3.0 * kB);
        if (g == 0 && te) *te = T;
        if (g == 1 && to) *to = T;
    }
}

void orc_dsmc_run(const orc_dsmc *d, long n, double *x, double *y, double *vx, double *vy,
                  double *vz, double *sgmax, long nsteps, uint64_t first_pass, double *T_even,
                  double *T_odd, long counts[2])
{
    const int nx = d->nx, ny = d->ny;
    const long nc = (long)nx * ny;
    const double dx = d->Lx / nx, dy = d->Ly / ny;
    long *cnt = (long *)calloc((size_t)nc + 1, sizeof(long));
    long *idx = (long *)malloc(sizeof(long) * (size_t)(n > 0 ? n : 1));
    long *cell = (long *)malloc(sizeof(long) * (size_t)(n > 0 ? n : 1));
    for (long st = 0; st < nsteps; ++st) {
        const uint64_t pass = first_pass + (uint64_t)st;
        memset(cnt, 0, sizeof(long) * ((size_t)nc + 1));
        for (long i = 0; i < n; ++i) {
            long cx = (long)floor(x[i] / dx), cy = (long)floor(y[i] / dy);
            if (cx >= nx) cx = nx - 1;
            if (cy >= ny) cy = ny - 1;
            if (cx < 0) cx = 0;
            if (cy < 0) cy = 0;
            cell[i] = cx + cy * nx;
            cnt[cell[i] + 1]++;
        }
        for (long c = 0; c < nc; ++c) cnt[c + 1] += cnt[c];
        {
            long *pos = (long *)malloc(sizeof(long) * (size_t)nc);
            memcpy(pos, cnt, sizeof(long) * (size_t)nc);
            for (long i = 0; i < n; ++i) idx[pos[cell[i]]++] = i;
            free(pos);
        }
        for (long c = 0; c < nc; ++c) {
            long o0 = cnt[c], m = cnt[c + 1] - o0;
            if (m < 2) continue;
            double sgm = sgmax[c];
            double want = d->coef * (double)m * (double)(m - 1) * sgm;
            uint32_t r0[4];
            philox_u4((uint32_t)c, (uint32_t)pass, 0u, STREAM_DSMC, d->seed, r0);
            double fl = floor(want);
            long ncand = (long)fl + (u24(r0[0]) < want - fl ? 1 : 0);
            for (long k = 0; k < ncand; ++k) {
                uint32_t r[4], r2[4];
                philox_u4((uint32_t)c, (uint32_t)pass, (uint32_t)(2 * k + 1), STREAM_DSMC, d->seed, r);
                long a = (long)(u24(r[0]) * m);
                if (a > m - 1) a = m - 1;
                long b = (long)(u24(r[1]) * (m - 1));
                if (b > m - 2) b = m - 2;
                if (b >= a) ++b;
                long i = idx[o0 + a], j = idx[o0 + b];
                double gx = vx[i] - vx[j], gy = vy[i] - vy[j], gz = vz[i] - vz[j];
                double g = sqrt(gx * gx + gy * gy + gz * gz), sg = d->sigma * g;
                if (sg > sgm) sgm = sg;
                counts[1]++;
                if (u24(r[2]) * sgm >= sg) continue;
                philox_u4((uint32_t)c, (uint32_t)pass, (uint32_t)(2 * k + 2), STREAM_DSMC, d->seed, r2);
                double cx_ = 2.0 * u24(r[3]) - 1.0, sx = sqrt(fmax(0.0, 1.0 - cx_ * cx_));
                double ph = 2.0 * M_PI * u24(r2[0]);
                double hx = 0.5 * g * cx_, hy = 0.5 * g * sx * cos(ph), hz = 0.5 * g * sx * sin(ph);
                double mx = 0.5 * (vx[i] + vx[j]), my = 0.5 * (vy[i] + vy[j]), mz = 0.5 * (vz[i] + vz[j]);
                vx[i] = mx + hx;
                vy[i] = my + hy;
                vz[i] = mz + hz;
                vx[j] = mx - hx;
                vy[j] = my - hy;
                vz[j] = mz - hz;
                counts[0]++;
            }
            sgmax[c] = sgm;
        }
        for (long i = 0; i < n; ++i) {
            x[i] += vx[i] * d->dt;
            y[i] += vy[i] * d->dt;
            x[i] -= d->Lx * floor(x[i] / d->Lx);
            y[i] -= d->Ly * floor(y[i] / d->Ly);
            if (x[i] >= d->Lx) x[i] -= d->Lx;
            if (y[i] >= d->Ly) y[i] -= d->Ly;
        }
        group_temps(n, vx, vy, vz, d->mass, T_even ? &T_even[st] : NULL, T_odd ? &T_odd[st] : NULL);
    }
    free(cnt);
    free(idx);
    free(cell);
}

/* ===================================================================== */
/* Part 5: adjoint of the physics step (FP64).                           */
/* ===================================================================== */
typedef struct adj_ctx {
    const orc_phys_cfg *c;
    int nx, ny;
    double dx, dy, dA;
    long n;
    double q, m;
    int nthreads;
} adj_ctx;

/* E from positions: deposit (with background) + spectral solve */
static void adj_fields(const adj_ctx *A, const double *x, const double *y, double *ex, double *ey)
{
    orc_species sp;
    sp.n = A->n;
    sp.q = A->q;
    sp.m = A->m;
    sp.x = (double *)x;
    sp.y = (double *)y;
    sp.vx = sp.vy = NULL;
    orc_phys_cfg c1 = *A->c;
    c1.nspecies = 1;
    orc_phys_fields(&c1, &sp, NULL, NULL, ex, ey, A->nthreads);
}

typedef struct cicw {
    int i00, i10, i01, i11;
    double fx, fy;
} cicw;

static inline cicw adj_locate(const adj_ctx *A, double x, double y)
{
    cicw w;
    int ix, iy;
    cic_locate(x, A->dx, A->nx, &ix, &w.fx);
    cic_locate(y, A->dy, A->ny, &iy, &w.fy);
    int ix1 = (ix + 1) % A->nx, iy1 = (iy + 1) % A->ny;
    w.i00 = iy * A->nx + ix;
    w.i10 = iy * A->nx + ix1;
    w.i01 = iy1 * A->nx + ix;
    w.i11 = iy1 * A->nx + ix1;
    return w;
}

/* F = sum_k w_k E_k for one particle */
static inline void adj_gather(const cicw *w, const double *ex, const double *ey, double *Fx, double *Fy)
{
    double gx = 1.0 - w->fx, gy = 1.0 - w->fy;
    *Fx = gx * gy * ex[w->i00] + w->fx * gy * ex[w->i10] + gx * w->fy * ex[w->i01] + w->fx * w->fy * ex[w->i11];
    *Fy = gx * gy * ey[w->i00] + w->fx * gy * ey[w->i10] + gx * w->fy * ey[w->i01] + w->fx * w->fy * ey[w->i11];
}

/* sum_k grad w_k * s_k  (s scalar per node), in physical units */
static inline void adj_grad_dot(const adj_ctx *A, const cicw *w, double s00, double s10, double s01,
                                double s11, double *gx, double *gy)
{
    double fx = w->fx, fy = w->fy;
    *gx = ((1.0 - fy) * (s10 - s00) + fy * (s11 - s01)) / A->dx;
    *gy = ((1.0 - fx) * (s01 - s00) + fx * (s11 - s10)) / A->dy;
}

/* psi = S^T g  with S: rho -> E (spectral, Nyquist derivative zeroed) */
static void adj_solve_T(const adj_ctx *A, const double *gxg, const double *gyg, double *psi)
{
    const int nx = A->nx, ny = A->ny, nh = nx / 2 + 1;
    const size_t nk = (size_t)ny * nh, ng = (size_t)nx * ny;
    double *ax = (double *)malloc(sizeof(double) * 2 * nk), *ay = (double *)malloc(sizeof(double) * 2 * nk);
    double *ph = (double *)malloc(sizeof(double) * 2 * nk);
    orc_fft2d_r2c(ny, nx, gxg, ax);
    orc_fft2d_r2c(ny, nx, gyg, ay);
    for (int my = 0; my < ny; ++my) {
        int sy = (my <= ny / 2) ? my : my - ny;
        double ky = 2.0 * M_PI * sy / A->c->Ly;
        for (int mx = 0; mx < nh; ++mx) {
            double kx = 2.0 * M_PI * mx / A->c->Lx;
            size_t qq = (size_t)my * nh + mx;
            double k2 = kx * kx + ky * ky;
            double kxe = ((nx % 2 == 0) && mx == nx / 2) ? 0.0 : kx;
            double kye = ((ny % 2 == 0) && my == ny / 2) ? 0.0 : ky;
            double hr = kxe * ax[2 * qq] + kye * ay[2 * qq];
            double hi = kxe * ax[2 * qq + 1] + kye * ay[2 * qq + 1];
            double inv = (mx == 0 && my == 0) ? 0.0 : 1.0 / (A->c->eps0 * k2);
            /* i (hr + i hi) = -hi + i hr */
            ph[2 * qq] = -hi * inv;
            ph[2 * qq + 1] = hr * inv;
        }
    }
    orc_fft2d_c2r(ny, nx, ph, psi);
    for (size_t i = 0; i < ng; ++i) psi[i] /= (double)ng;
    free(ax);
    free(ay);
    free(ph);
}

/* a_x += (q/dA) sum_m psi_m grad w_m(x) for every particle */
static void adj_gather_psi(const adj_ctx *A, const double *x, const double *y, const double *psi,
                           double *axv, double *ayv)
{
    const double s = A->q / A->dA;
#pragma omp parallel for num_threads(A->nthreads) schedule(static)
    for (long i = 0; i < A->n; ++i) {
        cicw w = adj_locate(A, x[i], y[i]);
        double gx, gy;
        adj_grad_dot(A, &w, psi[w.i00], psi[w.i10], psi[w.i01], psi[w.i11], &gx, &gy);
        axv[i] += s * gx;
        ayv[i] += s * gy;
    }
}

/* kick adjoint with coefficient C (= dt q/m, or -dt/2 q/m for the priming) */
static void adj_kick(const adj_ctx *A, const double *x, const double *y, const double *ex,
                     const double *ey, const double *avx, const double *avy, double C, double *axv,
                     double *ayv)
{
    const size_t ng = (size_t)A->nx * A->ny;
    double *g = (double *)calloc(2 * ng, sizeof(double));
    double *psi = (double *)malloc(sizeof(double) * ng);
    for (long i = 0; i < A->n; ++i) {  /* serial scatter: deterministic */
        cicw w = adj_locate(A, x[i], y[i]);
        double mx = C * avx[i], my = C * avy[i];
        double gx_ = 1.0 - w.fx, gy_ = 1.0 - w.fy;
        double w00 = gx_ * gy_, w10 = w.fx * gy_, w01 = gx_ * w.fy, w11 = w.fx * w.fy;
        g[w.i00] += w00 * mx; g[ng + w.i00] += w00 * my;
        g[w.i10] += w10 * mx; g[ng + w.i10] += w10 * my;
        g[w.i01] += w01 * mx; g[ng + w.i01] += w01 * my;
        g[w.i11] += w11 * mx; g[ng + w.i11] += w11 * my;
        /* local term: sum_k grad w_k (E_k . mu) */
        double s00 = ex[w.i00] * mx + ey[w.i00] * my, s10 = ex[w.i10] * mx + ey[w.i10] * my;
        double s01 = ex[w.i01] * mx + ey[w.i01] * my, s11 = ex[w.i11] * mx + ey[w.i11] * my;
        double lx, ly;
        adj_grad_dot(A, &w, s00, s10, s01, s11, &lx, &ly);
        axv[i] += lx;
        ayv[i] += ly;
    }
    adj_solve_T(A, g, g + ng, psi);
    adj_gather_psi(A, x, y, psi, axv, ayv);
    free(g);
    free(psi);
}

static void adj_forward(const adj_ctx *A, const double *x0, const double *y0, const double *vx0,
                        const double *vy0, long nsteps, double *X, double *Y, double *J)
{
    /* X, Y: (nsteps+1) * n positions; returns J */
    const size_t ng = (size_t)A->nx * A->ny;
    const long n = A->n;
    const double dt = A->c->dt, qm = A->q / A->m;
    double *vx = (double *)malloc(sizeof(double) * n), *vy = (double *)malloc(sizeof(double) * n);
    double *ex = (double *)malloc(sizeof(double) * ng), *ey = (double *)malloc(sizeof(double) * ng);
    memcpy(X, x0, sizeof(double) * n);
    memcpy(Y, y0, sizeof(double) * n);
    memcpy(vx, vx0, sizeof(double) * n);
    memcpy(vy, vy0, sizeof(double) * n);
    adj_fields(A, X, Y, ex, ey);
    for (long i = 0; i < n; ++i) { /* priming: v(-1/2) = v0 - (q/m) F(x0) dt/2 */
        cicw w = adj_locate(A, X[i], Y[i]);
        double Fx, Fy;
        adj_gather(&w, ex, ey, &Fx, &Fy);
        vx[i] -= 0.5 * dt * qm * Fx;
        vy[i] -= 0.5 * dt * qm * Fy;
    }
    for (long st = 0; st < nsteps; ++st) {
        const double *xs = X + (size_t)st * n, *ys = Y + (size_t)st * n;
        double *xn = X + (size_t)(st + 1) * n, *yn = Y + (size_t)(st + 1) * n;
        if (st > 0) adj_fields(A, xs, ys, ex, ey);
#pragma omp parallel for num_threads(A->nthreads) schedule(static)
        for (long i = 0; i < n; ++i) {
            cicw w = adj_locate(A, xs[i], ys[i]);
            double Fx, Fy;
            adj_gather(&w, ex, ey, &Fx, &Fy);
            vx[i] += dt * qm * Fx;
            vy[i] += dt * qm * Fy;
            double x = xs[i] + dt * vx[i], y = ys[i] + dt * vy[i];
            x -= A->c->Lx * floor(x / A->c->Lx);
            y -= A->c->Ly * floor(y / A->c->Ly);
            if (x >= A->c->Lx) x -= A->c->Lx;
            if (y >= A->c->Ly) y -= A->c->Ly;
            xn[i] = x;
            yn[i] = y;
        }
    }
    adj_fields(A, X + (size_t)nsteps * n, Y + (size_t)nsteps * n, ex, ey);
    double fe = 0.0;
    for (size_t i = 0; i < ng; ++i) fe += ex[i] * ex[i] + ey[i] * ey[i];
    *J = 0.5 * A->c->eps0 * fe * A->dA;
    free(vx);
    free(vy);
    free(ex);
    free(ey);
}

static adj_ctx make_ctx(const orc_phys_cfg *c, long n, double q, double m, int nthreads)
{
    adj_ctx A;
    A.c = c;
    A.nx = c->nx;
    A.ny = c->ny;
    A.dx = c->Lx / c->nx;
    A.dy = c->Ly / c->ny;
    A.dA = A.dx * A.dy;
    A.n = n;
    A.q = q;
    A.m = m;
    A.nthreads = clamp_threads(nthreads);
    return A;
}

double orc_forward_J(const orc_phys_cfg *c, long n, double q, double m, const double *x0,
                     const double *y0, const double *vx0, const double *vy0, long nsteps,
                     int nthreads)
{
    adj_ctx A = make_ctx(c, n, q, m, nthreads);
    double *X = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    double *Y = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    /* forward without keeping the trajectory: reuse two position slots */
    const size_t ng = (size_t)A.nx * A.ny;
    const double dt = c->dt, qm = q / m;
    double *vx = (double *)malloc(sizeof(double) * n), *vy = (double *)malloc(sizeof(double) * n);
    double *ex = (double *)malloc(sizeof(double) * ng), *ey = (double *)malloc(sizeof(double) * ng);
    memcpy(X, x0, sizeof(double) * n);
    memcpy(Y, y0, sizeof(double) * n);
    memcpy(vx, vx0, sizeof(double) * n);
    memcpy(vy, vy0, sizeof(double) * n);
    adj_fields(&A, X, Y, ex, ey);
    for (long i = 0; i < n; ++i) {
        cicw w = adj_locate(&A, X[i], Y[i]);
        double Fx, Fy;
        adj_gather(&w, ex, ey, &Fx, &Fy);
        vx[i] -= 0.5 * dt * qm * Fx;
        vy[i] -= 0.5 * dt * qm * Fy;
    }
    for (long st = 0; st < nsteps; ++st) {
        if (st > 0) adj_fields(&A, X, Y, ex, ey);
#pragma omp parallel for num_threads(A.nthreads) schedule(static)
        for (long i = 0; i < n; ++i) {
            cicw w = adj_locate(&A, X[i], Y[i]);
            double Fx, Fy;
            adj_gather(&w, ex, ey, &Fx, &Fy);
            vx[i] += dt * qm * Fx;
            vy[i] += dt * qm * Fy;
            double x = X[i] + dt * vx[i], y = Y[i] + dt * vy[i];
            x -= c->Lx * floor(x / c->Lx);
            y -= c->Ly * floor(y / c->Ly);
            if (x >= c->Lx) x -= c->Lx;
            if (y >= c->Ly) y -= c->Ly;
            X[i] = x;
            Y[i] = y;
        }
    }
    adj_fields(&A, X, Y, ex, ey);
    double fe = 0.0;
    for (size_t i = 0; i < ng; ++i) fe += ex[i] * ex[i] + ey[i] * ey[i];
    free(X);
    free(Y);
    free(vx);
    free(vy);
    free(ex);
    free(ey);
    return 0.5 * c->eps0 * fe * A.dA;
}

double orc_adjoint(const orc_phys_cfg *c, long n, double q, double m, const double *x0,
                   const double *y0, const double *vx0, const double *vy0, long nsteps,
                   double *gx0, double *gy0, double *gvx0, double *gvy0, int nthreads)
{
    adj_ctx A = make_ctx(c, n, q, m, nthreads);
    const size_t ng = (size_t)A.nx * A.ny;
    double *X = (double *)malloc(sizeof(double) * (size_t)(nsteps + 1) * n);
    double *Y = (double *)malloc(sizeof(double) * (size_t)(nsteps + 1) * n);
    double J = 0.0;
    adj_forward(&A, x0, y0, vx0, vy0, nsteps, X, Y, &J);
    double *ax = (double *)calloc(n, sizeof(double)), *ay = (double *)calloc(n, sizeof(double));
    double *avx = (double *)calloc(n, sizeof(double)), *avy = (double *)calloc(n, sizeof(double));
    double *ex = (double *)malloc(sizeof(double) * ng), *ey = (double *)malloc(sizeof(double) * ng);
    double *g = (double *)malloc(sizeof(double) * 2 * ng), *psi = (double *)malloc(sizeof(double) * ng);
    const double dt = c->dt, qm = q / m;
    /* terminal: a_x = grad W(x_N), W = 1/2 eps0 dA sum |E|^2 */
    {
        const double *xN = X + (size_t)nsteps * n, *yN = Y + (size_t)nsteps * n;
        adj_fields(&A, xN, yN, ex, ey);
        for (size_t i = 0; i < ng; ++i) {
            g[i] = c->eps0 * A.dA * ex[i];
            g[ng + i] = c->eps0 * A.dA * ey[i];
        }
        adj_solve_T(&A, g, g + ng, psi);
        adj_gather_psi(&A, xN, yN, psi, ax, ay);
    }
    for (long st = nsteps - 1; st >= 0; --st) {
        const double *xs = X + (size_t)st * n, *ys = Y + (size_t)st * n;
        for (long i = 0; i < n; ++i) {  /* drift adjoint */
            avx[i] += dt * ax[i];
            avy[i] += dt * ay[i];
        }
        adj_fields(&A, xs, ys, ex, ey);
        adj_kick(&A, xs, ys, ex, ey, avx, avy, dt * qm, ax, ay);
    }
    /* priming v(-1/2) = v0 - (q/m) F(x0) dt/2 */
    adj_fields(&A, X, Y, ex, ey);
    adj_kick(&A, X, Y, ex, ey, avx, avy, -0.5 * dt * qm, ax, ay);
    for (long i = 0; i < n; ++i) {
        if (gx0) gx0[i] = ax[i];
        if (gy0) gy0[i] = ay[i];
        if (gvx0) gvx0[i] = avx[i];
        if (gvy0) gvy0[i] = avy[i];
    }
    free(X);
    free(Y);
    free(ax);
    free(ay);
    free(avx);
    free(avy);
    free(ex);
    free(ey);
    free(g);
    free(psi);
    return J;
}
