/* A caller of the C ABI in plain C (no C++, no Python): a two-stream run
 * through the step interface, then the same particles through the one-call
 * host-to-host run.  Built and run by tests/test_c_abi_demo.py; prints one
 * line "fe <field energy> charge_ok <0|1> moved <0|1>" or an error and a
 * non-zero exit status. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "pic.h"

#define CHECK(call)                                                                   \
    do {                                                                              \
        pic_status s_ = (call);                                                       \
        if (s_ != PIC_OK) {                                                           \
            fprintf(stderr, "%s: %s (%s)\n", #call, pic_status_string(s_), pic_last_error()); \
            return 1;                                                                 \
        }                                                                             \
    } while (0)

int main(void)
{
    const int nx = 64, ny = 64, ppc = 8;
    const long long n = (long long)nx * ny * ppc;
    const double L = 4.0 * 3.14159265358979323846, A = L * L;
    pic_config c;
    CHECK(pic_config_default(&c));
    c.nx = nx;
    c.ny = ny;
    c.Lx = L;
    c.Ly = L;
    c.dt = 0.1;
    c.eps0 = 1.0;
    c.nspecies = 1;
    c.species[0].capacity = n;
    c.species[0].q = -A / (double)n;
    c.species[0].m = A / (double)n;
    c.species[0].q_int = -1;
    c.species[0].flags = 0;
    pic_handle *h = NULL;
    CHECK(pic_create(&c, &h));

    /* step interface: init, prime, K steps, diagnostics, particles back */
    pic_init_spec sp = {0};
    sp.n = n;
    sp.vth[0] = sp.vth[1] = 0.01;
    sp.beam_v = 0.2;
    sp.pert_kind = PIC_PERT_XDISP;
    sp.pert_amp = 1e-3;
    sp.pert_mx = 1;
    sp.seed = 5;
    CHECK(pic_init_particles(h, 0, &sp));
    CHECK(pic_prime_leapfrog(h));
    CHECK(pic_step(h, 20));
    CHECK(pic_synchronize(h));
    pic_diag d;
    CHECK(pic_diagnostics(h, &d));
    double *x = malloc(n * sizeof(double)), *y = malloc(n * sizeof(double));
    double *vx = malloc(n * sizeof(double)), *vy = malloc(n * sizeof(double));
    long long got = 0;
    CHECK(pic_get_particles(h, 0, &got, x, y, vx, vy, NULL));
    if (got != n) {
        fprintf(stderr, "count %lld, expected %lld\n", got, n);
        return 1;
    }

    /* the same particles through the one-call run, outputs aliasing inputs */
    double x0 = x[0];
    CHECK(pic_run_host(h, n, x, y, vx, vy, 5, 1, x, y, vx, vy));
    int moved = fabs(x[0] - x0) > 0.0;
    CHECK(pic_destroy(h));
    printf("fe %.17g charge_ok %d moved %d\n", d.field_energy,
           d.total_charge_fixed == d.expected_charge_fixed, moved);
    free(x);
    free(y);
    free(vx);
    free(vy);
    return 0;
}
