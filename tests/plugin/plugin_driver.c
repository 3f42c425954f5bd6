/* Driver of the REBOUND-plugin test (TEST INFRASTRUCTURE ONLY).
 *
 * Runs the same Plummer sphere through REBOUND's built-in leapfrog and through
 * the plugin's "gpu_leapfrog", with REBOUND's own reb_simulation_integrate /
 * reb_simulation_steps loops, and prints one line per phase:
 *   STATUS <phase> <built-in status> <plugin status>
 *   DIFF <phase> <max |plugin - built-in| over x..vz> <t difference>
 * Phases: integrate with a shortened last step, a modified particle, an added
 * particle, a removed particle, plain steps, a periodic boundary held by the
 * plugin, and the boundary handed back when the built-in integrator is
 * selected again.  With the argument "whfast" it runs the outer solar system
 * through REBOUND's WHFast and the plugin's "gpu_whfast" instead (one custom
 * integrator per process: see rgpu_rebound.h).  A failing GPU library ends the
 * run with
 *   ERROR <message REBOUND stored>
 * (the no-GPU path of the real library). */
#include <math.h>
#include <stdio.h>
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#include <stdlib.h>
#include <string.h>

#include "rgpu_rebound.h"

static struct reb_simulation* make(int n) {
    struct reb_simulation* r = reb_simulation_create();
    r->rand_seed = 7;
    reb_simulation_add_plummer(r, n, 1., 1.);
    r->softening = 0.01;
    r->dt = 1e-3;
    r->save_messages = 1;
    return r;
}

static double maxdiff(struct reb_simulation* a, struct reb_simulation* b) {
    if (a->N != b->N) return INFINITY;
    double m = 0.;
    for (size_t i = 0; i < a->N; i++) {
        const double* pa = &a->particles[i].x;
        const double* pb = &b->particles[i].x;
        for (int k = 0; k < 6; k++) {
            const double d = fabs(pa[k] - pb[k]);
            if (!(d <= m)) m = d;
        }
    }
    return m;
}

static int report(const char* phase, struct reb_simulation* a, struct reb_simulation* b, int sa, int sb) {
    printf("STATUS %s %d %d\n", phase, sa, sb);
    if (sb == REB_STATUS_GENERIC_ERROR) {
        for (int i = 0; b->messages && i < 10; i++)
            if (b->messages[i] && b->messages[i][0] == 'e') printf("ERROR %s\n", b->messages[i] + 1);
        return 1;
    }
    printf("DIFF %s %.17g %.17g\n", phase, maxdiff(a, b), b->t - a->t);
    return 0;
}

/* WHFast (safe_mode 1, Jacobi) on the outer solar system: built-in against the plugin. */
static int run_whfast(void) {
    rgpu_rebound_register(RGPU_INTEGRATOR_WHFAST, "gpu_whfast");
    struct reb_simulation* a = reb_simulation_create();
    struct reb_simulation* b = reb_simulation_create();
    reb_simulation_add_fmt(a, "outer solar system");
    reb_simulation_add_fmt(b, "outer solar system");
    a->dt = b->dt = 0.005 * 12. * 2. * M_PI;
    a->save_messages = b->save_messages = 1;
    reb_simulation_set_integrator(a, "whfast");
    struct rgpu_rebound_state* st = reb_simulation_set_integrator(b, "gpu_whfast");
    if (!st || st->scheme != RGPU_INTEGRATOR_WHFAST || st->safe_mode != 1) {
        printf("ERROR set_integrator did not return the plugin state\n");
        return 0;
    }
    int sa = reb_simulation_integrate(a, 100.), sb = reb_simulation_integrate(b, 100.);
    if (report("whfast_integrate", a, b, sa, sb)) return 0;
    a->particles[2].vx *= 1.0001; a->did_modify_particles = 1;
    b->particles[2].vx *= 1.0001; b->did_modify_particles = 1;
    sa = reb_simulation_integrate(a, 250.); sb = reb_simulation_integrate(b, 250.);
    if (report("whfast_modified", a, b, sa, sb)) return 0;
    printf("ENERGY %.17g %.17g\n", reb_simulation_energy(a), reb_simulation_energy(b));
    reb_simulation_free(a);
    reb_simulation_free(b);
    printf("DONE\n");
    return 0;
}

int main(int argc, char** argv) {
    if (argc > 1 && strcmp(argv[1], "whfast") == 0) return run_whfast();
    rgpu_rebound_register(RGPU_INTEGRATOR_LEAPFROG, "gpu_leapfrog");
    struct reb_simulation* a = make(64);
    struct reb_simulation* b = make(64);
    reb_simulation_set_integrator(a, "leapfrog");
    struct rgpu_rebound_state* st = reb_simulation_set_integrator(b, "gpu_leapfrog");
    if (!st || st->scheme != RGPU_INTEGRATOR_LEAPFROG) {
        printf("ERROR set_integrator did not return the plugin state\n");
        return 0;
    }
    int sa = reb_simulation_integrate(a, 0.0105), sb = reb_simulation_integrate(b, 0.0105);
    if (report("integrate", a, b, sa, sb)) return 0;

    a->particles[3].vx += 1e-3; a->did_modify_particles = 1;
    b->particles[3].vx += 1e-3; b->did_modify_particles = 1;
    sa = reb_simulation_integrate(a, 0.02); sb = reb_simulation_integrate(b, 0.02);
    if (report("modified", a, b, sa, sb)) return 0;

    struct reb_particle q = {0};
    q.m = 1e-3; q.x = 0.5; q.y = 0.1; q.z = -0.2; q.vy = 0.3;
    reb_simulation_add(a, q);
    reb_simulation_add(b, q);
    sa = reb_simulation_integrate(a, 0.03); sb = reb_simulation_integrate(b, 0.03);
    if (report("added", a, b, sa, sb)) return 0;

    reb_simulation_remove_particle(a, 5);
    reb_simulation_remove_particle(b, 5);
    sa = reb_simulation_integrate(a, 0.04); sb = reb_simulation_integrate(b, 0.04);
    if (report("removed", a, b, sa, sb)) return 0;

    reb_simulation_steps(a, 3);
    reb_simulation_steps(b, 3);
    if (report("steps", a, b, a->status, b->status)) return 0;

    a->root_size = 40.; b->root_size = 40.;
    a->boundary = REB_BOUNDARY_PERIODIC;
    b->boundary = REB_BOUNDARY_PERIODIC;
    sa = reb_simulation_integrate(a, 0.06); sb = reb_simulation_integrate(b, 0.06);
    if (report("periodic", a, b, sa, sb)) return 0;
    printf("HELD %d %d\n", (int)b->boundary, rgpu_rebound_boundary(b));

    reb_simulation_set_integrator(b, "leapfrog");
    printf("RETURNED %d\n", (int)b->boundary);
    sa = reb_simulation_integrate(a, 0.07); sb = reb_simulation_integrate(b, 0.07);
    if (report("builtin_again", a, b, sa, sb)) return 0;
    reb_simulation_free(a);
    reb_simulation_free(b);
    printf("DONE\n");
    return 0;
}
