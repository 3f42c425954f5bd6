/* Test double of librebound_gb300's C ABI for the CPU test of the REBOUND plugin.
 *
 * TEST INFRASTRUCTURE ONLY.  It implements the entry points that
 * rebound_gb300/plugin/rgpu_rebound.c calls, backed by a private REBOUND
 * simulation that runs the reference's own built-in integrator (leapfrog, SEI
 * or WHFast) with the reference's gravity.  A plugin that moves configuration,
 * time and particles across the boundary correctly therefore reproduces the
 * built-in integrator bit for bit, which is what the test checks.  Built only by
 * tests/test_rebound_plugin.py, against the reference's header and library. */
#include <stdlib.h>
#include <string.h>

#include "rebound.h"
#include "rebound_gb300.h"

struct rgpu_sim {
    struct reb_simulation* r;
    rgpu_config cfg;
    double (*eps_fn)(void*, double);
    void* eps_user;
    int integrator_set;           /* the private simulation starts with REBOUND's default (IAS15) */
};

static int64_t g_steps = 0;

void rgpu_config_default(rgpu_config* c) {
    memset(c, 0, sizeof(*c));
    c->G = 1.0;
    c->OMEGA = 1.0;
    c->OMEGAZ = -1.0;
    c->root_size = -1.0;
    c->opening_angle2 = 0.25;
    c->coefficient_of_restitution = 1.0;
    c->N_active = -1;
    c->N_root_x = c->N_root_y = c->N_root_z = 1;
    c->gravity = RGPU_GRAVITY_BASIC;
    c->whfast_safe_mode = 1;
    c->exact_finish_time = 1;
    c->status = -1;
}

int rgpu_sim_create(rgpu_sim** out) {
    rgpu_sim* s = calloc(1, sizeof(rgpu_sim));
    if (!s) return RGPU_ERR_NOMEM;
    s->r = reb_simulation_create();
    rgpu_config_default(&s->cfg);
    *out = s;
    return RGPU_OK;
}

void rgpu_sim_free(rgpu_sim* s) {
    if (!s) return;
    reb_simulation_free(s->r);
    free(s);
}

const char* rgpu_sim_last_error(const rgpu_sim* s) { (void)s; return "fake"; }

static double eps_trampoline(const struct reb_simulation* const r, double v) {
    rgpu_sim* s = (rgpu_sim*)r->extras;
    return s->eps_fn(s->eps_user, v);
}

int rgpu_sim_configure(rgpu_sim* s, const rgpu_config* c) {
    struct reb_simulation* r = s->r;
    const int changed = c->integrator != s->cfg.integrator || !s->integrator_set;
    s->cfg = *c;
    if (changed) {
        const char* name = c->integrator == RGPU_INTEGRATOR_SEI ? "sei"
                           : c->integrator == RGPU_INTEGRATOR_WHFAST ? "whfast" : "leapfrog";
        reb_simulation_set_integrator(r, name);
        s->integrator_set = 1;
    }
    r->G = c->G; r->softening = c->softening; r->dt = c->dt; r->t = c->t;
    r->OMEGA = c->OMEGA; r->OMEGAZ = c->OMEGAZ; r->opening_angle2 = c->opening_angle2;
    r->N_active = c->N_active < 0 ? SIZE_MAX : (size_t)c->N_active;
    r->testparticle_type = c->testparticle_type;
    r->gravity = c->gravity;
    r->boundary = c->boundary;
    r->collision = c->collision;
    r->rand_seed = c->rand_seed;
    r->collisions_log_n = c->collisions_log_n;
    r->collisions_plog = c->collisions_plog;
    r->minimum_collision_velocity = c->minimum_collision_velocity;
    r->collision_resolve = c->collision_resolve == RGPU_RESOLVE_HARDSPHERE ? reb_collision_resolve_hardsphere
                                                                          : reb_collision_resolve_halt;
    r->extras = s;
    r->coefficient_of_restitution = s->eps_fn ? eps_trampoline : NULL;
    if (c->integrator == RGPU_INTEGRATOR_WHFAST) {
        struct reb_integrator_whfast_state* w = (struct reb_integrator_whfast_state*)r->integrator.state;
        w->safe_mode = (unsigned)c->whfast_safe_mode;
        w->corrector = (unsigned)c->whfast_corrector;
        w->corrector2 = (unsigned)c->whfast_corrector2;
        w->kernel = c->whfast_kernel;
        w->coordinates = c->whfast_coordinates;
        w->keep_unsynchronized = (unsigned)c->whfast_keep_unsynchronized;
    } else if (c->integrator == RGPU_INTEGRATOR_LEAPFROG) {
        ((struct reb_integrator_leapfrog_state*)r->integrator.state)->order = c->leapfrog_order ? (unsigned)c->leapfrog_order : 2u;
    }
    r->root_size = c->root_size;
    r->N_root_x = (size_t)c->N_root_x; r->N_root_y = (size_t)c->N_root_y; r->N_root_z = (size_t)c->N_root_z;
    r->N_ghost_x = c->N_ghost_x; r->N_ghost_y = c->N_ghost_y; r->N_ghost_z = c->N_ghost_z;
    return RGPU_OK;
}

int rgpu_sim_get_config(const rgpu_sim* s, rgpu_config* c) {
    *c = s->cfg;
    return RGPU_OK;
}

int rgpu_sim_set_restitution_fn(rgpu_sim* s, double (*fn)(void*, double), void* user) {
    s->eps_fn = fn;
    s->eps_user = user;
    s->r->coefficient_of_restitution = fn ? eps_trampoline : NULL;
    return RGPU_OK;
}

int rgpu_sim_set_particles(rgpu_sim* s, const void* particles, size_t N, size_t stride) {
    struct reb_simulation* r = s->r;
    while (r->N) reb_simulation_remove_particle(r, r->N - 1);
    for (size_t i = 0; i < N; i++) {
        struct reb_particle p;
        memcpy(&p, (const char*)particles + i * stride, sizeof(p));
        p.ap = NULL;
        p.sim = NULL;
        reb_simulation_add(r, p);
    }
    r->did_modify_particles = 1;
    return RGPU_OK;
}

int rgpu_sim_get_particles(rgpu_sim* s, void* particles, size_t N, size_t stride) {
    if (N != s->r->N) return RGPU_ERR_ARG;
    for (size_t i = 0; i < N; i++) memcpy((char*)particles + i * stride, &s->r->particles[i], 11 * sizeof(double));
    return RGPU_OK;
}

size_t rgpu_sim_N(const rgpu_sim* s) { return s ? s->r->N : 0; }

int rgpu_steps(rgpu_sim* s, int64_t n) {
    struct reb_simulation* r = s->r;
    r->t = s->cfg.t;
    r->dt = s->cfg.dt;
    r->status = REB_STATUS_RUNNING;
    reb_simulation_steps(r, (size_t)n);
    g_steps += n;
    s->cfg.t = r->t;
    s->cfg.rand_seed = r->rand_seed;
    s->cfg.collisions_log_n = r->collisions_log_n;
    s->cfg.collisions_plog = r->collisions_plog;
    s->cfg.status = r->status;
    return RGPU_OK;
}

int rgpu_synchronize(rgpu_sim* s) {
    reb_simulation_synchronize(s->r);
    return RGPU_OK;
}

int64_t rgpu_launch_count(void) { return g_steps; }
