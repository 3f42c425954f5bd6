/* REBOUND-side binding of librebound_gb300 (see rgpu_rebound.h).
 *
 * Implements the callbacks of struct reb_integrator (src/rebound.h:170-179) on
 * top of the C ABI in include/rebound_gb300.h.  The host-side order of
 * operations follows reb_simulation_step (src/simulation.c:514-603): REBOUND
 * calls `step`, then runs its boundary check and collision search on the host;
 * the device performs those itself inside rgpu_steps, so this plugin holds
 * r->boundary and r->collision for the device while it is selected. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "rgpu_rebound.h"

static void rgpu_rebound_step(struct reb_simulation* r, void* p);
static void rgpu_rebound_synchronize(struct reb_simulation* r, void* p);
static void rgpu_rebound_free(void* p);
static void rgpu_rebound_did_add_particle(struct reb_simulation* r);
static void rgpu_rebound_will_remove_particle(struct reb_simulation* r, size_t index);

static struct rgpu_rebound_state* state_new(int scheme) {
    struct rgpu_rebound_state* st = calloc(1, sizeof(struct rgpu_rebound_state));
    if (!st) return NULL;
    st->scheme = scheme;
    st->order = 2;
    st->safe_mode = 1;
    return st;
}
static void* create_leapfrog(void) { return state_new(RGPU_INTEGRATOR_LEAPFROG); }
static void* create_sei(void) { return state_new(RGPU_INTEGRATOR_SEI); }
static void* create_whfast(void) { return state_new(RGPU_INTEGRATOR_WHFAST); }

#define RGPU_REBOUND_CALLBACKS(create_fn)                                                         \
    .step = rgpu_rebound_step, .synchronize = rgpu_rebound_synchronize, .create = create_fn,      \
    .free = rgpu_rebound_free, .did_add_particle = rgpu_rebound_did_add_particle,                 \
    .will_remove_particle = rgpu_rebound_will_remove_particle, .field_descriptor_list = NULL

const struct reb_integrator rgpu_integrator_leapfrog = {
    .documentation = "Leapfrog (orders 2, 4, 6, 8) on the GPU (librebound_gb300).",
    RGPU_REBOUND_CALLBACKS(create_leapfrog)};
const struct reb_integrator rgpu_integrator_sei = {
    .documentation = "SEI for shearing sheets on the GPU (librebound_gb300).",
    RGPU_REBOUND_CALLBACKS(create_sei)};
const struct reb_integrator rgpu_integrator_whfast = {
    .documentation = "WHFast on the GPU (librebound_gb300).",
    RGPU_REBOUND_CALLBACKS(create_whfast)};

void rgpu_rebound_register(int scheme, const char* name) {
    switch (scheme) {
        case RGPU_INTEGRATOR_LEAPFROG: reb_integrator_register(rgpu_integrator_leapfrog, name); break;
        case RGPU_INTEGRATOR_SEI: reb_integrator_register(rgpu_integrator_sei, name); break;
        case RGPU_INTEGRATOR_WHFAST: reb_integrator_register(rgpu_integrator_whfast, name); break;
        default: reb_simulation_error(NULL, "rgpu_rebound_register: unknown scheme");
    }
}

static struct rgpu_rebound_state* ours(struct reb_simulation* r) {
    if (!r || r->integrator.callbacks.step != rgpu_rebound_step) return NULL;
    return (struct rgpu_rebound_state*)r->integrator.state;
}

rgpu_sim* rgpu_rebound_handle(struct reb_simulation* r) {
    struct rgpu_rebound_state* st = ours(r);
    return st ? st->sim : NULL;
}

/* Values the device uses while these integrators hold the fields. */
int rgpu_rebound_boundary(struct reb_simulation* r) {
    struct rgpu_rebound_state* st = ours(r);
    if (!st) return r ? (int)r->boundary : 0;
    return r->boundary != REB_BOUNDARY_NONE ? (int)r->boundary : st->boundary;
}
int rgpu_rebound_collision(struct reb_simulation* r) {
    struct rgpu_rebound_state* st = ours(r);
    if (!st) return r ? (int)r->collision : 0;
    return r->collision != REB_COLLISION_NONE ? (int)r->collision : st->collision;
}

/* Report a failure of the GPU library the way REBOUND's integrators do. */
static void fail(struct reb_simulation* r, struct rgpu_rebound_state* st, const char* what, int rc) {
    char msg[512];
    snprintf(msg, sizeof(msg), "rgpu: %s failed (code %d): %s", what, rc,
             st->sim ? rgpu_sim_last_error(st->sim) : "no GPU simulation handle");
    reb_simulation_error(r, msg);
    r->status = REB_STATUS_GENERIC_ERROR;
}

/* Copy the device state into r->particles if it is newer. */
static int pull_particles(struct reb_simulation* r, struct rgpu_rebound_state* st, size_t n) {
    if (!st->sim || !st->device_ahead) return 0;
    const int rc = rgpu_sim_get_particles(st->sim, r->particles, n, sizeof(struct reb_particle));
    if (rc) {
        fail(r, st, "rgpu_sim_get_particles", rc);
        return rc;
    }
    st->device_ahead = 0;
    return 0;
}

static double restitution_trampoline(void* user, double v) {
    const struct reb_simulation* r = (const struct reb_simulation*)user;
    return r->coefficient_of_restitution(r, v);
}

/* rgpu_config from the REBOUND fields this path reads (src/rebound.h:238-413). */
static int make_config(struct reb_simulation* r, struct rgpu_rebound_state* st, rgpu_config* c) {
    rgpu_config_default(c);
    c->G = r->G;
    c->softening = r->softening;
    c->dt = r->dt;
    c->t = r->t;
    c->OMEGA = r->OMEGA;
    c->OMEGAZ = r->OMEGAZ;
    c->root_size = r->root_size;
    c->opening_angle2 = r->opening_angle2;
    c->coefficient_of_restitution = 1.0;          /* src/collision.c:603: perfect bouncing without a callback */
    c->minimum_collision_velocity = r->minimum_collision_velocity;
    c->N_active = r->N_active == SIZE_MAX ? -1 : (int64_t)r->N_active;
    c->testparticle_type = r->testparticle_type;
    c->gravity_ignore_terms = (int32_t)r->gravity_ignore_terms;
    c->N_root_x = r->N_root_x; c->N_root_y = r->N_root_y; c->N_root_z = r->N_root_z;
    c->N_ghost_x = r->N_ghost_x; c->N_ghost_y = r->N_ghost_y; c->N_ghost_z = r->N_ghost_z;
    switch (r->gravity) {
        case REB_GRAVITY_NONE: c->gravity = RGPU_GRAVITY_NONE; break;
        case REB_GRAVITY_BASIC: c->gravity = RGPU_GRAVITY_BASIC; break;
        case REB_GRAVITY_COMPENSATED: c->gravity = RGPU_GRAVITY_COMPENSATED; break;
        case REB_GRAVITY_TREE: c->gravity = RGPU_GRAVITY_TREE; break;
        default:
            reb_simulation_error(r, "rgpu: gravity must be NONE, BASIC, COMPENSATED or TREE on the GPU path.");
            r->status = REB_STATUS_GENERIC_ERROR;
            return -1;
    }
    c->collision = st->collision;                  /* REBOUND's enum values are the library's */
    c->boundary = st->boundary;
    if (!r->collision_resolve || r->collision_resolve == reb_collision_resolve_halt) {
        c->collision_resolve = RGPU_RESOLVE_HALT;   /* src/collision.c:346-349: halt by default */
    } else if (r->collision_resolve == reb_collision_resolve_hardsphere) {
        c->collision_resolve = RGPU_RESOLVE_HARDSPHERE;
    } else if (st->collision == REB_COLLISION_NONE) {
        c->collision_resolve = RGPU_RESOLVE_NONE;   /* never called without a search */
    } else {
        reb_simulation_error(r, "rgpu: collision_resolve must be reb_collision_resolve_halt or "
                                "reb_collision_resolve_hardsphere on the GPU path.");
        r->status = REB_STATUS_GENERIC_ERROR;
        return -1;
    }
    c->integrator = st->scheme;
    c->whfast_safe_mode = (int32_t)st->safe_mode;
    c->rand_seed = r->rand_seed;
    c->status = 0;
    c->collisions_log_n = r->collisions_log_n;
    c->collisions_plog = r->collisions_plog;
    c->leapfrog_order = (int32_t)st->order;
    c->whfast_coordinates = (int32_t)st->coordinates;
    c->whfast_corrector = (int32_t)st->corrector;
    c->whfast_corrector2 = (int32_t)st->corrector2;
    c->whfast_kernel = (int32_t)st->kernel;
    c->whfast_keep_unsynchronized = (int32_t)st->keep_unsynchronized;
    c->exact_finish_time = r->exact_finish_time;
    return 0;
}

/* Take the boundary and collision fields for the device (see rgpu_rebound.h). */
static void hold_fields(struct reb_simulation* r, struct rgpu_rebound_state* st) {
    st->r = r;
    if (r->boundary != REB_BOUNDARY_NONE) {
        st->boundary = (int)r->boundary;
        r->boundary = REB_BOUNDARY_NONE;
    }
    if (r->collision != REB_COLLISION_NONE) {
        st->collision = (int)r->collision;
        r->collision = REB_COLLISION_NONE;
    }
}

static void rgpu_rebound_step(struct reb_simulation* r, void* p) {
    struct rgpu_rebound_state* st = (struct rgpu_rebound_state*)p;
    if (!st) {
        reb_simulation_error(r, "rgpu: integrator state missing");
        r->status = REB_STATUS_GENERIC_ERROR;
        return;
    }
    int rc;
    if (!st->sim) {
        rc = rgpu_sim_create(&st->sim);
        if (rc) {
            st->sim = NULL;
            fail(r, st, "rgpu_sim_create", rc);
            return;
        }
    }
    hold_fields(r, st);
    rgpu_config c;
    if (make_config(r, st, &c)) return;
    if (!st->have_config || memcmp(&c, &st->pushed, sizeof(c)) != 0) {
        rc = rgpu_sim_configure(st->sim, &c);
        if (rc) { fail(r, st, "rgpu_sim_configure", rc); return; }
        rc = rgpu_sim_set_restitution_fn(st->sim, r->coefficient_of_restitution ? restitution_trampoline : NULL, r);
        if (rc) { fail(r, st, "rgpu_sim_set_restitution_fn", rc); return; }
        st->pushed = c;
        st->have_config = 1;
    }
    if (r->did_modify_particles || st->N_device != r->N || rgpu_sim_N(st->sim) != r->N) {
        rc = rgpu_sim_set_particles(st->sim, r->particles, r->N, sizeof(struct reb_particle));
        if (rc) { fail(r, st, "rgpu_sim_set_particles", rc); return; }
        st->N_device = r->N;
        st->device_ahead = 0;
    }
    rc = rgpu_steps(st->sim, 1);
    st->device_ahead = 1;
    rgpu_config after;
    if (rgpu_sim_get_config(st->sim, &after) == 0) {
        r->t = after.t;
        r->rand_seed = after.rand_seed;
        r->collisions_log_n = after.collisions_log_n;
        r->collisions_plog = after.collisions_plog;
        st->pushed.t = after.t;
        st->pushed.rand_seed = after.rand_seed;
        st->pushed.collisions_log_n = after.collisions_log_n;
        st->pushed.collisions_plog = after.collisions_plog;
        st->pushed.status = after.status;
        if (after.status == REB_STATUS_COLLISION) r->status = REB_STATUS_COLLISION;
    }
    if (rc) { fail(r, st, "rgpu_steps", rc); return; }
    r->dt_last_done = r->dt;
    if (st->scheme == RGPU_INTEGRATOR_WHFAST && !st->safe_mode) r->is_synchronized = 0;
}

static void rgpu_rebound_synchronize(struct reb_simulation* r, void* p) {
    struct rgpu_rebound_state* st = (struct rgpu_rebound_state*)p;
    if (!st || !st->sim) return;
    if (st->scheme == RGPU_INTEGRATOR_WHFAST) {
        const int rc = rgpu_synchronize(st->sim);
        if (rc) { fail(r, st, "rgpu_synchronize", rc); return; }
        st->device_ahead = 1;
    }
    if (pull_particles(r, st, st->N_device)) return;
    r->is_synchronized = 1;
}

static void rgpu_rebound_did_add_particle(struct reb_simulation* r) {
    struct rgpu_rebound_state* st = ours(r);
    if (!st || !st->sim) return;
    /* the new record is already appended: bring the older ones up to date */
    if (st->N_device <= r->N) pull_particles(r, st, st->N_device);
    r->did_modify_particles = 1;
}

static void rgpu_rebound_will_remove_particle(struct reb_simulation* r, size_t index) {
    (void)index;
    struct rgpu_rebound_state* st = ours(r);
    if (!st || !st->sim) return;
    if (st->N_device == r->N) pull_particles(r, st, st->N_device);
    r->did_modify_particles = 1;
}

static void rgpu_rebound_free(void* p) {
    struct rgpu_rebound_state* st = (struct rgpu_rebound_state*)p;
    if (!st) return;
    struct reb_simulation* r = st->r;
    if (r && st->sim) {
        if (st->N_device == r->N) pull_particles(r, st, st->N_device);
        if (r->boundary == REB_BOUNDARY_NONE) r->boundary = st->boundary;
        if (r->collision == REB_COLLISION_NONE) r->collision = st->collision;
    }
    if (st->sim) rgpu_sim_free(st->sim);
    free(st);
}
