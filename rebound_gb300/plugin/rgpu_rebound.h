/* REBOUND-side binding of librebound_gb300: integrator plugins for REBOUND's
 * own C core.
 *
 * Compiled against REBOUND's public header (src/rebound.h of REBOUND 5.0.0) and
 * linked with librebound and librebound_gb300.  Each object below is a
 * `struct reb_integrator` (src/rebound.h:170-179); registering one with
 * reb_integrator_register (src/rebound.c:86-113) and selecting it with
 * reb_simulation_set_integrator (src/simulation.c:217-238) makes
 * reb_simulation_integrate / reb_simulation_steps run the GPU path:
 *
 *     rgpu_rebound_register(RGPU_INTEGRATOR_LEAPFROG, "gpu_leapfrog");
 *     struct rgpu_rebound_state* st = reb_simulation_set_integrator(r, "gpu_leapfrog");
 *     r->gravity = REB_GRAVITY_BASIC;              // BASIC, COMPENSATED, TREE or NONE
 *     reb_simulation_integrate(r, 10.);
 *
 * Particle state lives in GPU memory between steps.  r->particles is brought
 * up to date by reb_simulation_synchronize (which integrate calls on exit, and
 * before the pre/post timestep hooks), before a particle is removed, and when
 * the integrator is freed.  Host-side changes to particles reach the device
 * when r->did_modify_particles is set (as REBOUND's own setters do), when
 * particles are added or removed, or when N changes.
 *
 * While one of these integrators is selected, the device also runs the
 * boundary condition and the collision search (with the halt or hardsphere
 * resolve, and r->coefficient_of_restitution called on the host per
 * collision): the plugin moves r->boundary and r->collision into its state
 * and sets them to NONE on the REBOUND side, so that REBOUND's own host-side
 * boundary check and collision search (src/simulation.c:573-586) do not run on
 * stale host particles.  Setting either field again while the integrator is
 * selected hands the new value to the device; rgpu_rebound_boundary /
 * rgpu_rebound_collision read the values in effect.  Freeing the integrator
 * (switching integrators or reb_simulation_free) gives them back.
 *
 * Errors of the GPU library (no device, out of memory, an unsupported
 * configuration) are reported with reb_simulation_error and set r->status to
 * REB_STATUS_GENERIC_ERROR, so integrate returns with that status.
 *
 * Speed: the GPU pays off for direct sums and trees of thousands of particles
 * and more.  The plain WHFast path runs one small system per call on one warp,
 * about 37 µs per step for 5 bodies against about 2.5 µs for REBOUND's WHFast
 * on one CPU core; many systems belong in the batched ensemble
 * (rgpu_ensemble_*) or the request loop (rgpu_server_*).
 *
 * REBOUND 5.0.0's registry compares a new name against the entry after each
 * registered one (src/rebound.c:100-104), which reads its terminator once one
 * custom integrator exists: register at most one custom integrator per process.
 */
#ifndef RGPU_REBOUND_H
#define RGPU_REBOUND_H

#include "rebound.h"
#include "rebound_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Integrator state returned by reb_simulation_set_integrator for these
 * integrators.  The public fields mirror struct reb_integrator_whfast_state
 * (src/integrator_whfast.h:28-55) and struct reb_integrator_leapfrog_state
 * (src/integrator_leapfrog.h) and may be set between steps. */
struct rgpu_rebound_state {
    int scheme;                        /* RGPU_INTEGRATOR_LEAPFROG, _SEI or _WHFAST */
    unsigned int order;                /* leapfrog: 2 (default), 4, 6 or 8 */
    unsigned int corrector;            /* WHFast: 0, 3, 5, 7, 11 or 17 */
    unsigned int corrector2;           /* WHFast: 1 = second corrector */
    unsigned int kernel;               /* WHFast: 0 DEFAULT, 1 MODIFIEDKICK, 2 COMPOSITION, 3 LAZY */
    unsigned int coordinates;          /* WHFast: 0 JACOBI, 1 DEMOCRATICHELIOCENTRIC, 2 WHDS, 3 BARYCENTRIC */
    unsigned int safe_mode;            /* WHFast: 1 (default) */
    unsigned int keep_unsynchronized;  /* WHFast */
    /* internal */
    rgpu_sim* sim;                     /* device handle, created at the first step */
    struct reb_simulation* r;          /* the simulation whose boundary / collision fields are held */
    size_t N_device;                   /* particles on the device */
    int device_ahead;                  /* device state newer than r->particles */
    int boundary;                      /* REB_BOUNDARY_* held for the device */
    int collision;                     /* REB_COLLISION_* held for the device */
    int have_config;
    rgpu_config pushed;                /* last configuration sent to the device */
};

extern const struct reb_integrator rgpu_integrator_leapfrog;
extern const struct reb_integrator rgpu_integrator_sei;
extern const struct reb_integrator rgpu_integrator_whfast;

/* Register one of the three under `name` (it must not be a built-in name). */
void rgpu_rebound_register(int scheme, const char* name);
/* The device handle behind r's integrator (NULL before the first step or when
 * another integrator is selected). */
rgpu_sim* rgpu_rebound_handle(struct reb_simulation* r);
/* Boundary condition and collision search that the device runs for r. */
int rgpu_rebound_boundary(struct reb_simulation* r);
int rgpu_rebound_collision(struct reb_simulation* r);

#ifdef __cplusplus
}
#endif
#endif
