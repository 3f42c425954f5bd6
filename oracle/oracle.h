/*
 * oracle.h -- CPU restatement of the REBOUND 5.0.0 force-and-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 * The product (rebound_gb300) never links, loads or calls it.
 *
 * Every routine restates the reference algorithm it names (file:line in the
 * REBOUND source tree) with the same floating-point operation order, so that
 * built with -ffp-contract=off it reproduces the reference bit for bit where
 * the reference itself is deterministic.  Parity of this restatement is pinned
 * against golden vectors produced by the unmodified reference library
 * (tests/golden/make_golden.py, tests/test_oracle_golden.py).
 */
#ifndef REBOUND_GB300_ORACLE_H
#define REBOUND_GB300_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same field order and size (112 B on LP64) as struct reb_particle,
 * src/rebound.h:86-104. */
typedef struct orc_particle {
    double x, y, z, vx, vy, vz, ax, ay, az, m, r;
    const void* name;
    void* ap;
    void* sim;
} orc_particle;

/* One pair as in struct reb_collision (src/rebound.h:144-149). */
typedef struct orc_collision {
    size_t p1, p2;
    double gb[6];
    size_t ri;
} orc_collision;

/* One tree cell, exported in depth-first order for membership parity. */
typedef struct orc_cell {
    int32_t root;       /* root box index */
    int32_t depth;      /* 0 for a root cell */
    uint64_t path;      /* octant digits, 3 bits per level, most significant first */
    double x, y, z, w;  /* geometric centre and width */
    double m, mx, my, mz;
    int64_t pt;         /* leaf: particle index; internal: -(particle count) */
} orc_cell;

/* Hot-path configuration: the subset of struct reb_simulation
 * (src/rebound.h:238-413) that the path reads. */
typedef struct orc_sim {
    double t, G, softening, dt, OMEGA, OMEGAZ, root_size, opening_angle2;
    size_t N;
    size_t N_active;            /* SIZE_MAX = all active */
    int testparticle_type;
    int gravity_ignore_terms;   /* 0 none, 1 between 0 and 1, 2 involving 0 */
    int N_root_x, N_root_y, N_root_z;
    int N_ghost_x, N_ghost_y, N_ghost_z;
    int boundary;               /* 0 none, 1 open, 2 periodic, 3 shear */
    int whfast_safe_mode;
    int whfast_is_synchronized;
    int whfast_did_modify;
    unsigned int rand_seed;
    int error;                  /* nonzero after a reference error condition */
    orc_particle* particles;
    orc_particle* p_jh;         /* WHFast Jacobi state, N entries (caller-owned) */
    double* cs;                 /* compensated-sum scratch, 3N (caller-owned) */
    double sei_lastdt, sei_sindt, sei_tandt, sei_sindtz, sei_tandtz;
    /* WHFast options (src/integrator_whfast.h:29-50), Jacobi coordinates */
    int whfast_corrector;       /* 0, 3, 5, 7, 11, 17 */
    int whfast_corrector2;
    int whfast_kernel;          /* 0 DEFAULT, 1 MODIFIEDKICK, 2 COMPOSITION, 3 LAZY */
    int whfast_keep_unsynchronized;
    int tree_quadrupole;        /* 1: the reference built with -DQUADRUPOLE (src/tree.c:147-320) */
    int whfast_coordinates;     /* 0 Jacobi, 1 democratic heliocentric, 2 WHDS, 3 barycentric */
    int whfast_gravity;         /* the gravity WHFast evaluates: 0 BASIC, 1 COMPENSATED, 2 NONE */
    int reserved0;
} orc_sim;

/* Gravity (src/gravity.c). *_serial = the reference built without OpenMP;
 * *_omp = the reference's OpenMP gather loops, run with omp threads. */
void orc_gravity_basic_serial(orc_sim* r);
void orc_gravity_basic_omp(orc_sim* r);
void orc_gravity_basic_omp_rows(orc_sim* r, size_t i0, size_t i1);
void orc_gravity_compensated_serial(orc_sim* r);
void orc_gravity_compensated_omp(orc_sim* r);
void orc_gravity_compensated_omp_rows(orc_sim* r, size_t i0, size_t i1);
void orc_gravity_tree(orc_sim* r);
void orc_gravity_tree_rows(orc_sim* r, size_t i0, size_t i1);
int  orc_tree_export(orc_sim* r, orc_cell* out, size_t cap, size_t* n_out);

/* Boundary (src/boundary.c). */
void orc_boundary_check(orc_sim* r);
void orc_boundary_ghostbox(const orc_sim* r, int i, int j, int k, double gb[6]);

/* Collision search (src/collision.c:49-342); fills out[] in the reference's
 * discovery order, without the random shuffle. Returns the number of pairs
 * (which may exceed cap; only cap are written). */
size_t orc_collision_search_direct(orc_sim* r, orc_collision* out, size_t cap);
size_t orc_collision_search_tree(orc_sim* r, orc_collision* out, size_t cap);
size_t orc_collision_search_tree_omp(orc_sim* r, orc_collision* out, size_t cap);
size_t orc_collision_search_line(orc_sim* r, double dt_last_done, orc_collision* out, size_t cap);
size_t orc_collision_search_linetree(orc_sim* r, double dt_last_done, orc_collision* out, size_t cap);

/* Integrators. */
void orc_leapfrog_step(orc_sim* r, int gravity);              /* order 2 DKD */
void orc_sei_step(orc_sim* r, int gravity);
int orc_leapfrog_step_order(orc_sim* r, int gravity, int order);   /* order 2, 4, 6, 8; nonzero: unsupported */
void orc_whfast_step(orc_sim* r);                             /* Jacobi, DEFAULT kernel */
void orc_whfast_steps(orc_sim* r, long n);                    /* n steps (timing) */
void orc_whfast_synchronize(orc_sim* r);
void orc_whfast_kepler_solver(orc_particle* p, double mu, double dt);
void orc_inertial_to_jacobi_posvel(const orc_particle* ps, orc_particle* pj, const orc_particle* pm, size_t N, size_t N_active);
void orc_jacobi_to_inertial_posvel(orc_particle* ps, const orc_particle* pj, const orc_particle* pm, size_t N, size_t N_active);

/* Diagnostics (src/tools.c:108-162). */
double orc_energy(const orc_sim* r);
/* Hardsphere resolution with constant restitution (src/collision.c:573-665). */
void orc_collision_resolve_hardsphere(orc_sim* r, const orc_collision* c, double eps, double minimum_collision_velocity);

/* Seeded Plummer sphere (src/tools.c:463-502), truncated at r <= rmax. */
void orc_ic_plummer(unsigned int seed, size_t N, double M, double R, double rmax, orc_particle* out);

#ifdef __cplusplus
}
#endif
#endif
