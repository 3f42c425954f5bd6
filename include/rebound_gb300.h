/*
 * rebound_gb300.h -- C ABI of the GB300-native (sm_103a) force-and-step path
 * for REBOUND 5.0.0.
 *
 * Plain C types only: pointers, sizes, doubles.  No CUDA or torch types cross
 * this boundary.  The library keeps particle state resident in GPU memory
 * between calls; the host copy is only touched by rgpu_sim_set_particles /
 * rgpu_sim_get_particles, exactly the points where REBOUND's own core hands
 * over or reads back `r->particles`.
 *
 * Every function returns 0 (RGPU_OK) on success or an RGPU_ERR_* code; the
 * message for the last failure of a handle is available from
 * rgpu_sim_last_error().  Nothing here calls exit() or traps the GPU: device
 * errors (non-finite input, duplicate tree positions, Kepler non-convergence,
 * output overflow) are written to a device status word that the host reads.
 *
 * Each entry point names the reference interface it replaces (file:line in the
 * REBOUND source tree).
 */
#ifndef REBOUND_GB300_H
#define REBOUND_GB300_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define RGPU_OK                 0
#define RGPU_ERR_ARG            1   /* invalid argument or configuration */
#define RGPU_ERR_CUDA           2   /* CUDA runtime error (no device, launch failure) */
#define RGPU_ERR_NOMEM          3   /* device allocation failed */
#define RGPU_ERR_UNSUPPORTED    4   /* mode combination the reference also rejects */
#define RGPU_ERR_NONFINITE      5   /* particle with non-finite coordinates (src/tree.c:66-69) */
#define RGPU_ERR_OUT_OF_BOX     6   /* particle outside the root boxes (src/tree.c:263-268) */
#define RGPU_ERR_DUPLICATE      7   /* two particles at the same position in the tree (src/tree.c:119-123) */
#define RGPU_ERR_TREE_DEPTH     8   /* octree deeper than the device key supports */
#define RGPU_ERR_OVERFLOW       9   /* caller's output buffer too small (count is still reported) */
#define RGPU_ERR_CAPACITY      10   /* request exceeds a fixed capacity of the entry point */
#define RGPU_ERR_TIMEOUT       11   /* a host-side wait ran out; the request is still in flight */

/* ---- enumerations: values equal REBOUND's enums (src/rebound.h:372-393) -- */
enum { RGPU_GRAVITY_NONE = 0, RGPU_GRAVITY_BASIC = 1, RGPU_GRAVITY_COMPENSATED = 2,
       RGPU_GRAVITY_TREE = 3,
       /* GB300 additions: FP64 displacement, FP32 rsqrt/force, compensated FP32-pair
        * accumulation (MIXED); the same with the FP64 displacement formed exactly
        * from a two-float split of each coordinate (MIXED_SPLIT). */
       RGPU_GRAVITY_MIXED = 64, RGPU_GRAVITY_MIXED_SPLIT = 65,
       /* TREE with the work split: roots within ceil(1/theta)+1 root widths of a
        * particle are walked exactly as the reference does; every other root is
        * provably never opened and its monopole is summed by a tiled sweep in
        * mixed precision (FP64 displacement via two-float splits, FP32 force). */
       RGPU_GRAVITY_TREE_SPLIT = 66 };
enum { RGPU_COLLISION_NONE = 0, RGPU_COLLISION_DIRECT = 1, RGPU_COLLISION_TREE = 2,
       RGPU_COLLISION_LINE = 4, RGPU_COLLISION_LINETREE = 5 };   /* paths over the last step */
enum { RGPU_BOUNDARY_NONE = 0, RGPU_BOUNDARY_OPEN = 1, RGPU_BOUNDARY_PERIODIC = 2, RGPU_BOUNDARY_SHEAR = 3 };
enum { RGPU_INTEGRATOR_LEAPFROG = 0, RGPU_INTEGRATOR_SEI = 1, RGPU_INTEGRATOR_WHFAST = 2 };
enum { RGPU_RESOLVE_HALT = 0, RGPU_RESOLVE_HARDSPHERE = 1, RGPU_RESOLVE_NONE = 2 };

/* Hot-path fields of struct reb_simulation (src/rebound.h:238-413). */
typedef struct rgpu_config {
    double G;                  /* :240 */
    double softening;          /* :241 */
    double dt;                 /* :244 */
    double t;                  /* current time; advanced by the steppers */
    double OMEGA, OMEGAZ;      /* :242-243 (SEI, shear boundary); OMEGAZ=-1 means OMEGA */
    double root_size;          /* :313 */
    double opening_angle2;     /* :276 */
    double coefficient_of_restitution;  /* constant epsilon for hardsphere resolve */
    double minimum_collision_velocity;  /* src/collision.c:624-628 */
    int64_t N_active;          /* -1: all particles active (SIZE_MAX in REBOUND) */
    int32_t testparticle_type;
    int32_t gravity_ignore_terms;       /* 0 none, 1 between 0 and 1, 2 involving 0 */
    int32_t N_root_x, N_root_y, N_root_z;
    int32_t N_ghost_x, N_ghost_y, N_ghost_z;
    int32_t gravity;           /* RGPU_GRAVITY_* */
    int32_t collision;         /* RGPU_COLLISION_* */
    int32_t collision_resolve; /* RGPU_RESOLVE_* */
    int32_t boundary;          /* RGPU_BOUNDARY_* */
    int32_t integrator;        /* RGPU_INTEGRATOR_* */
    int32_t whfast_safe_mode;  /* src/integrator_whfast.h: safe_mode, default 1 */
    uint32_t rand_seed;        /* src/rebound.h:359; drives the pair-list shuffle */
    int32_t status;            /* REB_STATUS_* value after a step (7 = collision halt) */
    int64_t collisions_log_n;  /* number of resolved hardsphere collisions */
    int32_t leapfrog_order;    /* 2 (default; 0 means 2), 4, 6 or 8: src/integrator_leapfrog.c:97-203 */
    int32_t whfast_coordinates; /* 0 Jacobi (default), 1 democratic heliocentric, 2 WHDS, 3 barycentric (src/integrator_whfast.h:39-43) */
    /* src/integrator_whfast.h:29-47 (Jacobi coordinates only where not 0): */
    int32_t whfast_corrector;   /* first symplectic corrector order: 0 (off), 3, 5, 7, 11 or 17 */
    int32_t whfast_corrector2;  /* 1: second symplectic corrector */
    int32_t whfast_kernel;      /* 0 DEFAULT, 1 MODIFIEDKICK, 2 COMPOSITION, 3 LAZY */
    int32_t whfast_keep_unsynchronized;  /* 1: synchronize leaves the integrator state unsynchronized */
    int32_t exact_finish_time;  /* src/rebound.h: 1 (default) lands integrate exactly on tmax */
    int32_t tree_quadrupole;    /* 1: tree cells carry mass quadrupoles, as the reference built with
                                   -DQUADRUPOLE (src/tree.c:147-320, src/Makefile.defs:90-91) */
    double collisions_plog;     /* src/rebound.h:346: y-momentum transferred by hardsphere collisions
                                   (src/collision.c:655-662), accumulated by the resolve */
} rgpu_config;

/* One overlapping, approaching pair: same layout as struct reb_collision
 * (src/rebound.h:144-149). gb = ghost-box offset (x,y,z,vx,vy,vz). */
typedef struct rgpu_collision {
    size_t p1, p2;
    double gb[6];
    size_t ri;                 /* root box of p2 (TREE search) */
} rgpu_collision;

typedef struct rgpu_sim rgpu_sim;   /* opaque device-resident simulation */

/* rgpu_config with REBOUND's defaults (src/simulation.c:100-120). */
void rgpu_config_default(rgpu_config* cfg);

/* Create / destroy a device-resident simulation on the current CUDA device.
 * Replaces the integrator-state create/free callbacks (src/rebound.h:170-179). */
int  rgpu_sim_create(rgpu_sim** out);
void rgpu_sim_free(rgpu_sim* sim);
const char* rgpu_sim_last_error(const rgpu_sim* sim);

/* Set / read the hot-path configuration (t, status, rand_seed,
 * collisions_log_n and collisions_plog are updated by the steppers). */
int rgpu_sim_configure(rgpu_sim* sim, const rgpu_config* cfg);
int rgpu_sim_get_config(const rgpu_sim* sim, rgpu_config* cfg);
/* Velocity-dependent coefficient of restitution for the hardsphere resolve:
 * fn(user, v) is called on the host for each resolved pair with the normal
 * relative velocity v, as REBOUND calls r->coefficient_of_restitution(r, v)
 * (src/collision.c:603-606); fn == NULL restores the constant
 * cfg.coefficient_of_restitution. */
int rgpu_sim_set_restitution_fn(rgpu_sim* sim, double (*fn)(void* user, double v), void* user);
/* Host wall time spent in the collision resolve stage (shuffle, gather of the
 * touched particles, hardsphere, scatter) since the handle was created, and the
 * number of resolves.  No reference counterpart (diagnostic). */
int rgpu_sim_resolve_time(rgpu_sim* sim, double* ms, int64_t* calls);

/* Upload / download particles.  `particles` points at N records of `stride`
 * bytes whose first 11 doubles are x,y,z,vx,vy,vz,ax,ay,az,m,r -- the layout of
 * struct reb_particle (src/rebound.h:86-104, stride 112) or a dense 88-byte
 * record.  get_particles writes only those 11 doubles of each record.
 * set_particles marks the state modified (r->did_modify_particles,
 * src/particle.c:75) so WHFast recomputes Jacobi coordinates. */
int rgpu_sim_set_particles(rgpu_sim* sim, const void* particles, size_t N, size_t stride);
int rgpu_sim_get_particles(rgpu_sim* sim, void* particles, size_t N, size_t stride);
size_t rgpu_sim_N(const rgpu_sim* sim);

/* Accelerations for the configured gravity mode.
 * Replaces reb_simulation_update_acceleration (src/simulation.c:640-689) for
 * REB_GRAVITY_NONE/BASIC/COMPENSATED/TREE (src/gravity.c:47-531). */
int rgpu_update_acceleration(rgpu_sim* sim);

/* Build the octree for the current positions (src/tree.c:254-271 and
 * :209-229) and write its cells depth-first (roots by index, octants 0..7) as
 * 88-byte records {int32 root, int32 depth, uint64 path (3 bits per level),
 * double x, y, z, w, m, mx, my, mz, int64 pt} -- pt is the particle index of a
 * leaf or minus the particle count of an internal cell (struct reb_treecell,
 * src/tree.h:81-103).  Requires root_size > 0.  RGPU_ERR_OVERFLOW if more than
 * cap cells (the count is still written). */
int rgpu_tree_export(rgpu_sim* sim, void* cells, size_t cap, size_t* n_cells);

/* Overlapping + approaching pairs for the configured collision mode, in the
 * reference's discovery order, before its random shuffle.  Replaces the search
 * half of reb_collision_search (src/collision.c:49-342).  *n_found receives the
 * full count; if it exceeds cap, RGPU_ERR_OVERFLOW is returned. */
int rgpu_collision_search(rgpu_sim* sim, rgpu_collision* out, size_t cap, size_t* n_found);

/* N_steps full steps: integrator step (leapfrog order 2, SEI, or WHFast
 * Jacobi/DEFAULT kernel), boundary check, collision search + shuffle + resolve.
 * Replaces reb_simulation_steps (src/simulation.c:500-512) with the step body
 * reb_simulation_step (src/simulation.c:514-603). */
int rgpu_steps(rgpu_sim* sim, int64_t N_steps);

/* Integrate to t = tmax with fixed dt, the last step shortened to land on tmax
 * (exact_finish_time = 1, src/simulation.c:318-341, 456-460). */
int rgpu_integrate(rgpu_sim* sim, double tmax);

/* WHFast: bring inertial particles up to date (src/integrator_whfast.c:1051-1111). */
int rgpu_synchronize(rgpu_sim* sim);

/* Total energy, unsoftened, test-particle aware (src/tools.c:108-162), of the
 * synchronized state; a WHFast run with safe_mode 0 keeps its unsynchronized
 * coordinates, so the call does not change the trajectory. */
int rgpu_energy(rgpu_sim* sim, double* energy);

/* Wait for the simulation's stream; returns the first device error, if any. */
int rgpu_sim_sync(rgpu_sim* sim);

/* ---- snapshots and archives (Simulationarchive counterpart) ------------ */
/* A snapshot is the device-resident state as it is -- configuration, particles
 * (not synchronized), WHFast coordinates and flags, dt_last_done, SEI cache,
 * step count -- so that a handle restored from it continues bit for bit.
 * Replaces reb_simulation_save_to_file / reb_simulation_create_from_simulationarchive
 * (src/simulationarchive.c:410-470) for this path; the byte layout is this
 * library's own (one record per snapshot, appended). */
int rgpu_sim_snapshot_size(rgpu_sim* sim, size_t* bytes);
int rgpu_sim_snapshot_write(rgpu_sim* sim, void* buf, size_t cap, size_t* written);
int rgpu_sim_snapshot_read(rgpu_sim* sim, const void* buf, size_t n);
/* interval = step = 0: append one snapshot now (reb_simulation_save_to_file);
 * interval != 0: a snapshot whenever t passes the next multiple
 * (reb_simulation_save_to_file_interval, src/simulationarchive.c:639-648);
 * step != 0: every `step` steps (reb_simulation_save_to_file_step, :657-666).
 * Automatic snapshots are taken before each step and at the end of
 * rgpu_integrate, as reb_simulationarchive_heartbeat (:377-408).
 * delete_file: remove the file first. */
int rgpu_sim_save_to_file(rgpu_sim* sim, const char* path, double interval, int64_t step, int delete_file);
/* Times and byte offsets of the whole snapshots in an archive (host only; a record
 * cut short by an interrupted write ends the list).  n = number found. */
int rgpu_archive_scan(const char* path, double* times, int64_t* offsets, size_t cap, size_t* n);
/* Restore snapshot `index` (negative counts from the end). */
int rgpu_sim_load_from_file(rgpu_sim* sim, const char* path, int64_t index);

/* ---- measurement helpers ---------------------------------------------- */
/* Average duration (ms) of the last launch of the dominant force kernel of
 * this handle, measured with CUDA events on the handle's stream. */
double rgpu_sim_last_kernel_ms(const rgpu_sim* sim);
/* Dominant-kernel timer: when enabled, every launch of the handle's force
 * kernel is bracketed by CUDA events on the handle's stream; kernel_time
 * returns the summed device time and the number of launches since enabling. */
int rgpu_sim_kernel_timer(rgpu_sim* sim, int enable);
int rgpu_sim_kernel_time(rgpu_sim* sim, double* total_ms, int64_t* launches);
/* Run n steps bracketed by CUDA events on the handle's stream; *ms = device time. */
int rgpu_sim_time_steps(rgpu_sim* sim, int64_t n, double* ms);
/* Overwrite `bytes` of scratch on the handle's stream (evicts L2 between timed steps). */
int rgpu_l2_flush(rgpu_sim* sim, size_t bytes);
/* Select how the FP64 kernels evaluate m/r^3 (0: library rsqrt; 1: FP32-seeded
 * binomial series in FP64; 2: the same with its h^2 term in FP32 via cvt; 3 (default):
 * as 2 with the conversions done on the integer pipe) and how MIXED
 * rounds the FP64 displacement to FP32 (1: conversion instruction; 0 (default):
 * integer-pipe rounding).  All variants meet the FP64 / mixed tolerances. */
int rgpu_set_kernel_variant(int rinv_variant, int mixed_cvt);
/* Pair arithmetic of BASIC/COMPENSATED (and the displacement of MIXED) in
 * direct summation without ghost boxes or pair exclusions: 2 (default) =
 * int64 fixed-point positions at a scale chosen per evaluation, displacement
 * and (r^2+eps^2)^(-3/2) on the integer pipes, FP64 for G m f and the sums;
 * 1 = fixed-point displacement (equal to the FP64 subtraction for coordinates
 * >= 2^-8 of the largest) with FP64 r^2 and m/r^3; 0 = FP64 throughout.
 * In modes 1 and 2 BASIC and COMPENSATED keep the FP64 result on every input:
 * an exactness guard bounds, per particle, the force error that rounding
 * smaller coordinates onto the fixed-point grid can cause, and recomputes in
 * FP64 (the FP64 subtraction) every particle whose bound exceeds 5e-15 of its
 * force -- or every particle, when more than a quarter of the bodies are off
 * the grid.  No reference counterpart (tuning only). */
int rgpu_set_displacement_mode(int mode);
/* Counters of the exactness guard from the handle's last BASIC/COMPENSATED
 * fixed-point evaluation (synchronises the handle's stream): bodies with a
 * coordinate off the fixed-point grid, and particles recomputed in FP64
 * (N when all were).  Both -1 before the first such evaluation.
 * No reference counterpart (diagnostic). */
int rgpu_sim_guard_stats(rgpu_sim* sim, int64_t* n_inexact, int64_t* n_redo);
/* Count of this library's kernel launches since load. */
int64_t rgpu_launch_count(void);
/* Measured sustained lane-operation rate (ops/s) of one instruction class or
 * FP64 routine on the current device: 0 = FP64 FMA, 1 = FP32 FMA,
 * 2 = FP64<->FP32 conversion, 3 = FP32 rsqrt (MUFU), 4 = integer ALU (3-input
 * logic op); the exact tree walk's IEEE routines on the integer pipes:
 * 5 = division, 6 = square root, 7 = square, 8 = product, 9 = sum of two
 * non-negative numbers; and the hardware FP64 forms: 10 = division,
 * 11 = square root, 12 = addition. */
int rgpu_probe_rate(int which, double* ops_per_s);
/* Self-check of the integer-pipe IEEE FP64 arithmetic used by the exact tree
 * walk (division, square root, non-negative addition, multiplication, square):
 * n pseudo-random operand sets from `seed`, each compared bit for bit with the
 * hardware operation; *mismatches counts differences.  No reference
 * counterpart. */
int rgpu_selftest_exactfp(long long n, unsigned long long seed, long long* mismatches);
/* Self-check of the serving kernel's FP64 division and square root
 * (hardware approximations refined by Newton steps) against the IEEE operations
 * on n pseudo-random operand sets: the largest differences in ulps.
 * No reference counterpart. */
int rgpu_selftest_fastmath(long long n, unsigned long long seed, double* worst_div_ulps, double* worst_sqrt_ulps);

/* Kepler drift of n independent bodies with gravitational parameters mu[i]
 * over dt[i] (universal variables, Stumpff series, Newton / quartic solver
 * with bisection fallback).  Device counterpart of the reference's public
 * reb_integrator_whfast_kepler_solver (src/integrator_whfast.c:241-427).
 * Inputs: records of `stride` bytes starting with x, y, z, vx, vy, vz; outputs
 * 6 doubles per body. */
int rgpu_kepler_solve(const void* bodies, size_t stride, const double* mu, const double* dt,
                      double* out, size_t n);

/* Direct-sum accelerations that allocate nothing -- for callers that cannot
 * call cudaMalloc when they need forces (a host framework that owns every
 * device allocation through its own pool, an embedding process whose
 * allocator is locked down).  No counterpart in the reference: REBOUND
 * computes forces on host memory it owns.
 * x, y, z, m (inputs) and ax, ay, az (outputs) are the caller's DEVICE arrays
 * of n doubles; stream is a cudaStream_t passed as a plain pointer (NULL for the
 * default stream); the call is asynchronous on that stream.  gravity is BASIC,
 * COMPENSATED, MIXED or MIXED_SPLIT; all particles active, no ghost boxes.
 * Scratch lives in a fixed 10 MiB device array inside the library (held by
 * every GPU that loads it until exit): n <= 65,536, else RGPU_ERR_CAPACITY.
 * The first call on each device looks up that array's address with the device
 * current; make it before any stream capture.  The address is kept for the life
 * of the process, so a cudaDeviceReset (or any teardown of the device's primary
 * context) invalidates it: do not call this entry point after one.  Calls share
 * the array: calls that overlap on the GPU race and must be serialised by the
 * caller. */
int rgpu_direct_accel_noalloc(const double* x, const double* y, const double* z, const double* m,
                              double* ax, double* ay, double* az, int64_t n, double G, double softening,
                              int gravity, void* stream);

/* ---- batched WHFast ensemble ------------------------------------------ */
/* Many independent small systems (2..16 bodies each; each one a REBOUND
 * simulation with WHFast, Jacobi coordinates, DEFAULT kernel, safe_mode 1,
 * no softening; src/integrator_whfast.c:1113-1259) advanced together.
 * particles: all systems' records back to back (stride bytes each, layout of
 * struct reb_particle); system s owns records [offsets[s], offsets[s+1]).
 * dts: per-system timestep.  exact = 1 selects kernels compiled without FMA
 * contraction (bit-identical to the reference's serial build); 0 selects the
 * faster FMA-contracted kernels; 2 runs democratic heliocentric coordinates
 * (the splitting of WHFast512, src/integrator_whfast512.c), bit-identical to
 * WHFast with coordinates = DEMOCRATICHELIOCENTRIC and safe_mode 1. */
typedef struct rgpu_ensemble rgpu_ensemble;
int  rgpu_ensemble_create(rgpu_ensemble** out, const void* particles, size_t stride, const int64_t* offsets,
                          size_t n_systems, const double* dts, double G, int exact);
void rgpu_ensemble_free(rgpu_ensemble* ens);
const char* rgpu_ensemble_last_error(const rgpu_ensemble* ens);
/* CTA size (32/64/128) of the persistent grid and steps fused per kernel launch. */
int  rgpu_ensemble_set_launch(rgpu_ensemble* ens, int block, int64_t steps_per_launch);
/* How systems map onto threads: RGPU_ENSEMBLE_THREAD (one thread advances one
 * system; the throughput mapping for many systems) or RGPU_ENSEMBLE_WARP (one warp
 * per system, lane i holding body i; the latency mapping, FMA flavour only).
 * No reference counterpart (the reference runs one simulation per call). */
enum { RGPU_ENSEMBLE_THREAD = 0, RGPU_ENSEMBLE_WARP = 1 };
int  rgpu_ensemble_set_mapping(rgpu_ensemble* ens, int mapping);
/* The mapping, CTA size and steps per launch in effect (after an autotune). */
int  rgpu_ensemble_get_launch(const rgpu_ensemble* ens, int* mapping, int* block, int64_t* steps_per_launch);
/* Advance every system by n steps (CUDA-graph replays of fused chunks). */
int  rgpu_ensemble_steps(rgpu_ensemble* ens, int64_t n);
int  rgpu_ensemble_time_steps(rgpu_ensemble* ens, int64_t n, double* ms);
/* Autotuner on the live ensemble (its probe steps advance the state): times
 * every mapping x CTA size over probe_steps, then max_steps_per_launch / 256, / 64,
 * / 16, / 4 and itself as steps per launch, and keeps the fastest combination (read it
 * back with rgpu_ensemble_get_launch). */
int  rgpu_ensemble_autotune(rgpu_ensemble* ens, int64_t probe_steps, int64_t max_steps_per_launch,
                            int* best_block, double* best_ms_per_step);
/* Write positions, velocities and masses back into the caller's records. */
int  rgpu_ensemble_get_particles(rgpu_ensemble* ens, void* particles, size_t stride);
/* Per-system total energy (src/tools.c:108-162) and time. */
int  rgpu_ensemble_energy(rgpu_ensemble* ens, double* energies);
int  rgpu_ensemble_times(rgpu_ensemble* ens, double* t);

/* ---- serving: continuous batching of integrate requests --------------- */
/* A request is one system the reference would run as one reb_simulation:
 * RGPU_SERVE_WHFAST: 2..16 bodies, WHFast (Jacobi, DEFAULT kernel), G = 1, no
 *   softening; one warp per system steps it in blocks of 32 steps, counted from
 *   its last step back, that merge the drifts of consecutive steps as the
 *   reference's safe_mode 0 does and end synchronised (the same map as
 *   safe_mode 1 to rounding); thread_per_system = 1 runs safe_mode 1 step by step;
 * RGPU_SERVE_CLUSTER: any N up to the pool, leapfrog (order 2) with the
 *   mixed-precision direct sum (RGPU_GRAVITY_MIXED_SPLIT), softening given.
 * A worker thread admits queued requests FIFO while the device bytes of the
 * resident ones stay within hbm_budget_bytes, and advances every resident
 * request in batched kernels each tick (WHFast: tick_ns of device time or
 * steps_per_launch steps per slot; clusters: cluster_steps_per_tick leapfrog
 * steps).  A request's result does not depend on which other requests share
 * its ticks, nor on how its steps fall into ticks. */
enum { RGPU_SERVE_WHFAST = 1, RGPU_SERVE_CLUSTER = 2 };
typedef struct rgpu_server_config {
    size_t hbm_budget_bytes;         /* default 120 GiB */
    int64_t steps_per_launch;        /* WHFast steps per slot per tick when tick_ns is 0 (warp
                                        slots extend it to the end of a 32-step block) or
                                        thread_per_system is 1 (default 64) */
    int32_t slots_per_bucket;        /* WHFast slots per body count (default 16,384) */
    int32_t pool_particles;          /* cluster particle pool (default 4,194,304) */
    int32_t cluster_steps_per_tick;  /* default 8 */
    int32_t thread_per_system;       /* 0 (default): one warp per WHFast system, lanes = bodies
                                        (lowest latency); 1: one thread per system */
    int64_t tick_ns;                 /* warp per system: > 0 (default 8,000,000, at most 1e9), each
                                        slot steps for about this much device time per tick, so
                                        light systems are not held back by the heaviest one of the
                                        tick; 0: each slot takes exactly steps_per_launch steps per
                                        tick */
} rgpu_server_config;
typedef struct rgpu_server_stats {
    int64_t completed, waiting, resident, ticks;
    double system_steps;             /* WHFast system-steps + cluster steps done */
    double pair_interactions;        /* cluster pair interactions done */
    size_t bytes_in_use;
} rgpu_server_stats;
typedef struct rgpu_server rgpu_server;
void rgpu_server_config_default(rgpu_server_config* cfg);
int  rgpu_server_create(rgpu_server** out, const rgpu_server_config* cfg);
void rgpu_server_free(rgpu_server* srv);
/* Queue one request (records of `stride` bytes as struct reb_particle); thread-safe. */
int  rgpu_server_submit(rgpu_server* srv, int kind, const void* particles, size_t n, size_t stride, double dt,
                        int64_t n_steps, double G, double softening, int64_t* request_id);
/* Wait up to timeout_s for a request; on completion copy its particles out (if
 * non-NULL), report submit-to-finish latency and forget the request.
 * RGPU_ERR_TIMEOUT if it is still running (call again). */
int  rgpu_server_wait(rgpu_server* srv, int64_t request_id, void* particles, size_t stride, double timeout_s,
                      double* latency_s);
int  rgpu_server_get_stats(rgpu_server* srv, rgpu_server_stats* out);

/* ---- seeded synthetic workloads (reference RNG conventions) ------------ */
/* Plummer sphere as reb_simulation_add_plummer (src/tools.c:463-502), keeping
 * only draws with r <= rmax; masses M/N. */
int rgpu_ic_plummer(unsigned int seed, size_t N, double M, double R, double rmax, void* out, size_t stride);
/* Shearing-sheet ring patch (examples/shearing_sheet/problem.c shape). */
int rgpu_ic_ring_patch(unsigned int seed, double Lx, double Ly, double Lz, double OMEGA, double surface_density,
                       double particle_density, double rmin, double rmax, double sigma_z, double sigma_v,
                       void* out, size_t stride, size_t cap, size_t* n_out);
/* One star + k planets (orbital elements as reb_particle_from_orbit,
 * src/tools.c:940-996), moved to the barycentre; *seed is advanced. */
int rgpu_ic_planetary(unsigned int* seed, int k, double G, double mmin, double mmax, double amin, double amax,
                      double sig_e, double sig_i, double hill_sep, void* out, size_t stride, double* p_inner);

#ifdef __cplusplus
}
#endif
#endif
