// Internal declarations shared by the CUDA translation units of librebound_gb300.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <atomic>
#include <string>
#include <vector>
#include "../../include/rebound_gb300.h"

// Device status word bits (OR-ed by kernels, read by the host).
enum : uint32_t {
    DEV_ERR_NONFINITE = 1u << 0,
    DEV_ERR_OUT_OF_BOX = 1u << 1,
    DEV_ERR_DUPLICATE = 1u << 2,
    DEV_ERR_TREE_DEPTH = 1u << 3,
    DEV_ERR_OVERFLOW = 1u << 4,
    DEV_ERR_KEPLER = 1u << 5,
    DEV_ERR_STACK = 1u << 6,
    DEV_ERR_PROGRAM = 1u << 7,
};

// Particle state in HBM, structure of arrays.  All arrays have `cap` entries.
struct ParticlesSoA {
    double *x, *y, *z, *vx, *vy, *vz, *ax, *ay, *az, *m, *r;
};

struct TreeBuffers;      // tree.cu
struct FixGuard;         // direct.cu
struct SeiCache { double lastdt = 0., sindt = 0., tandt = 0., sindtz = 0., tandtz = 0.; };  // src/integrator_sei.c:91-101
struct WhfastBuffers;    // whfast.cu

struct rgpu_sim {
    rgpu_config cfg{};
    size_t N = 0, cap = 0;
    cudaStream_t stream = nullptr;
    ParticlesSoA p{};
    double* soa_block = nullptr;       // backing allocation of p
    double4_32a* jpos = nullptr;           // packed (x, y, z, G*m) per particle for direct sums
    float4* jsplit = nullptr;          // (hi, lo) float split of x,y,z and G*m: 2 float4 per particle
    double* partial = nullptr;         // j-split partial accelerations [splits][3][cap]
    size_t partial_cap = 0;
    FixGuard* fixg = nullptr;          // fixed-point exactness guard buffers (direct.cu)
    void* stage = nullptr;             // device staging for AoS upload/download
    size_t stage_cap = 0;
    uint32_t* d_status = nullptr;      // device error word
    double* d_scalar = nullptr;        // small device scratch (energy etc.)
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // Dominant-kernel timer: event pairs recorded around each force-kernel launch
    // on the handle's stream, accumulated lazily.
    bool ktimer_on = false;
    std::vector<cudaEvent_t> kt_ev;     // 2 per slot
    std::vector<char> kt_pending;
    size_t kt_next = 0;
    double kt_ms = 0.;
    int64_t kt_count = 0;
    void* flush_buf = nullptr;
    size_t flush_bytes = 0;
    bool did_modify = true;
    bool whfast_synchronized = true;
    double dt_last_done = 0.;          // dt of the last completed step (src/rebound.h: dt_last_done)
    int64_t steps_done = 0;            // src/rebound.h: steps_done
    std::string archive_path;          // automatic snapshots (src/rebound.h: simulationarchive_*)
    double archive_interval = 0., archive_next = 0.;
    int64_t archive_step = 0, archive_next_step = 0;
    SeiCache sei{};
    // last collision search result (device), consumed by the resolve stage
    size_t n_pairs = 0;
    rgpu_collision* dev_pairs = nullptr;
    int* pc_count = nullptr;            // direct search: per (ghost box, particle) counts
    long long* pc_off = nullptr;
    size_t pc_cap = 0;
    rgpu_collision* dp_pairs = nullptr; // direct search output
    size_t dp_cap = 0;
    TreeBuffers* tree = nullptr;
    WhfastBuffers* wh = nullptr;
    // velocity-dependent restitution for the hardsphere resolve (host callback)
    double (*eps_fn)(void*, double) = nullptr;
    void* eps_user = nullptr;
    double resolve_ms = 0.;             // host wall time spent in the collision resolve
    int64_t resolve_calls = 0;
    std::string msg;
};

// Kernel launches of this library since load (worker threads and host callers
// count concurrently, hence atomic).
extern std::atomic<int64_t> g_launches;

int set_error(rgpu_sim* s, int code, const std::string& what);
int check_cuda(rgpu_sim* s, cudaError_t e, const char* what);
int read_status(rgpu_sim* s);
int ensure_partial(rgpu_sim* s, size_t splits);
// Bracket a dominant-kernel launch with the handle's kernel timer (no-ops when off).
void ktimer_begin(rgpu_sim* s);
void ktimer_end(rgpu_sim* s);

// direct.cu
int direct_accel(rgpu_sim* s, int mode);
int direct_energy(rgpu_sim* s, double* e);
void direct_free(rgpu_sim* s);
// tree.cu
int tree_accel(rgpu_sim* s);
int tree_collisions(rgpu_sim* s, rgpu_collision* out, size_t cap, size_t* n_found, bool device_only,
                    bool line = false);
void tree_free(rgpu_sim* s);
// collide.cu
int direct_collisions(rgpu_sim* s, rgpu_collision* out, size_t cap, size_t* n_found, bool device_only,
                      bool line = false);
int resolve_collisions_device(rgpu_sim* s);
void collide_free(rgpu_sim* s);
// whfast.cu
int whfast_step(rgpu_sim* s);
int whfast_synchronize(rgpu_sim* s);
void whfast_free(rgpu_sim* s);
int whfast_load_coordinates(rgpu_sim* s, const double* host7N);   // 7 N doubles, field-major
// snapshot.cu
int archive_heartbeat(rgpu_sim* s);
// step.cu
int boundary_check(rgpu_sim* s);
void ghostbox(const rgpu_config& c, int i, int j, int k, double gb[6]);

static inline size_t n_active(const rgpu_sim* s) {
    return s->cfg.N_active < 0 ? s->N : (size_t)s->cfg.N_active;
}

#define RGPU_TRY(expr) do { int _rc = (expr); if (_rc) return _rc; } while (0)
#define RGPU_CUDA(s, expr) do { cudaError_t _e = (expr); if (_e != cudaSuccess) return check_cuda((s), _e, #expr); } while (0)

static inline unsigned grid_for(size_t n, unsigned block) {
    return (unsigned)((n + block - 1) / block);
}
