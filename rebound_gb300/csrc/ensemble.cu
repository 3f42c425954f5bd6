// Batched WHFast ensemble: thousands of independent small planetary systems
// (one REBOUND simulation each, WHFast DEFAULT kernel / safe_mode 1, Jacobi or
// democratic heliocentric coordinates) advanced together on one GPU.
//
// Systems are grouped into buckets by body count; each bucket is a
// structure-of-arrays block [field][body][system] in HBM.  One thread advances
// one system (fully unrolled over bodies).  A persistent grid sized to the
// GPU's resident capacity drains a queue of 32-system work units ordered
// largest body count first, so every SM stays busy until the cheapest units at
// the end.  A chunk of `steps_per_launch` steps (counter reset + persistent
// launch) is captured once into a CUDA graph and replayed.
//
// Second mapping, warp per system (whfast_warp.cuh, FMA flavour): lane i holds
// body i, so one system's Kepler drifts and force rows run in parallel; a
// persistent grid hands out single systems, largest first.  It wins when there
// are too few systems to fill the GPU thread-per-system.  The autotuner times
// both mappings (thread per system at 32 / 64 / 128 threads per CTA, warp per
// system) and a set of steps-per-launch values on the live ensemble and keeps
// the fastest combination.
#define ENSEMBLE_NS ens_fast
#define WH_FAST_MATH 1          // FMA-contracted flavour (whfast_core.cuh)
#define WH_INT_DIVSQRT 1        // IEEE division and sqrt on the integer pipes (whfast_core.cuh)
#include "ensemble_kernels.cuh"
#include "whfast_warp.cuh"
#include <algorithm>
#include <cstring>
#include <map>
#include <new>
#include <vector>

void* ensemble_exact_persistent_fn();
void* ensemble_exact_energy_fn(int nb);
void* ensemble_dh_persistent_fn();

struct EnsBucket {
    int nb = 0;
    int count = 0;
    double* st = nullptr;        // 7 * nb * count
    double* dt = nullptr;        // count
    double* t = nullptr;         // count
    std::vector<int> ids;        // system index of each slot
    cudaStream_t stream = nullptr;
};

// One system for the warp mapping.
struct WarpSys {
    double* st;
    const double* dt;
    double* t;
    int count, nb, sid, pad;
};

namespace {

template <int NB>
__device__ __noinline__ void warp_system(const WarpSys& S, int n_steps, double G, uint32_t* status) {
    const double h = S.dt[S.sid];
    whw::warp_steps<NB>(S.st, S.count, S.sid, n_steps, h, G, status);
    if ((threadIdx.x & 31) == 0) S.t[S.sid] += h * n_steps;
}

// Persistent warp-per-system scheduler: each warp takes the next system from a
// global counter (systems ordered by decreasing body count).
__global__ void __launch_bounds__(128) persistent_warp_kernel(const WarpSys* __restrict__ sys, int n, int n_steps,
                                                              double G, unsigned int* counter, uint32_t* status) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned int u = 0;
        if (lane == 0) u = atomicAdd(counter, 1u);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= (unsigned)n) return;
        const WarpSys S = sys[u];
        switch (S.nb) {
            case 2: warp_system<2>(S, n_steps, G, status); break;
            case 3: warp_system<3>(S, n_steps, G, status); break;
            case 4: warp_system<4>(S, n_steps, G, status); break;
            case 5: warp_system<5>(S, n_steps, G, status); break;
            case 6: warp_system<6>(S, n_steps, G, status); break;
            case 7: warp_system<7>(S, n_steps, G, status); break;
            case 8: warp_system<8>(S, n_steps, G, status); break;
            case 9: warp_system<9>(S, n_steps, G, status); break;
            case 10: warp_system<10>(S, n_steps, G, status); break;
            case 11: warp_system<11>(S, n_steps, G, status); break;
            case 12: warp_system<12>(S, n_steps, G, status); break;
            case 13: warp_system<13>(S, n_steps, G, status); break;
            case 14: warp_system<14>(S, n_steps, G, status); break;
            case 15: warp_system<15>(S, n_steps, G, status); break;
            default: warp_system<16>(S, n_steps, G, status); break;
        }
    }
}

// Self-check of the FP64-refined division and square root (wh::fast_div,
// wh::fast_sqrt; the serving kernel's forms) against the IEEE operations: the
// largest difference in ulps of
// the IEEE result over n operand sets from a counter-based generator.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double ulps(double got, double ref) {
    if (got == ref) return 0.;
    const double u = fabs(ref) * 0x1p-52;     // one ulp of a normal result, within a factor 2
    return fabs(got - ref) / (u > 0. ? u : 1e-300);
}
__global__ void fastmath_check(long long n, unsigned long long seed, unsigned long long* worst_div,
                               unsigned long long* worst_sqrt) {
    double wd = 0., ws = 0.;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const unsigned long long r1 = mix64(seed + 2 * (unsigned long long)k), r2 = mix64(seed + 2 * (unsigned long long)k + 1);
        // mantissas uniform, exponents in [-60, 60], signs mixed
        const double a = ldexp(1.0 + (double)(r1 >> 12) * 0x1p-52, (int)(r1 & 127) - 64) * ((r2 & 1) ? -1. : 1.);
        const double b = ldexp(1.0 + (double)(r2 >> 12) * 0x1p-52, (int)((r2 >> 1) & 127) - 64);
        wd = fmax(wd, ulps(wh::fast_div(a, b), a / b));
        wd = fmax(wd, ulps(wh::fast_rcp(b), 1. / b));
        ws = fmax(ws, ulps(wh::fast_sqrt(b), sqrt(b)));
    }
    atomicMax(worst_div, (unsigned long long)__double_as_longlong(wd));
    atomicMax(worst_sqrt, (unsigned long long)__double_as_longlong(ws));
}

}  // namespace

extern "C" int rgpu_selftest_fastmath(long long n, unsigned long long seed, double* worst_div_ulps,
                                      double* worst_sqrt_ulps) {
    if (n < 1 || !worst_div_ulps || !worst_sqrt_ulps) return RGPU_ERR_ARG;
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) { cudaGetLastError(); return RGPU_ERR_CUDA; }
    cudaMemset(d, 0, 2 * sizeof(unsigned long long));
    fastmath_check<<<152 * 8, 256>>>(n, seed, d, d + 1);
    g_launches++;
    unsigned long long h[2] = {0, 0};
    const cudaError_t e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) { cudaGetLastError(); return RGPU_ERR_CUDA; }
    *worst_div_ulps = __builtin_bit_cast(double, h[0]);
    *worst_sqrt_ulps = __builtin_bit_cast(double, h[1]);
    return RGPU_OK;
}

struct rgpu_ensemble {
    std::vector<EnsBucket> b;
    std::vector<int64_t> offsets;      // n_systems + 1 particle offsets
    size_t n_systems = 0;
    double G = 1.0;
    int exact = 0;               // 1: no FMA contraction (bit-identical to the reference)
    int dh = 0;                  // 1: democratic heliocentric coordinates (implies exact)
    int block = 128;
    int mapping = RGPU_ENSEMBLE_THREAD;  // RGPU_ENSEMBLE_THREAD or RGPU_ENSEMBLE_WARP
    int64_t steps_per_launch = 256;
    WarpSys* d_wsys = nullptr;           // systems for the warp mapping, largest first
    cudaStream_t stream = nullptr;
    uint32_t* d_status = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr, fork = nullptr;
    std::vector<cudaEvent_t> joins;
    ens_fast::Unit* d_units = nullptr;   // work units, largest body count first
    int n_units = 0;
    unsigned int* d_counter = nullptr;
    cudaGraphExec_t graph = nullptr;
    int64_t graph_steps = -1;
    int graph_block = -1;
    int graph_mapping = -1;
    std::string msg;
};

namespace {

int ens_err(rgpu_ensemble* e, int code, const std::string& m) {
    if (e) e->msg = m;
    return code;
}

#define ENS_CUDA(e, expr) do { cudaError_t _x = (expr); if (_x != cudaSuccess) { \
    return ens_err((e), _x == cudaErrorMemoryAllocation ? RGPU_ERR_NOMEM : RGPU_ERR_CUDA, \
                   std::string(#expr) + ": " + cudaGetErrorString(_x)); } } while (0)

typedef void (*EnergyFn)(const double*, int, double, double*);

EnergyFn energy_fn(const rgpu_ensemble* e, int nb) {
    return e->exact ? (EnergyFn)ensemble_exact_energy_fn(nb) : ens_fast::energy_for(nb);
}

typedef void (*PersistentFn)(const ens_fast::Unit*, int, int, double, unsigned int*, uint32_t*);

PersistentFn persistent_fn(const rgpu_ensemble* e) {
    if (e->dh) return (PersistentFn)ensemble_dh_persistent_fn();
    return e->exact ? (PersistentFn)ensemble_exact_persistent_fn() : ens_fast::persistent_kernel;
}

// Enqueue one chunk of `n` steps for every system: the unit counter is reset and
// a persistent grid (all SMs, occupancy-limited) drains the unit queue.
int enqueue_chunk(rgpu_ensemble* e, int n) {
    int dev = 0, nsm = 1, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e->mapping == RGPU_ENSEMBLE_WARP) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, persistent_warp_kernel, 128, 0) != cudaSuccess ||
            per_sm < 1) {
            cudaGetLastError();
            per_sm = 1;
        }
        const int ns = (int)e->n_systems;
        const int grid = std::max(1, std::min(nsm * per_sm, (ns + 3) / 4));
        ENS_CUDA(e, cudaMemsetAsync(e->d_counter, 0, sizeof(unsigned int), e->stream));
        persistent_warp_kernel<<<grid, 128, 0, e->stream>>>(e->d_wsys, ns, n, e->G, e->d_counter, e->d_status);
        g_launches++;
        ENS_CUDA(e, cudaGetLastError());
        return RGPU_OK;
    }
    PersistentFn f = persistent_fn(e);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, e->block, 0) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    const int warps_needed = e->n_units;
    int grid = nsm * per_sm;
    const int warps_per_block = e->block / 32;
    grid = std::max(1, std::min(grid, (warps_needed + warps_per_block - 1) / warps_per_block));
    ENS_CUDA(e, cudaMemsetAsync(e->d_counter, 0, sizeof(unsigned int), e->stream));
    f<<<grid, e->block, 0, e->stream>>>(e->d_units, e->n_units, n, e->G, e->d_counter, e->d_status);
    g_launches++;
    ENS_CUDA(e, cudaGetLastError());
    return RGPU_OK;
}

int build_graph(rgpu_ensemble* e, int64_t n) {
    if (e->graph && e->graph_steps == n && e->graph_block == e->block && e->graph_mapping == e->mapping)
        return RGPU_OK;
    if (e->graph) { cudaGraphExecDestroy(e->graph); e->graph = nullptr; }
    cudaGraph_t g;
    ENS_CUDA(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = enqueue_chunk(e, (int)n);
    const cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
    if (rc) return rc;
    ENS_CUDA(e, ce);
    const cudaError_t ie = cudaGraphInstantiate(&e->graph, g, 0);
    cudaGraphDestroy(g);
    ENS_CUDA(e, ie);
    e->graph_steps = n;
    e->graph_block = e->block;
    e->graph_mapping = e->mapping;
    return RGPU_OK;
}

int run_steps(rgpu_ensemble* e, int64_t n) {
    const int64_t spl = std::max<int64_t>(1, e->steps_per_launch);
    int64_t full = n / spl, rest = n % spl;
    if (full > 0) {
        const int rc = build_graph(e, spl);
        if (rc) return rc;
        for (int64_t k = 0; k < full; k++) ENS_CUDA(e, cudaGraphLaunch(e->graph, e->stream));
    }
    if (rest > 0) return enqueue_chunk(e, (int)rest);
    return RGPU_OK;
}

int read_status(rgpu_ensemble* e) {
    uint32_t st = 0;
    ENS_CUDA(e, cudaMemcpyAsync(&st, e->d_status, sizeof(st), cudaMemcpyDeviceToHost, e->stream));
    ENS_CUDA(e, cudaStreamSynchronize(e->stream));
    if (st) {
        cudaMemsetAsync(e->d_status, 0, sizeof(uint32_t), e->stream);
        return ens_err(e, RGPU_ERR_ARG, "Kepler solver hit its iteration cap");
    }
    return RGPU_OK;
}

}  // namespace

extern "C" {

int rgpu_ensemble_create(rgpu_ensemble** out, const void* particles, size_t stride, const int64_t* offsets,
                         size_t n_systems, const double* dts, double G, int exact) {
    if (!out || !particles || !offsets || !dts || stride < 88 || n_systems == 0) return RGPU_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { cudaGetLastError(); return RGPU_ERR_CUDA; }
    rgpu_ensemble* e = new (std::nothrow) rgpu_ensemble();
    if (!e) return RGPU_ERR_NOMEM;
    e->n_systems = n_systems;
    e->G = G;
    if (exact < 0 || exact > 2) { delete e; return RGPU_ERR_ARG; }
    e->exact = exact != 0;
    e->dh = exact == 2;
    e->offsets.assign(offsets, offsets + n_systems + 1);
    std::map<int, std::vector<int>> groups;
    for (size_t s = 0; s < n_systems; s++) {
        const int64_t nb = offsets[s + 1] - offsets[s];
        if (nb < 2 || nb > wh::kMaxBodies) { delete e; return RGPU_ERR_UNSUPPORTED; }
        groups[(int)nb].push_back((int)s);
    }
    int rc = RGPU_OK;
    if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&e->d_status, sizeof(uint32_t)) != cudaSuccess ||
        cudaMemset(e->d_status, 0, sizeof(uint32_t)) != cudaSuccess ||
        cudaEventCreate(&e->e0) != cudaSuccess || cudaEventCreate(&e->e1) != cudaSuccess ||
        cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming) != cudaSuccess)
        rc = RGPU_ERR_CUDA;
    const char* base = (const char*)particles;
    for (auto& kv : groups) {
        if (rc) break;
        EnsBucket B;
        B.nb = kv.first;
        B.count = (int)kv.second.size();
        B.ids = kv.second;
        const size_t nf = (size_t)B.nb * B.count;
        std::vector<double> h(7 * nf), hdt(B.count), ht(B.count, 0.0);
        for (int q = 0; q < B.count; q++) {
            const int s = B.ids[q];
            hdt[q] = dts[s];
            for (int i = 0; i < B.nb; i++) {
                const double* r = (const double*)(base + (size_t)(offsets[s] + i) * stride);
                const size_t o = (size_t)i * B.count + q;
                h[0 * nf + o] = r[0]; h[1 * nf + o] = r[1]; h[2 * nf + o] = r[2];
                h[3 * nf + o] = r[3]; h[4 * nf + o] = r[4]; h[5 * nf + o] = r[5];
                h[6 * nf + o] = r[9];
            }
        }
        if (cudaMalloc(&B.st, sizeof(double) * 7 * nf) != cudaSuccess ||
            cudaMalloc(&B.dt, sizeof(double) * B.count) != cudaSuccess ||
            cudaMalloc(&B.t, sizeof(double) * B.count) != cudaSuccess ||
            cudaStreamCreateWithFlags(&B.stream, cudaStreamNonBlocking) != cudaSuccess) {
            rc = RGPU_ERR_NOMEM;
        } else {
            cudaMemcpy(B.st, h.data(), sizeof(double) * 7 * nf, cudaMemcpyHostToDevice);
            cudaMemcpy(B.dt, hdt.data(), sizeof(double) * B.count, cudaMemcpyHostToDevice);
            cudaMemcpy(B.t, ht.data(), sizeof(double) * B.count, cudaMemcpyHostToDevice);
        }
        e->b.push_back(B);
        cudaEvent_t j;
        cudaEventCreateWithFlags(&j, cudaEventDisableTiming);
        e->joins.push_back(j);
    }
    if (!rc) {
        std::vector<ens_fast::Unit> units;
        for (auto it = e->b.rbegin(); it != e->b.rend(); ++it)          // largest body count first
            for (int f = 0; f < it->count; f += 32)
                units.push_back(ens_fast::Unit{it->st, it->dt, it->t, it->count, it->nb, f, 0});
        e->n_units = (int)units.size();
        std::vector<WarpSys> ws;
        for (auto it = e->b.rbegin(); it != e->b.rend(); ++it)
            for (int q = 0; q < it->count; q++) ws.push_back(WarpSys{it->st, it->dt, it->t, it->count, it->nb, q, 0});
        if (cudaMalloc(&e->d_units, sizeof(ens_fast::Unit) * units.size()) != cudaSuccess ||
            cudaMalloc(&e->d_wsys, sizeof(WarpSys) * ws.size()) != cudaSuccess ||
            cudaMalloc(&e->d_counter, sizeof(unsigned int)) != cudaSuccess) {
            rc = RGPU_ERR_NOMEM;
        } else {
            cudaMemcpy(e->d_units, units.data(), sizeof(ens_fast::Unit) * units.size(), cudaMemcpyHostToDevice);
            cudaMemcpy(e->d_wsys, ws.data(), sizeof(WarpSys) * ws.size(), cudaMemcpyHostToDevice);
        }
    }
    if (rc) { rgpu_ensemble_free(e); return rc; }
    *out = e;
    return RGPU_OK;
}

void rgpu_ensemble_free(rgpu_ensemble* e) {
    if (!e) return;
    if (e->stream) cudaStreamSynchronize(e->stream);
    if (e->graph) cudaGraphExecDestroy(e->graph);
    for (auto& B : e->b) {
        if (B.stream) cudaStreamSynchronize(B.stream);
        cudaFree(B.st); cudaFree(B.dt); cudaFree(B.t);
        if (B.stream) cudaStreamDestroy(B.stream);
    }
    for (auto j : e->joins) cudaEventDestroy(j);
    cudaFree(e->d_units);
    cudaFree(e->d_wsys);
    cudaFree(e->d_counter);
    if (e->fork) cudaEventDestroy(e->fork);
    if (e->e0) cudaEventDestroy(e->e0);
    if (e->e1) cudaEventDestroy(e->e1);
    cudaFree(e->d_status);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
}

const char* rgpu_ensemble_last_error(const rgpu_ensemble* e) { return e ? e->msg.c_str() : "null handle"; }

int rgpu_ensemble_set_launch(rgpu_ensemble* e, int block, int64_t steps_per_launch) {
    if (!e || (block != 32 && block != 64 && block != 128) || steps_per_launch < 1) return RGPU_ERR_ARG;
    e->block = block;
    e->steps_per_launch = steps_per_launch;
    return RGPU_OK;
}

int rgpu_ensemble_set_mapping(rgpu_ensemble* e, int mapping) {
    if (!e || (mapping != RGPU_ENSEMBLE_THREAD && mapping != RGPU_ENSEMBLE_WARP)) return RGPU_ERR_ARG;
    if (mapping == RGPU_ENSEMBLE_WARP && (e->exact || e->dh))
        return ens_err(e, RGPU_ERR_UNSUPPORTED, "the warp-per-system mapping runs the FMA flavour (Jacobi) only");
    e->mapping = mapping;
    return RGPU_OK;
}

int rgpu_ensemble_get_launch(const rgpu_ensemble* e, int* mapping, int* block, int64_t* steps_per_launch) {
    if (!e || !mapping || !block || !steps_per_launch) return RGPU_ERR_ARG;
    *mapping = e->mapping;
    *block = e->block;
    *steps_per_launch = e->steps_per_launch;
    return RGPU_OK;
}

int rgpu_ensemble_steps(rgpu_ensemble* e, int64_t n) {
    if (!e || n < 0) return RGPU_ERR_ARG;
    RGPU_TRY(run_steps(e, n));
    return read_status(e);
}

int rgpu_ensemble_time_steps(rgpu_ensemble* e, int64_t n, double* ms) {
    if (!e || !ms || n < 0) return RGPU_ERR_ARG;
    ENS_CUDA(e, cudaEventRecord(e->e0, e->stream));
    RGPU_TRY(run_steps(e, n));
    ENS_CUDA(e, cudaEventRecord(e->e1, e->stream));
    ENS_CUDA(e, cudaEventSynchronize(e->e1));
    float f = 0.f;
    ENS_CUDA(e, cudaEventElapsedTime(&f, e->e0, e->e1));
    *ms = f;
    return read_status(e);
}

// Autotuner, on the live ensemble (the probed steps advance the state: callers
// that need the initial state tune a scratch copy of the same systems).
// 1. mapping and CTA size: thread per system at 32 / 64 / 128 threads per CTA,
//    and warp per system (FMA flavour only), each timed over `probe_steps` steps
//    after one untimed run (graph build);
// 2. steps per launch for the winner: `max_steps_per_launch` / 256, / 64, / 16, / 4
//    and itself (at least 1), each timed over max_steps_per_launch steps; the fastest
//    wins, the smaller value on a tie within 2 %.  Shorter chunks rebalance the
//    persistent queue more often: a warp slowed by one hard system (many Kepler
//    iterations near a close encounter) holds up the end of each launch.
int rgpu_ensemble_autotune(rgpu_ensemble* e, int64_t probe_steps, int64_t max_steps_per_launch,
                           int* best_block, double* best_ms_per_step) {
    if (!e || probe_steps < 1 || max_steps_per_launch < 1) return RGPU_ERR_ARG;
    struct Choice { int mapping, block; };
    std::vector<Choice> cands = {{RGPU_ENSEMBLE_THREAD, 32}, {RGPU_ENSEMBLE_THREAD, 64}, {RGPU_ENSEMBLE_THREAD, 128}};
    if (!e->exact && !e->dh) cands.push_back({RGPU_ENSEMBLE_WARP, 128});
    double best = 1e300;
    Choice bc = {e->mapping, e->block};
    for (const Choice& c : cands) {
        e->mapping = c.mapping;
        e->block = c.block;
        e->steps_per_launch = probe_steps;
        double ms = 0.;
        RGPU_TRY(rgpu_ensemble_time_steps(e, probe_steps, &ms));   // includes graph build
        RGPU_TRY(rgpu_ensemble_time_steps(e, probe_steps, &ms));
        if (ms < best) { best = ms; bc = c; }
    }
    e->mapping = bc.mapping;
    e->block = bc.block;
    const int64_t spls[5] = {std::max<int64_t>(1, max_steps_per_launch / 256),
                             std::max<int64_t>(1, max_steps_per_launch / 64),
                             std::max<int64_t>(1, max_steps_per_launch / 16),
                             std::max<int64_t>(1, max_steps_per_launch / 4), max_steps_per_launch};
    double best_spl_ms = 1e300;
    int64_t bspl = max_steps_per_launch;
    for (int k = 0; k < 5; k++) {
        if (k > 0 && spls[k] == spls[k - 1]) continue;
        e->steps_per_launch = spls[k];
        double ms = 0.;
        RGPU_TRY(rgpu_ensemble_time_steps(e, spls[k], &ms));       // graph build
        RGPU_TRY(rgpu_ensemble_time_steps(e, max_steps_per_launch, &ms));
        if (ms < best_spl_ms * 0.98) { best_spl_ms = ms; bspl = spls[k]; }
    }
    e->steps_per_launch = bspl;
    if (best_block) *best_block = bc.block;
    if (best_ms_per_step) *best_ms_per_step = best_spl_ms / (double)max_steps_per_launch;
    return RGPU_OK;
}

int rgpu_ensemble_get_particles(rgpu_ensemble* e, void* particles, size_t stride) {
    if (!e || !particles || stride < 88) return RGPU_ERR_ARG;
    ENS_CUDA(e, cudaStreamSynchronize(e->stream));
    char* base = (char*)particles;
    for (auto& B : e->b) {
        const size_t nf = (size_t)B.nb * B.count;
        std::vector<double> h(7 * nf);
        ENS_CUDA(e, cudaMemcpy(h.data(), B.st, sizeof(double) * 7 * nf, cudaMemcpyDeviceToHost));
        for (int q = 0; q < B.count; q++) {
            const int s = B.ids[q];
            for (int i = 0; i < B.nb; i++) {
                double* r = (double*)(base + (size_t)(e->offsets[s] + i) * stride);
                const size_t o = (size_t)i * B.count + q;
                r[0] = h[0 * nf + o]; r[1] = h[1 * nf + o]; r[2] = h[2 * nf + o];
                r[3] = h[3 * nf + o]; r[4] = h[4 * nf + o]; r[5] = h[5 * nf + o];
                r[9] = h[6 * nf + o];
            }
        }
    }
    return RGPU_OK;
}

int rgpu_ensemble_energy(rgpu_ensemble* e, double* energies) {
    if (!e || !energies) return RGPU_ERR_ARG;
    for (auto& B : e->b) {
        double* d = nullptr;
        ENS_CUDA(e, cudaMalloc(&d, sizeof(double) * B.count));
        EnergyFn f = energy_fn(e, B.nb);
        f<<<(B.count + 127) / 128, 128, 0, e->stream>>>(B.st, B.count, e->G, d);
        g_launches++;
        std::vector<double> h(B.count);
        const cudaError_t ce = cudaMemcpyAsync(h.data(), d, sizeof(double) * B.count, cudaMemcpyDeviceToHost, e->stream);
        cudaStreamSynchronize(e->stream);
        cudaFree(d);
        ENS_CUDA(e, ce);
        for (int q = 0; q < B.count; q++) energies[B.ids[q]] = h[q];
    }
    return RGPU_OK;
}

int rgpu_ensemble_times(rgpu_ensemble* e, double* t) {
    if (!e || !t) return RGPU_ERR_ARG;
    for (auto& B : e->b) {
        std::vector<double> h(B.count);
        ENS_CUDA(e, cudaMemcpy(h.data(), B.t, sizeof(double) * B.count, cudaMemcpyDeviceToHost));
        for (int q = 0; q < B.count; q++) t[B.ids[q]] = h[q];
    }
    return RGPU_OK;
}

}  // extern "C"
