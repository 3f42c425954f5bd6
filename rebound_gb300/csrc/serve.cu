// Serving engine: a C++ request loop that accepts integrate-to-time requests for
// systems of different sizes as they arrive, keeps each system's state on the
// device between requests' steps, admits work against an HBM budget, and packs
// everything resident into batched kernels (continuous batching: a request that
// arrives while others run joins the next tick).
//
// Two request kinds (the reference runs each as one reb_simulation):
//  * WHFast planetary systems (src/integrator_whfast.c, Jacobi, safe_mode 1):
//    slots in per-body-count buckets, warp per slot (thread per slot on
//    request); each tick, every live warp steps its slot until a device-time
//    budget (tick_ns) has passed, so a tick lasts about the budget and no light
//    system waits for the heaviest one (or, with tick_ns = 0, chunk steps
//    extended to a block end; on the thread path min(chunk, remaining) steps).
//    Warp slots merge the drifts of consecutive steps within 32-step blocks
//    (safe_mode 0 inside a block, synchronised at its end); FMA contraction and
//    the FP64-refined division and square root (WH_FAST_MATH);
//  * Plummer clusters with leapfrog (src/integrator_leapfrog.c) and the
//    mixed-precision direct sum (FP64 displacement formed from two-float
//    splits, FP32 force, compensated FP32 accumulation): particles in a pooled
//    SoA, one CTA per (cluster, 256-particle tile), each thread summing its
//    cluster's j-range in a fixed order.
// Per-request results do not depend on which other requests share a tick, nor on
// how a request's steps fall into ticks.
#define WH_FAST_MATH 1          // approximate-then-refined FP64 division and sqrt (whfast_core.cuh)
#include "whfast_warp.cuh"
#include <algorithm>
#include <cstdint>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

using Clock = std::chrono::steady_clock;
constexpr int kT = 256;

// ---------------------------------------------------------------- kernels
template <int NB>
__global__ void __launch_bounds__(128) wh_slots_kernel(double* __restrict__ st, const double* __restrict__ dt,
                                                       int64_t* __restrict__ remaining, int cap, int chunk,
                                                       double G, uint32_t* status) {
    const int sid = blockIdx.x * blockDim.x + threadIdx.x;
    if (sid >= cap) return;
    const int64_t rem = remaining[sid];
    if (rem <= 0) return;
    const int n = (int)(rem < chunk ? rem : chunk);
    const size_t f = (size_t)NB * cap;
    wh::System<NB> s;
#pragma unroll
    for (int i = 0; i < NB; i++) {
        const size_t o = (size_t)i * cap + sid;
        s.x[i] = st[0 * f + o]; s.y[i] = st[1 * f + o]; s.z[i] = st[2 * f + o];
        s.vx[i] = st[3 * f + o]; s.vy[i] = st[4 * f + o]; s.vz[i] = st[5 * f + o];
        s.m[i] = st[6 * f + o];
    }
    const double h = dt[sid];
    for (int k = 0; k < n; k++) wh::step_safe<NB>(s, G, 0.0, h, NB, NB, 0, status);
#pragma unroll
    for (int i = 0; i < NB; i++) {
        const size_t o = (size_t)i * cap + sid;
        st[0 * f + o] = s.x[i]; st[1 * f + o] = s.y[i]; st[2 * f + o] = s.z[i];
        st[3 * f + o] = s.vx[i]; st[4 * f + o] = s.vy[i]; st[5 * f + o] = s.vz[i];
    }
    remaining[sid] = rem - n;
}

// --- warp per system (whfast_warp.cuh) -------------------------------------------
// A request's steps run in blocks of kServeBlock steps, counted from its last step
// back (the first block takes the remainder): within a block the drifts of
// consecutive steps merge as with the reference's safe_mode = 0, and each block ends
// synchronised.  A slot stops only at a block end or at the request's end, so the
// blocks, and the results, depend on the request alone, not on ticks or budgets.
constexpr int kServeBlock = 32;

// Advance WHFast slot `sid` of one bucket by `chunk` steps extended to the next
// block end, and with budget_ns > 0 only for about that much device time; called by
// a whole warp.
template <int NB>
__device__ __noinline__ void warp_advance(double* __restrict__ st, const double* __restrict__ dt,
                                          int64_t* __restrict__ remaining, int cap, int sid, int chunk, double G,
                                          long long budget_ns, uint32_t* status) {
    const int lane = (int)(threadIdx.x & 31);
    const int64_t rem = remaining[sid];
    if (rem <= 0) return;
    int64_t n = rem < chunk ? rem : chunk;
    if (n < rem) {
        n = rem - (rem - n) / kServeBlock * kServeBlock;     // extend to a block end
        if (n > INT32_MAX) n -= kServeBlock;                  // still a block end
    }
    const int first = (int)(rem % kServeBlock);
    const int done = whw::warp_steps<NB>(st, cap, sid, (int)n, dt[sid], G, status, budget_ns, kServeBlock, first);
    if (lane == 0) remaining[sid] = rem - done;
}

// One launch per tick over the live slots of every bucket: a unit is up to four
// consecutive slots of one bucket, one block of four warps.  (Per-bucket launches
// on concurrent streams stacked their few blocks on the same SMs.)
struct WarpUnit {
    double* st;
    const double* dt;
    int64_t* remaining;
    int cap, nb, slot0, nslots;
};

__global__ void __launch_bounds__(128) wh_warp_units(const WarpUnit* __restrict__ units, int chunk, double G,
                                                     long long budget_ns, uint32_t* status) {
    const WarpUnit U = units[blockIdx.x];
    const int w = (int)(threadIdx.x >> 5);
    if (w >= U.nslots) return;                       // whole warps exit together
    const int sid = U.slot0 + w;
    switch (U.nb) {
        case 2: warp_advance<2>(U.st, U.dt, U.remaining, U.cap, sid, chunk, G, budget_ns, status); break;
        case 3: warp_advance<3>(U.st, U.dt, U.remaining, U.cap, sid, chunk, G, budget_ns, status); break;
        case 4: warp_advance<4>(U.st, U.dt, U.remaining, U.cap, sid, chunk, G, budget_ns, status); break;
        case 5: warp_advance<5>(U.st, U.dt, U.remaining, U.cap, sid, chunk, G, budget_ns, status); break;
        case 6: warp_advance<6>(U.st, U.dt, U.remaining, U.cap, sid, chunk, G, budget_ns, status); break;
        case 7: warp_advance<7>(U.st, U.dt, U.remaining, U.cap, sid, chunk, G, budget_ns, status); break;
        case 8: warp_advance<8>(U.st, U.dt, U.remaining, U.cap, sid, chunk, G, budget_ns, status); break;
        case 9: warp_advance<9>(U.st, U.dt, U.remaining, U.cap, sid, chunk, G, budget_ns, status); break;
        case 10: warp_advance<10>(U.st, U.dt, U.remaining, U.cap, sid, chunk, G, budget_ns, status); break;
        case 11: warp_advance<11>(U.st, U.dt, U.remaining, U.cap, sid, chunk, G, budget_ns, status); break;
        case 12: warp_advance<12>(U.st, U.dt, U.remaining, U.cap, sid, chunk, G, budget_ns, status); break;
        case 13: warp_advance<13>(U.st, U.dt, U.remaining, U.cap, sid, chunk, G, budget_ns, status); break;
        case 14: warp_advance<14>(U.st, U.dt, U.remaining, U.cap, sid, chunk, G, budget_ns, status); break;
        case 15: warp_advance<15>(U.st, U.dt, U.remaining, U.cap, sid, chunk, G, budget_ns, status); break;
        default: warp_advance<16>(U.st, U.dt, U.remaining, U.cap, sid, chunk, G, budget_ns, status); break;
    }
}

typedef void (*WhSlotsFn)(double*, const double*, int64_t*, int, int, double, uint32_t*);

WhSlotsFn wh_slots_for(int nb) {
    switch (nb) {
        case 2: return wh_slots_kernel<2>; case 3: return wh_slots_kernel<3>; case 4: return wh_slots_kernel<4>;
        case 5: return wh_slots_kernel<5>; case 6: return wh_slots_kernel<6>; case 7: return wh_slots_kernel<7>;
        case 8: return wh_slots_kernel<8>; case 9: return wh_slots_kernel<9>; case 10: return wh_slots_kernel<10>;
        case 11: return wh_slots_kernel<11>; case 12: return wh_slots_kernel<12>; case 13: return wh_slots_kernel<13>;
        case 14: return wh_slots_kernel<14>; case 15: return wh_slots_kernel<15>; case 16: return wh_slots_kernel<16>;
        default: return nullptr;
    }
}

// Admission / retirement of WHFast slots in one batched copy per tick.
struct SlotRec {
    double* st;                 // bucket state base
    double* dt;
    int64_t* remaining;
    int cap, nb, slot, pad;
    double v[7 * wh::kMaxBodies];   // x, y, z, vx, vy, vz, m per body (field-major)
    double h;
    int64_t steps;
};

__global__ void slots_admit(const SlotRec* __restrict__ recs, int n) {
    const int k = blockIdx.x;
    if (k >= n) return;
    const SlotRec& r = recs[k];
    const size_t f = (size_t)r.nb * r.cap;
    for (int t = threadIdx.x; t < 7 * r.nb; t += blockDim.x) {
        const int field = t / r.nb, body = t % r.nb;
        r.st[field * f + (size_t)body * r.cap + r.slot] = r.v[field * wh::kMaxBodies + body];
    }
    if (threadIdx.x == 0) { r.dt[r.slot] = r.h; r.remaining[r.slot] = r.steps; }
}

__global__ void slots_gather(SlotRec* __restrict__ recs, int n) {
    const int k = blockIdx.x;
    if (k >= n) return;
    SlotRec& r = recs[k];
    const size_t f = (size_t)r.nb * r.cap;
    for (int t = threadIdx.x; t < 6 * r.nb; t += blockDim.x) {
        const int field = t / r.nb, body = t % r.nb;
        r.v[field * wh::kMaxBodies + body] = r.st[field * f + (size_t)body * r.cap + r.slot];
    }
}

struct ClusterItem {      // one resident cluster in this tick
    int off, n;           // range in the particle pool
    int steps_now;        // steps to run this tick
    double dt, eps2, G;
};

// Pool: SoA x, y, z, vx, vy, vz, ax, ay, az, m (10 arrays of `cap`) + split (2 float4 per particle).
struct Pool {
    double *x, *y, *z, *vx, *vy, *vz, *ax, *ay, *az, *m;
    float4* split;
};

__global__ void cl_drift(Pool p, const ClusterItem* __restrict__ items, int k, double frac) {
    const ClusterItem it = items[blockIdx.y];
    const int i = blockIdx.x * kT + threadIdx.x;
    if (k >= it.steps_now || i >= it.n) return;
    const int q = it.off + i;
    const double h = it.dt * frac;
    p.x[q] += h * p.vx[q]; p.y[q] += h * p.vy[q]; p.z[q] += h * p.vz[q];
}

__global__ void cl_split(Pool p, const ClusterItem* __restrict__ items, int k) {
    const ClusterItem it = items[blockIdx.y];
    const int i = blockIdx.x * kT + threadIdx.x;
    if (k >= it.steps_now || i >= it.n) return;
    const int q = it.off + i;
    const double x = p.x[q], y = p.y[q], z = p.z[q];
    const float xh = (float)x, yh = (float)y, zh = (float)z;
    p.split[2 * q] = make_float4(xh, yh, zh, (float)(it.G * p.m[q]));
    p.split[2 * q + 1] = make_float4((float)(x - (double)xh), (float)(y - (double)yh), (float)(z - (double)zh), 0.f);
}

// Mixed-precision force of one cluster tile (the MIXED_SPLIT form of the direct
// sum): two-float displacements and FP32 G m / r^3 on the packed FP32x2 pipe, two
// j-bodies per instruction, FP32 sums over 32 j-pairs folded into a compensated
// FP32 pair per particle.  The tile is repacked in shared memory so one 64-bit
// register holds the same field of two bodies.
struct __align__(16) ClPair {
    float4 a, b, c, d;     // (xh0, xh1, yh0, yh1), (zh0, zh1, m0, m1), (xl0, xl1, yl0, yl1), (zl0, zl1, -, -)
};

__global__ void __launch_bounds__(kT) cl_force(Pool p, const ClusterItem* __restrict__ items, int k) {
    __shared__ ClPair tile[kT / 2];
    const ClusterItem it = items[blockIdx.y];
    if (k >= it.steps_now || blockIdx.x * kT >= it.n) return;
    const int i = blockIdx.x * kT + threadIdx.x;
    const bool live = i < it.n;
    float4 hi = make_float4(0.f, 0.f, 0.f, 0.f), lo = hi;
    if (live) { hi = p.split[2 * (it.off + i)]; lo = p.split[2 * (it.off + i) + 1]; }
    const float2 nxh = make_float2(-hi.x, -hi.x), nyh = make_float2(-hi.y, -hi.y), nzh = make_float2(-hi.z, -hi.z);
    const float2 nxl = make_float2(-lo.x, -lo.x), nyl = make_float2(-lo.y, -lo.y), nzl = make_float2(-lo.z, -lo.z);
    const float e = (float)it.eps2;
    const float2 e2 = make_float2(e, e);
    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    for (int jt = 0; jt < it.n; jt += kT) {
        __syncthreads();
        {
            const int jl = jt + threadIdx.x;
            float4 h = make_float4(0.f, 0.f, 0.f, 0.f), l = h;   // missing partner: massless, far from i below
            if (jl < it.n) { h = p.split[2 * (it.off + jl)]; l = p.split[2 * (it.off + jl) + 1]; }
            float* t = reinterpret_cast<float*>(&tile[threadIdx.x >> 1]);
            const int q = threadIdx.x & 1;
            t[0 + q] = h.x; t[2 + q] = h.y; t[4 + q] = h.z; t[6 + q] = h.w;
            t[8 + q] = l.x; t[10 + q] = l.y; t[12 + q] = l.z;
        }
        __syncthreads();
        const int nj = min(kT, it.n - jt);
        const int nq = (nj + 1) >> 1;
        for (int qs = 0; qs < nq; qs += 32) {
            const int qe = min(nq, qs + 32);
            float2 ax = make_float2(0.f, 0.f), ay = ax, az = ax;
#pragma unroll 4
            for (int q = qs; q < qe; q++) {
                const ClPair J = tile[q];
                const float2 dx = __fadd2_rn(__fadd2_rn(make_float2(J.a.x, J.a.y), nxh),
                                             __fadd2_rn(make_float2(J.c.x, J.c.y), nxl));
                const float2 dy = __fadd2_rn(__fadd2_rn(make_float2(J.a.z, J.a.w), nyh),
                                             __fadd2_rn(make_float2(J.c.z, J.c.w), nyl));
                const float2 dz = __fadd2_rn(__fadd2_rn(make_float2(J.b.x, J.b.y), nzh),
                                             __fadd2_rn(make_float2(J.d.x, J.d.y), nzl));
                const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __ffma2_rn(dz, dz, e2)));
                const float2 ri = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
                float2 sv = __fmul2_rn(__fmul2_rn(ri, ri), __fmul2_rn(make_float2(J.b.z, J.b.w), ri));
                const int j = jt + 2 * q;
                sv.x = (j == i) ? 0.f : sv.x;                           // self pair (and eps = 0)
                sv.y = (j + 1 == i || j + 1 >= jt + nj) ? 0.f : sv.y;   // and the missing partner
                ax = __ffma2_rn(sv, dx, ax);
                ay = __ffma2_rn(sv, dy, ay);
                az = __ffma2_rn(sv, dz, az);
            }
            const float tx = ax.x + ax.y, ty = ay.x + ay.y, tz = az.x + az.y;
            float t, y;
            y = tx - cx; t = sx + y; cx = (t - sx) - y; sx = t;
            y = ty - cy; t = sy + y; cy = (t - sy) - y; sy = t;
            y = tz - cz; t = sz + y; cz = (t - sz) - y; sz = t;
        }
    }
    if (!live) return;
    const int q = it.off + i;
    p.ax[q] = (double)sx - (double)cx; p.ay[q] = (double)sy - (double)cy; p.az[q] = (double)sz - (double)cz;
}

__global__ void cl_kick_drift(Pool p, const ClusterItem* __restrict__ items, int k) {
    const ClusterItem it = items[blockIdx.y];
    const int i = blockIdx.x * kT + threadIdx.x;
    if (k >= it.steps_now || i >= it.n) return;
    const int q = it.off + i;
    const double vx = p.vx[q] + it.dt * p.ax[q], vy = p.vy[q] + it.dt * p.ay[q], vz = p.vz[q] + it.dt * p.az[q];
    p.vx[q] = vx; p.vy[q] = vy; p.vz[q] = vz;
    const double h = it.dt * 0.5;
    p.x[q] += h * vx; p.y[q] += h * vy; p.z[q] += h * vz;
}

// ---------------------------------------------------------------- host state
struct Request {
    int64_t id;
    int kind;                       // RGPU_SERVE_WHFAST or RGPU_SERVE_CLUSTER
    std::vector<double> rec;        // n * 11 doubles (x..r), the AoS payload
    int n;
    double dt, G, softening;
    int64_t steps;
    size_t bytes;                   // device footprint for admission
    Clock::time_point submitted, admitted, finished;
    bool done = false;
    int status = RGPU_OK;
    // residency
    int bucket = -1, slot = -1;     // WHFast
    int pool_off = -1;              // cluster
    int64_t remaining = 0;
};

struct WhBucket {
    int nb = 0, cap = 0, live = 0;
    int hw = 0;                     // slots in [hw, cap) have never been used
    double* st = nullptr;           // 7 * nb * cap
    double* dt = nullptr;
    int64_t* remaining = nullptr;
    std::vector<int64_t> owner;     // request id per slot, -1 free
    std::vector<int> free_slots;
    std::vector<int64_t> rem_host;  // remaining steps, copied back each tick
};

}  // namespace

struct rgpu_server {
    rgpu_server_config cfg{};
    uint32_t* d_status = nullptr;
    std::map<int, WhBucket> buckets;
    // cluster pool
    Pool pool{};
    int pool_cap = 0;
    std::map<int, int> pool_free;   // offset -> length (free ranges)
    ClusterItem* d_items = nullptr;
    int items_cap = 0;
    SlotRec* d_slots = nullptr;     // staging for slot admission / retirement
    int slots_cap = 0;
    std::vector<SlotRec> pending_admit;
    // requests
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<int64_t> waiting[3];       // per kind (1 WHFast, 2 cluster)
    std::unordered_map<int64_t, Request> req;
    std::vector<int64_t> resident[3];
    cudaStream_t kstream[3] = {nullptr, nullptr, nullptr};
    // one stream per WHFast body count, so the buckets of a tick run side by side
    // (a tick then lasts as long as its slowest bucket, not the sum of them)
    cudaStream_t bstream[wh::kMaxBodies + 1] = {};
    WarpUnit* d_units = nullptr;     // per-tick unit table of the warp-per-system kernel
    int units_cap = 0;
    std::vector<WarpUnit> units;
    int64_t next_id = 1;
    size_t bytes_in_use = 0;
    bool stop = false;
    std::thread worker[3];
    // stats
    int64_t completed = 0;
    double system_steps = 0, pair_interactions = 0;
    int64_t ticks = 0;
    std::string msg;
};

namespace {

size_t wh_bytes(int n) { return (size_t)n * 7 * 8 + 16; }
size_t cluster_bytes(int n) { return (size_t)n * (10 * 8 + 32); }

int pool_alloc(rgpu_server* s, int n) {
    for (auto it = s->pool_free.begin(); it != s->pool_free.end(); ++it) {
        if (it->second >= n) {
            const int off = it->first, len = it->second;
            s->pool_free.erase(it);
            if (len > n) s->pool_free[off + n] = len - n;
            return off;
        }
    }
    return -1;
}

void pool_release(rgpu_server* s, int off, int n) {
    auto it = s->pool_free.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != s->pool_free.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        s->pool_free.erase(nx);
    }
    if (it != s->pool_free.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            s->pool_free.erase(it);
        }
    }
}

int ensure_bucket(rgpu_server* s, int nb) {
    WhBucket& B = s->buckets[nb];
    if (B.cap) return RGPU_OK;
    B.nb = nb;
    B.cap = s->cfg.slots_per_bucket;
    if (cudaMalloc(&B.st, sizeof(double) * 7 * nb * (size_t)B.cap) != cudaSuccess ||
        cudaMalloc(&B.dt, sizeof(double) * B.cap) != cudaSuccess ||
        cudaMalloc(&B.remaining, sizeof(int64_t) * B.cap) != cudaSuccess) {
        cudaGetLastError();
        B.cap = 0;
        return RGPU_ERR_NOMEM;
    }
    cudaMemset(B.remaining, 0, sizeof(int64_t) * B.cap);
    B.owner.assign(B.cap, -1);
    B.free_slots.clear();
    for (int q = B.cap - 1; q >= 0; q--) B.free_slots.push_back(q);
    return RGPU_OK;
}

// Stage a WHFast request into a free slot (lock held; the copy happens in the
// worker's next batched admission).
int admit_whfast(rgpu_server* s, Request& r) {
    const int n = r.n;
    if (ensure_bucket(s, n)) return RGPU_ERR_NOMEM;
    WhBucket& B = s->buckets[n];
    if (B.free_slots.empty()) return RGPU_ERR_CAPACITY;
    const int q = B.free_slots.back();
    B.free_slots.pop_back();
    B.owner[q] = r.id;
    B.live++;
    B.hw = std::max(B.hw, q + 1);
    r.bucket = n;
    r.slot = q;
    r.remaining = r.steps;
    SlotRec rec{};
    rec.st = B.st; rec.dt = B.dt; rec.remaining = B.remaining;
    rec.cap = B.cap; rec.nb = n; rec.slot = q;
    const int map[7] = {0, 1, 2, 3, 4, 5, 9};
    for (int i = 0; i < n; i++)
        for (int k = 0; k < 7; k++) rec.v[k * wh::kMaxBodies + i] = r.rec[(size_t)i * 11 + map[k]];
    rec.h = r.dt;
    rec.steps = r.steps;
    s->pending_admit.push_back(rec);
    return RGPU_OK;
}

int stage_slots(rgpu_server* s, const std::vector<SlotRec>& recs, cudaStream_t st) {
    if ((int)recs.size() > s->slots_cap) {
        cudaFree(s->d_slots);
        s->d_slots = nullptr;
        s->slots_cap = 0;
        if (cudaMalloc(&s->d_slots, sizeof(SlotRec) * recs.size() * 2) != cudaSuccess) { cudaGetLastError(); return RGPU_ERR_NOMEM; }
        s->slots_cap = (int)recs.size() * 2;
    }
    cudaMemcpyAsync(s->d_slots, recs.data(), sizeof(SlotRec) * recs.size(), cudaMemcpyHostToDevice, st);
    return RGPU_OK;
}

void finish(rgpu_server* s, Request& r) {
    r.done = true;
    r.finished = Clock::now();
    s->completed++;
    s->bytes_in_use -= r.bytes;
}

// WHFast worker: batched admission, one chunk of steps per live slot per tick,
// batched retirement.
void whfast_worker(rgpu_server* s) {
    cudaStream_t st = s->kstream[RGPU_SERVE_WHFAST];
    std::unique_lock<std::mutex> lk(s->mu);
    std::vector<int64_t>& resident = s->resident[RGPU_SERVE_WHFAST];
    std::deque<int64_t>& waiting = s->waiting[RGPU_SERVE_WHFAST];
    while (!s->stop) {
        while (!waiting.empty()) {
            Request& r = s->req[waiting.front()];
            if (s->bytes_in_use + r.bytes > s->cfg.hbm_budget_bytes) break;
            const int rc = admit_whfast(s, r);
            if (rc == RGPU_ERR_CAPACITY) break;
            waiting.pop_front();
            if (rc) { r.status = rc; r.done = true; r.finished = Clock::now(); continue; }
            s->bytes_in_use += r.bytes;
            r.admitted = Clock::now();
            resident.push_back(r.id);
        }
        if (!s->pending_admit.empty()) {
            std::vector<SlotRec> batch;
            batch.swap(s->pending_admit);
            if (stage_slots(s, batch, st) == RGPU_OK) {
                slots_admit<<<(unsigned)batch.size(), 128, 0, st>>>(s->d_slots, (int)batch.size());
                g_launches++;
                cudaStreamSynchronize(st);   // batch is host memory
            }
        }
        if (resident.empty()) {
            s->cv_done.notify_all();
            s->cv_work.wait_for(lk, std::chrono::milliseconds(20));
            continue;
        }
        // fixed chunk, or (warp per system, tick_ns > 0) a device-time budget per slot
        const bool sliced = !s->cfg.thread_per_system && s->cfg.tick_ns > 0;
        const int chunk = sliced ? INT32_MAX : (int)s->cfg.steps_per_launch;
        std::vector<WhBucket*> live;
        for (auto& kv : s->buckets) if (kv.second.cap && kv.second.live) live.push_back(&kv.second);
        lk.unlock();
        if (s->cfg.thread_per_system) {
            for (WhBucket* B : live) {
                cudaStream_t bs = s->bstream[B->nb];
                wh_slots_for(B->nb)<<<(B->hw + 127) / 128, 128, 0, bs>>>(B->st, B->dt, B->remaining, B->cap, chunk,
                                                                         1.0, s->d_status);
                g_launches++;
                B->rem_host.resize(B->cap);
                cudaMemcpyAsync(B->rem_host.data(), B->remaining, sizeof(int64_t) * B->hw, cudaMemcpyDeviceToHost, bs);
            }
            for (WhBucket* B : live) cudaStreamSynchronize(s->bstream[B->nb]);
        } else {
            s->units.clear();
            for (WhBucket* B : live)
                for (int q0 = 0; q0 < B->hw; q0 += 4)
                    s->units.push_back(WarpUnit{B->st, B->dt, B->remaining, B->cap, B->nb, q0, std::min(4, B->hw - q0)});
            const int nu = (int)s->units.size();
            if (nu > s->units_cap) {
                cudaFree(s->d_units);
                s->d_units = nullptr;
                s->units_cap = 0;
                if (cudaMalloc(&s->d_units, sizeof(WarpUnit) * (size_t)nu * 2) == cudaSuccess) s->units_cap = nu * 2;
                else cudaGetLastError();
            }
            if (nu && nu <= s->units_cap) {
                cudaMemcpyAsync(s->d_units, s->units.data(), sizeof(WarpUnit) * nu, cudaMemcpyHostToDevice, st);
                wh_warp_units<<<nu, 128, 0, st>>>(s->d_units, chunk, 1.0, (long long)s->cfg.tick_ns, s->d_status);
                g_launches++;
            }
            for (WhBucket* B : live) {
                B->rem_host.resize(B->cap);
                cudaMemcpyAsync(B->rem_host.data(), B->remaining, sizeof(int64_t) * B->hw, cudaMemcpyDeviceToHost, st);
            }
            cudaStreamSynchronize(st);
        }
        lk.lock();
        s->ticks++;
        std::vector<int64_t> still, fin;
        std::vector<SlotRec> gather;
        for (int64_t id : resident) {
            Request& r = s->req[id];
            WhBucket& B = s->buckets[r.bucket];
            const int64_t rem = B.rem_host[r.slot];
            s->system_steps += (double)(r.remaining - rem);
            r.remaining = rem;
            if (rem <= 0) {
                SlotRec g{};
                g.st = B.st; g.cap = B.cap; g.nb = B.nb; g.slot = r.slot;
                gather.push_back(g);
                fin.push_back(id);
            } else {
                still.push_back(id);
            }
        }
        resident.swap(still);
        if (!gather.empty() && stage_slots(s, gather, st) == RGPU_OK) {
            slots_gather<<<(unsigned)gather.size(), 128, 0, st>>>(s->d_slots, (int)gather.size());
            g_launches++;
            cudaMemcpyAsync(gather.data(), s->d_slots, sizeof(SlotRec) * gather.size(), cudaMemcpyDeviceToHost, st);
            cudaStreamSynchronize(st);
            for (size_t q = 0; q < gather.size(); q++) {
                Request& r = s->req[fin[q]];
                for (int i = 0; i < r.n; i++)
                    for (int k = 0; k < 6; k++) r.rec[(size_t)i * 11 + k] = gather[q].v[k * wh::kMaxBodies + i];
                WhBucket& B = s->buckets[r.bucket];
                B.owner[r.slot] = -1;
                B.free_slots.push_back(r.slot);
                B.live--;
                finish(s, r);
            }
        }
        uint32_t flag = 0;
        cudaMemcpy(&flag, s->d_status, 4, cudaMemcpyDeviceToHost);
        if (flag) { s->msg = "Kepler solver hit its iteration cap"; cudaMemset(s->d_status, 0, 4); }
        s->cv_done.notify_all();
    }
}

// Cluster worker: pooled particles, cluster_steps_per_tick leapfrog steps per tick.
void cluster_worker(rgpu_server* s) {
    cudaStream_t st = s->kstream[RGPU_SERVE_CLUSTER];
    std::unique_lock<std::mutex> lk(s->mu);
    std::vector<int64_t>& resident = s->resident[RGPU_SERVE_CLUSTER];
    std::deque<int64_t>& waiting = s->waiting[RGPU_SERVE_CLUSTER];
    std::vector<ClusterItem> items;
    std::vector<double> col;
    double* fields[10] = {s->pool.x, s->pool.y, s->pool.z, s->pool.vx, s->pool.vy, s->pool.vz,
                          s->pool.ax, s->pool.ay, s->pool.az, s->pool.m};
    while (!s->stop) {
        std::vector<int64_t> admitted;
        while (!waiting.empty()) {
            Request& r = s->req[waiting.front()];
            if (s->bytes_in_use + r.bytes > s->cfg.hbm_budget_bytes) break;
            const int off = pool_alloc(s, r.n);
            if (off < 0) break;
            waiting.pop_front();
            r.pool_off = off;
            r.remaining = r.steps;
            s->bytes_in_use += r.bytes;
            admitted.push_back(r.id);
        }
        if (!admitted.empty()) {
            // copy payloads outside the lock (the records are owned by the worker until done)
            std::vector<Request*> rs;
            for (int64_t id : admitted) rs.push_back(&s->req[id]);
            lk.unlock();
            for (Request* r : rs) {
                col.resize((size_t)r->n);
                for (int k = 0; k < 10; k++) {
                    for (int i = 0; i < r->n; i++) col[i] = r->rec[(size_t)i * 11 + k];
                    cudaMemcpyAsync(fields[k] + r->pool_off, col.data(), 8 * (size_t)r->n, cudaMemcpyHostToDevice, st);
                    cudaStreamSynchronize(st);
                }
            }
            lk.lock();
            for (Request* r : rs) { r->admitted = Clock::now(); resident.push_back(r->id); }
        }
        if (resident.empty()) {
            s->cv_done.notify_all();
            s->cv_work.wait_for(lk, std::chrono::milliseconds(20));
            continue;
        }
        items.clear();
        int max_tiles = 0, max_steps = 0;
        for (int64_t id : resident) {
            Request& r = s->req[id];
            ClusterItem it;
            it.off = r.pool_off; it.n = r.n;
            it.steps_now = (int)std::min<int64_t>(r.remaining, s->cfg.cluster_steps_per_tick);
            it.dt = r.dt; it.eps2 = r.softening * r.softening; it.G = r.G;
            items.push_back(it);
            max_tiles = std::max(max_tiles, (r.n + kT - 1) / kT);
            max_steps = std::max(max_steps, it.steps_now);
        }
        const std::vector<int64_t> tick_ids = resident;
        lk.unlock();
        bool ok = true;
        if ((int)items.size() > s->items_cap) {
            cudaFree(s->d_items);
            s->d_items = nullptr;
            s->items_cap = 0;
            if (cudaMalloc(&s->d_items, sizeof(ClusterItem) * items.size() * 2) == cudaSuccess) {
                s->items_cap = (int)items.size() * 2;
            } else {
                cudaGetLastError();
                ok = false;
            }
        }
        if (ok) {
            ok = cudaMemcpyAsync(s->d_items, items.data(), sizeof(ClusterItem) * items.size(), cudaMemcpyHostToDevice,
                                 st) == cudaSuccess;
            const dim3 grid(max_tiles, (unsigned)items.size());
            for (int k = 0; ok && k < max_steps; k++) {
                cl_drift<<<grid, kT, 0, st>>>(s->pool, s->d_items, k, 0.5);
                cl_split<<<grid, kT, 0, st>>>(s->pool, s->d_items, k);
                cl_force<<<grid, kT, 0, st>>>(s->pool, s->d_items, k);
                cl_kick_drift<<<grid, kT, 0, st>>>(s->pool, s->d_items, k);
                g_launches += 4;
                ok = cudaGetLastError() == cudaSuccess;
            }
        }
        if (cudaStreamSynchronize(st) != cudaSuccess) {
            cudaGetLastError();
            ok = false;
        }
        std::vector<Request*> done_now;
        lk.lock();
        s->ticks++;
        if (!ok) {
            // the tick did not run: its requests fail with RGPU_ERR_CUDA and give back their pool range
            s->msg = "cluster tick failed (device allocation, launch or stream error)";
            std::vector<int64_t> keep;
            for (int64_t id : resident)
                if (std::find(tick_ids.begin(), tick_ids.end(), id) == tick_ids.end()) keep.push_back(id);
            resident.swap(keep);
            for (int64_t id : tick_ids) {
                Request& r = s->req[id];
                r.status = RGPU_ERR_CUDA;
                pool_release(s, r.pool_off, r.n);
                finish(s, r);
            }
            s->cv_done.notify_all();
            continue;
        }
        std::vector<int64_t> still;
        for (size_t q = 0; q < tick_ids.size(); q++) {
            Request& r = s->req[tick_ids[q]];
            r.remaining -= items[q].steps_now;
            s->pair_interactions += (double)items[q].steps_now * r.n * (double)(r.n - 1);
            s->system_steps += items[q].steps_now;
            if (r.remaining <= 0) done_now.push_back(&r); else still.push_back(r.id);
        }
        // requests admitted by this worker meanwhile stay resident
        for (int64_t id : resident)
            if (std::find(tick_ids.begin(), tick_ids.end(), id) == tick_ids.end()) still.push_back(id);
        resident.swap(still);
        lk.unlock();
        for (Request* r : done_now) {
            col.resize((size_t)r->n);
            for (int k = 0; k < 9; k++) {
                cudaMemcpyAsync(col.data(), fields[k] + r->pool_off, 8 * (size_t)r->n, cudaMemcpyDeviceToHost, st);
                cudaStreamSynchronize(st);
                for (int i = 0; i < r->n; i++) r->rec[(size_t)i * 11 + k] = col[i];
            }
        }
        lk.lock();
        for (Request* r : done_now) {
            pool_release(s, r->pool_off, r->n);
            finish(s, *r);
        }
        s->cv_done.notify_all();
    }
}

}  // namespace

extern "C" {

void rgpu_server_config_default(rgpu_server_config* c) {
    std::memset(c, 0, sizeof(*c));
    c->hbm_budget_bytes = (size_t)120 << 30;
    c->slots_per_bucket = 16384;
    c->pool_particles = 1 << 22;
    c->steps_per_launch = 64;
    c->cluster_steps_per_tick = 8;
    c->tick_ns = 8000000;
}

int rgpu_server_create(rgpu_server** out, const rgpu_server_config* cfg) {
    if (!out) return RGPU_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { cudaGetLastError(); return RGPU_ERR_CUDA; }
    rgpu_server* s = new (std::nothrow) rgpu_server();
    if (!s) return RGPU_ERR_NOMEM;
    if (cfg) s->cfg = *cfg; else rgpu_server_config_default(&s->cfg);
    if (s->cfg.slots_per_bucket < 32 || s->cfg.pool_particles < 256 || s->cfg.steps_per_launch < 1 ||
        s->cfg.steps_per_launch > INT32_MAX || s->cfg.cluster_steps_per_tick < 1 || s->cfg.tick_ns < 0 ||
        s->cfg.tick_ns > 1000000000) {   // a tick of at most 1 s keeps admission and waits responsive
        delete s;
        return RGPU_ERR_ARG;
    }
    const int P = (int)s->cfg.pool_particles;
    s->pool_cap = P;
    double** f[10] = {&s->pool.x, &s->pool.y, &s->pool.z, &s->pool.vx, &s->pool.vy, &s->pool.vz,
                      &s->pool.ax, &s->pool.ay, &s->pool.az, &s->pool.m};
    bool ok = cudaStreamCreateWithFlags(&s->kstream[RGPU_SERVE_WHFAST], cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&s->kstream[RGPU_SERVE_CLUSTER], cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&s->d_status, 4) == cudaSuccess && cudaMemset(s->d_status, 0, 4) == cudaSuccess;
    for (int nb = 2; ok && nb <= wh::kMaxBodies; nb++)
        ok = cudaStreamCreateWithFlags(&s->bstream[nb], cudaStreamNonBlocking) == cudaSuccess;
    for (int k = 0; ok && k < 10; k++) ok = cudaMalloc(f[k], sizeof(double) * P) == cudaSuccess;
    ok = ok && cudaMalloc(&s->pool.split, sizeof(float4) * 2 * (size_t)P) == cudaSuccess;
    if (!ok) { cudaGetLastError(); rgpu_server_free(s); return RGPU_ERR_NOMEM; }
    s->pool_free[0] = P;
    s->worker[RGPU_SERVE_WHFAST] = std::thread(whfast_worker, s);
    s->worker[RGPU_SERVE_CLUSTER] = std::thread(cluster_worker, s);
    *out = s;
    return RGPU_OK;
}

void rgpu_server_free(rgpu_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto& w : s->worker) if (w.joinable()) w.join();
    for (cudaStream_t st : s->kstream) if (st) cudaStreamSynchronize(st);
    for (cudaStream_t st : s->bstream) if (st) cudaStreamSynchronize(st);
    for (auto& kv : s->buckets) { cudaFree(kv.second.st); cudaFree(kv.second.dt); cudaFree(kv.second.remaining); }
    double* f[10] = {s->pool.x, s->pool.y, s->pool.z, s->pool.vx, s->pool.vy, s->pool.vz,
                     s->pool.ax, s->pool.ay, s->pool.az, s->pool.m};
    for (double* p : f) cudaFree(p);
    cudaFree(s->pool.split);
    cudaFree(s->d_items);
    cudaFree(s->d_slots);
    cudaFree(s->d_units);
    cudaFree(s->d_status);
    for (cudaStream_t st : s->kstream) if (st) cudaStreamDestroy(st);
    for (cudaStream_t st : s->bstream) if (st) cudaStreamDestroy(st);
    delete s;
}

int rgpu_server_submit(rgpu_server* s, int kind, const void* particles, size_t n, size_t stride, double dt,
                       int64_t n_steps, double G, double softening, int64_t* request_id) {
    if (!s || !particles || !request_id || stride < 88 || n_steps < 0) return RGPU_ERR_ARG;
    if (kind == RGPU_SERVE_WHFAST) {
        if (n < 2 || n > (size_t)wh::kMaxBodies) return RGPU_ERR_UNSUPPORTED;
        if (G != 1.0) return RGPU_ERR_UNSUPPORTED;          // the batched slots run with G = 1
    } else if (kind == RGPU_SERVE_CLUSTER) {
        if (n < 1 || n > (size_t)s->pool_cap) return RGPU_ERR_CAPACITY;
    } else {
        return RGPU_ERR_ARG;
    }
    Request r;
    r.kind = kind;
    r.n = (int)n;
    r.dt = dt; r.G = G; r.softening = softening; r.steps = n_steps;
    r.rec.resize(n * 11);
    for (size_t i = 0; i < n; i++)
        std::memcpy(&r.rec[i * 11], (const char*)particles + i * stride, 88);
    r.bytes = kind == RGPU_SERVE_WHFAST ? wh_bytes((int)n) : cluster_bytes((int)n);
    if (r.bytes > s->cfg.hbm_budget_bytes) return RGPU_ERR_CAPACITY;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r.id = s->next_id++;
        r.submitted = Clock::now();
        *request_id = r.id;
        s->waiting[kind].push_back(r.id);
        s->req.emplace(r.id, std::move(r));
    }
    s->cv_work.notify_all();
    return RGPU_OK;
}

int rgpu_server_wait(rgpu_server* s, int64_t id, void* particles, size_t stride, double timeout_s, double* latency_s) {
    if (!s || stride < 88) return RGPU_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->req.find(id);
    if (it == s->req.end()) return RGPU_ERR_ARG;
    const auto deadline = Clock::now() +
        std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 0.0));
    while (!it->second.done) {
        if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !it->second.done)
            return RGPU_ERR_TIMEOUT;    // still running: the caller may wait again
        it = s->req.find(id);
    }
    Request& r = it->second;
    const int status = r.status;
    if (particles)
        for (int i = 0; i < r.n; i++) std::memcpy((char*)particles + (size_t)i * stride, &r.rec[(size_t)i * 11], 88);
    if (latency_s) *latency_s = std::chrono::duration<double>(r.finished - r.submitted).count();
    s->req.erase(it);
    return status;
}

int rgpu_server_get_stats(rgpu_server* s, rgpu_server_stats* out) {
    if (!s || !out) return RGPU_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    out->completed = s->completed;
    out->waiting = (int64_t)(s->waiting[1].size() + s->waiting[2].size());
    out->resident = (int64_t)(s->resident[1].size() + s->resident[2].size());
    out->ticks = s->ticks;
    out->system_steps = s->system_steps;
    out->pair_interactions = s->pair_interactions;
    out->bytes_in_use = s->bytes_in_use;
    return RGPU_OK;
}

}  // extern "C"
