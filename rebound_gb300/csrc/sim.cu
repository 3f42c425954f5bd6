// Device-resident simulation handle and the C ABI entry points of
// librebound_gb300: lifecycle, particle upload/download, the step loop
// (src/simulation.c:500-603), the leapfrog and SEI kernels
// (src/integrator_leapfrog.c:72-107, src/integrator_sei.c:86-174) and the
// periodic/shear boundary (src/boundary.c:35-201).
//
// Compiled with --fmad=false: the per-particle update arithmetic rounds exactly
// like the reference's -ffp-contract=off build.
#include "rgpu_internal.cuh"
#include <cmath>
#include <cstring>
#include <new>

std::atomic<int64_t> g_launches{0};

int set_error(rgpu_sim* s, int code, const std::string& what) {
    if (s) s->msg = what;
    return code;
}

int check_cuda(rgpu_sim* s, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return RGPU_OK;
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return set_error(s, RGPU_ERR_NOMEM, std::string(what) + ": " + cudaGetErrorString(e));
    }
    return set_error(s, RGPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Read (and clear) the device status word; map its bits to an error code.
int read_status(rgpu_sim* s) {
    uint32_t st = 0;
    RGPU_CUDA(s, cudaMemcpyAsync(&st, s->d_status, sizeof(st), cudaMemcpyDeviceToHost, s->stream));
    RGPU_CUDA(s, cudaStreamSynchronize(s->stream));
    if (!st) return RGPU_OK;
    RGPU_CUDA(s, cudaMemsetAsync(s->d_status, 0, sizeof(uint32_t), s->stream));
    if (st & DEV_ERR_NONFINITE) return set_error(s, RGPU_ERR_NONFINITE, "Particle has non-finite coordinates. Cannot add to tree.");
    if (st & DEV_ERR_OUT_OF_BOX) return set_error(s, RGPU_ERR_OUT_OF_BOX, "Particle is outside of simulation box. Cannot add to tree.");
    if (st & DEV_ERR_DUPLICATE) return set_error(s, RGPU_ERR_DUPLICATE, "Cannot add two particles with the same coordinates to the tree.");
    if (st & DEV_ERR_TREE_DEPTH) return set_error(s, RGPU_ERR_TREE_DEPTH, "Octree deeper than the device key supports.");
    if (st & DEV_ERR_STACK) return set_error(s, RGPU_ERR_TREE_DEPTH, "Tree walk stack overflow.");
    if (st & DEV_ERR_OVERFLOW) return set_error(s, RGPU_ERR_OVERFLOW, "Device output buffer overflow.");
    if (st & DEV_ERR_KEPLER) return set_error(s, RGPU_ERR_ARG, "Kepler solver did not converge.");
    if (st & DEV_ERR_PROGRAM) return set_error(s, RGPU_ERR_ARG, "Unknown operator in a WHFast program.");
    return set_error(s, RGPU_ERR_CUDA, "unknown device status");
}

static constexpr size_t kTimerSlots = 256;

static void ktimer_collect(rgpu_sim* s, size_t slot) {
    if (!s->kt_pending[slot]) return;
    float ms = 0.f;
    if (cudaEventSynchronize(s->kt_ev[2 * slot + 1]) == cudaSuccess &&
        cudaEventElapsedTime(&ms, s->kt_ev[2 * slot], s->kt_ev[2 * slot + 1]) == cudaSuccess) {
        s->kt_ms += ms;
        s->kt_count++;
    }
    s->kt_pending[slot] = 0;
}

void ktimer_begin(rgpu_sim* s) {
    if (!s->ktimer_on) return;
    if (s->kt_ev.empty()) {
        s->kt_ev.resize(2 * kTimerSlots);
        s->kt_pending.assign(kTimerSlots, 0);
        for (auto& e : s->kt_ev) cudaEventCreate(&e);
    }
    ktimer_collect(s, s->kt_next);
    cudaEventRecord(s->kt_ev[2 * s->kt_next], s->stream);
}

void ktimer_end(rgpu_sim* s) {
    if (!s->ktimer_on || s->kt_ev.empty()) return;
    cudaEventRecord(s->kt_ev[2 * s->kt_next + 1], s->stream);
    // Also keep the last launch in ev0/ev1 for rgpu_sim_last_kernel_ms.
    s->kt_pending[s->kt_next] = 1;
    s->kt_next = (s->kt_next + 1) % kTimerSlots;
}

void ghostbox(const rgpu_config& c, int i, int j, int k, double gb[6]) {
    // src/boundary.c:145-201
    const double bx = c.root_size * (double)c.N_root_x;
    const double by = c.root_size * (double)c.N_root_y;
    const double bz = c.root_size * (double)c.N_root_z;
    for (int q = 0; q < 6; q++) gb[q] = 0.0;
    if (c.boundary == RGPU_BOUNDARY_OPEN || c.boundary == RGPU_BOUNDARY_PERIODIC) {
        gb[0] = bx * (double)i; gb[1] = by * (double)j; gb[2] = bz * (double)k;
    } else if (c.boundary == RGPU_BOUNDARY_SHEAR) {
        const double vy = -1.5 * (double)i * c.OMEGA * bx;
        double shift;
        if (i == 0) shift = -fmod(vy * c.t, by);
        else if (i > 0) shift = -fmod(vy * c.t - by / 2., by) - by / 2.;
        else shift = -fmod(vy * c.t + by / 2., by) + by / 2.;
        gb[0] = bx * (double)i;
        gb[1] = by * (double)j - shift;
        gb[2] = bz * (double)k;
        gb[4] = vy;
    }
}

namespace {

__global__ void aos_to_soa(const char* __restrict__ src, size_t stride, int N, ParticlesSoA p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double* r = (const double*)(src + (size_t)i * stride);
    p.x[i] = r[0]; p.y[i] = r[1]; p.z[i] = r[2];
    p.vx[i] = r[3]; p.vy[i] = r[4]; p.vz[i] = r[5];
    p.ax[i] = r[6]; p.ay[i] = r[7]; p.az[i] = r[8];
    p.m[i] = r[9]; p.r[i] = r[10];
}

__global__ void soa_to_aos88(ParticlesSoA p, int N, double* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    double* r = dst + (size_t)i * 11;
    r[0] = p.x[i]; r[1] = p.y[i]; r[2] = p.z[i];
    r[3] = p.vx[i]; r[4] = p.vy[i]; r[5] = p.vz[i];
    r[6] = p.ax[i]; r[7] = p.ay[i]; r[8] = p.az[i];
    r[9] = p.m[i]; r[10] = p.r[i];
}

// Leapfrog drift (src/integrator_leapfrog.c:72-82).
__global__ void lf_drift(ParticlesSoA p, int N, double dt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    p.x[i] += dt * p.vx[i];
    p.y[i] += dt * p.vy[i];
    p.z[i] += dt * p.vz[i];
}

// Kick (src/integrator_leapfrog.c:84-93) fused with the closing half drift.
__global__ void lf_kick_drift(ParticlesSoA p, int N, double dt, double dt_half) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double vx = p.vx[i] + dt * p.ax[i];
    const double vy = p.vy[i] + dt * p.ay[i];
    const double vz = p.vz[i] + dt * p.az[i];
    p.vx[i] = vx; p.vy[i] = vy; p.vz[i] = vz;
    p.x[i] += dt_half * vx;
    p.y[i] += dt_half * vy;
    p.z[i] += dt_half * vz;
}

struct SeiCoef { double sindt, tandt, sindtz, tandtz, OMEGA, OMEGAZ, dt; };

// operator_H012 (src/integrator_sei.c:126-157): exact epicyclic motion by
// three shears in z and in the xy epicycle frame.
__device__ __forceinline__ void sei_h012(const SeiCoef& c, double& x, double& y, double& z,
                                         double& vx, double& vy, double& vz) {
    const double zx = z * c.OMEGAZ, zy = vz;
    const double zt1 = zx - c.tandtz * zy;
    const double zyt = c.sindtz * zt1 + zy;
    const double zxt = zt1 - c.tandtz * zyt;
    z = zxt / c.OMEGAZ;
    vz = zyt;
    const double aO = 2. * vy + 4. * x * c.OMEGA;
    const double bO = y * c.OMEGA - 2. * vx;
    const double ys = (y * c.OMEGA - bO) / 2.;
    const double xs = (x * c.OMEGA - aO);
    const double xst1 = xs - c.tandt * ys;
    const double yst = c.sindt * xst1 + ys;
    const double xst = xst1 - c.tandt * yst;
    x = (xst + aO) / c.OMEGA;
    y = (yst * 2. + bO) / c.OMEGA - 3. / 4. * aO * c.dt;
    vx = yst;
    vy = -xst * 2. - 3. / 2. * aO;
}

__global__ void sei_first(ParticlesSoA p, int N, SeiCoef c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    double x = p.x[i], y = p.y[i], z = p.z[i], vx = p.vx[i], vy = p.vy[i], vz = p.vz[i];
    sei_h012(c, x, y, z, vx, vy, vz);
    p.x[i] = x; p.y[i] = y; p.z[i] = z; p.vx[i] = vx; p.vy[i] = vy; p.vz[i] = vz;
}

// operator_phi1 (src/integrator_sei.c:168-174) then the second H012.
__global__ void sei_second(ParticlesSoA p, int N, SeiCoef c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    double x = p.x[i], y = p.y[i], z = p.z[i];
    double vx = p.vx[i] + p.ax[i] * c.dt, vy = p.vy[i] + p.ay[i] * c.dt, vz = p.vz[i] + p.az[i] * c.dt;
    sei_h012(c, x, y, z, vx, vy, vz);
    p.x[i] = x; p.y[i] = y; p.z[i] = z; p.vx[i] = vx; p.vy[i] = vy; p.vz[i] = vz;
}

struct BoxCoef { double bx, by, bz, offp1, offm1, dvy; int shear; };

// src/boundary.c:78-135 (shear and periodic wrap): the reference's repeated
// whole-box shifts, each loop capped at kWrapCap shifts.  A coordinate further out
// (or infinite) is left where it is and reported, instead of looping on it.
constexpr int kWrapCap = 1024;

__global__ void boundary_wrap(ParticlesSoA p, int N, BoxCoef b, uint32_t* status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    double x = p.x[i], y = p.y[i], z = p.z[i], vy = p.vy[i];
    int nx = 0, ny = 0, nz = 0;
    if (b.shear) {
        for (; x > b.bx / 2. && nx < kWrapCap; nx++) { x -= b.bx; y += b.offp1; vy += b.dvy; }
        for (; x < -b.bx / 2. && nx < kWrapCap; nx++) { x += b.bx; y += b.offm1; vy -= b.dvy; }
    } else {
        for (; x > b.bx / 2. && nx < kWrapCap; nx++) x -= b.bx;
        for (; x < -b.bx / 2. && nx < kWrapCap; nx++) x += b.bx;
    }
    for (; y > b.by / 2. && ny < kWrapCap; ny++) y -= b.by;
    for (; y < -b.by / 2. && ny < kWrapCap; ny++) y += b.by;
    for (; z > b.bz / 2. && nz < kWrapCap; nz++) z -= b.bz;
    for (; z < -b.bz / 2. && nz < kWrapCap; nz++) z += b.bz;
    if (nx >= kWrapCap || ny >= kWrapCap || nz >= kWrapCap) {
        atomicOr(status, DEV_ERR_OUT_OF_BOX);
        return;
    }
    p.x[i] = x; p.y[i] = y; p.z[i] = z; p.vy[i] = vy;
}

__global__ void zero_acc(ParticlesSoA p, int N) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    p.ax[i] = 0.; p.ay[i] = 0.; p.az[i] = 0.;
}

int ensure_capacity(rgpu_sim* s, size_t N) {
    if (N <= s->cap) return RGPU_OK;
    size_t cap = s->cap ? s->cap : 256;
    while (cap < N) cap *= 2;
    double* block = nullptr;
    RGPU_CUDA(s, cudaMalloc(&block, sizeof(double) * 11 * cap));
    double4_32a* jpos = nullptr;
    float4* jsplit = nullptr;
    cudaError_t e1 = cudaMalloc(&jpos, sizeof(double4_32a) * cap);
    cudaError_t e2 = cudaMalloc(&jsplit, sizeof(float4) * 2 * cap);
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
        cudaFree(block); cudaFree(jpos); cudaFree(jsplit);
        return check_cuda(s, e1 != cudaSuccess ? e1 : e2, "cudaMalloc particle buffers");
    }
    if (s->soa_block) {
        // keep the current state when growing
        for (int f = 0; f < 11; f++)
            cudaMemcpyAsync(block + f * cap, s->soa_block + f * s->cap, sizeof(double) * s->N, cudaMemcpyDeviceToDevice, s->stream);
        cudaStreamSynchronize(s->stream);
        cudaFree(s->soa_block);
    }
    cudaFree(s->jpos);
    cudaFree(s->jsplit);
    s->soa_block = block;
    s->jpos = jpos;
    s->jsplit = jsplit;
    s->cap = cap;
    double** f[11] = {&s->p.x, &s->p.y, &s->p.z, &s->p.vx, &s->p.vy, &s->p.vz, &s->p.ax, &s->p.ay, &s->p.az, &s->p.m, &s->p.r};
    for (int q = 0; q < 11; q++) *f[q] = block + (size_t)q * cap;
    if (s->partial) { cudaFree(s->partial); s->partial = nullptr; s->partial_cap = 0; }
    return RGPU_OK;
}

int ensure_stage(rgpu_sim* s, size_t bytes) {
    if (bytes <= s->stage_cap) return RGPU_OK;
    cudaFree(s->stage);
    s->stage = nullptr;
    s->stage_cap = 0;
    RGPU_CUDA(s, cudaMalloc(&s->stage, bytes));
    s->stage_cap = bytes;
    return RGPU_OK;
}

int update_acceleration(rgpu_sim* s) {
    const int N = (int)s->N;
    switch (s->cfg.gravity) {
        case RGPU_GRAVITY_NONE:
            if (N) { zero_acc<<<grid_for(N, 256), 256, 0, s->stream>>>(s->p, N); g_launches++; }
            return RGPU_OK;
        case RGPU_GRAVITY_BASIC:
        case RGPU_GRAVITY_COMPENSATED:
        case RGPU_GRAVITY_MIXED:
        case RGPU_GRAVITY_MIXED_SPLIT:
            return direct_accel(s, s->cfg.gravity);
        case RGPU_GRAVITY_TREE:
        case RGPU_GRAVITY_TREE_SPLIT:
            return tree_accel(s);
        default:
            return set_error(s, RGPU_ERR_ARG, "Gravity module not found.");
    }
}

// Composition coefficients of the order-4, -6 and -8 leapfrog schemes
// (src/integrator_leapfrog.c:68-70): the order-4 value is Yoshida's
// 1 / (2 (2 - 2^(1/3))); the order-6 and -8 kick weights are the symmetric
// composition coefficients the reference uses, kept digit for digit so that the
// drift and kick lengths round exactly as there.
constexpr double kLf4A = 0.675603595979828817023843904485;
constexpr double kLf6A[5] = {0.1867, 0.5554970237124784, 0.1294669489134754, -0.843265623387734, 0.9432033015235604};
constexpr double kLf8A[9] = {0.128865979381443, 0.581514087105251, -0.410175371469850, 0.1851469357165877,
                             -0.4095523434208514, 0.1444059410800120, 0.2783355003936797, 0.3149566839162949,
                             -0.6269948254051343979};

// Drift lengths d[0..nk] and kick lengths k[0..nk-1] of one step: the scheme is
// D(d0) [a K(k0) D(d1)] ... [a K(k_{nk-1}) D(d_nk)], with the reference's own
// expressions for each length (src/integrator_leapfrog.c:97-203).
int leapfrog_scheme(int order, double dt, double* d, double* k) {
    switch (order) {
        case 0:
        case 2:
            d[0] = dt * 0.5; k[0] = dt; d[1] = dt * 0.5;
            return 1;
        case 4:
            d[0] = dt * kLf4A; k[0] = dt * 2. * kLf4A; d[1] = dt * (0.5 - kLf4A);
            k[1] = dt * (1. - 4. * kLf4A); d[2] = dt * (0.5 - kLf4A); k[2] = dt * 2. * kLf4A; d[3] = dt * kLf4A;
            return 3;
        case 6:
        case 8: {
            const double* a = order == 6 ? kLf6A : kLf8A;
            const int m = order == 6 ? 5 : 9;
            const int nk = 2 * m - 1;                // kick weights a0 .. a_{m-1} .. a0
            d[0] = dt * a[0] * 0.5;
            for (int q = 0; q < nk; q++) {
                const int ia = q < m ? q : nk - 1 - q;
                k[q] = dt * a[ia];
                if (q + 1 < nk) {
                    const int ib = q + 1 < m ? q + 1 : nk - 2 - q;
                    const int lo = ia < ib ? ia : ib, hi = ia < ib ? ib : ia;
                    d[q + 1] = dt * (a[lo] + a[hi]) * 0.5;
                }
            }
            d[nk] = dt * a[0] * 0.5;
            return nk;
        }
        default:
            return -1;
    }
}

int leapfrog_step(rgpu_sim* s) {
    // src/integrator_leapfrog.c:97-203: drift, then (accelerations, kick, drift) per stage;
    // the time advances with each drift as in the reference.
    const int N = (int)s->N;
    s->cfg.gravity_ignore_terms = 0;
    double d[18], k[17];
    const int nk = leapfrog_scheme(s->cfg.leapfrog_order, s->cfg.dt, d, k);
    if (nk < 0) return set_error(s, RGPU_ERR_ARG, "leapfrog order must be 2, 4, 6 or 8");
    if (N) { lf_drift<<<grid_for(N, 256), 256, 0, s->stream>>>(s->p, N, d[0]); g_launches++; }
    s->cfg.t += d[0];
    for (int q = 0; q < nk; q++) {
        RGPU_TRY(update_acceleration(s));
        if (N) { lf_kick_drift<<<grid_for(N, 256), 256, 0, s->stream>>>(s->p, N, k[q], d[q + 1]); g_launches++; }
        s->cfg.t += d[q + 1];
    }
    return RGPU_OK;
}

int sei_step(rgpu_sim* s, SeiCache& cache) {
    // src/integrator_sei.c:86-117; sin/tan are evaluated on the host like the reference.
    rgpu_config& c = s->cfg;
    const int N = (int)s->N;
    c.gravity_ignore_terms = 0;
    if (cache.lastdt != c.dt) {
        if (c.OMEGAZ == -1) c.OMEGAZ = c.OMEGA;
        cache.sindt = sin(c.OMEGA * (-c.dt / 2.));
        cache.tandt = tan(c.OMEGA * (-c.dt / 4.));
        cache.sindtz = sin(c.OMEGAZ * (-c.dt / 2.));
        cache.tandtz = tan(c.OMEGAZ * (-c.dt / 4.));
        cache.lastdt = c.dt;
    }
    const SeiCoef k{cache.sindt, cache.tandt, cache.sindtz, cache.tandtz, c.OMEGA, c.OMEGAZ, c.dt};
    if (N) { sei_first<<<grid_for(N, 256), 256, 0, s->stream>>>(s->p, N, k); g_launches++; }
    c.t += c.dt / 2.;
    RGPU_TRY(update_acceleration(s));
    if (N) { sei_second<<<grid_for(N, 256), 256, 0, s->stream>>>(s->p, N, k); g_launches++; }
    c.t += c.dt / 2.;
    return RGPU_OK;
}

}  // namespace

int boundary_check(rgpu_sim* s) {
    const rgpu_config& c = s->cfg;
    const int N = (int)s->N;
    if (!N) return RGPU_OK;
    if (c.boundary == RGPU_BOUNDARY_OPEN)
        return set_error(s, RGPU_ERR_UNSUPPORTED, "open boundary (particle removal) is not on the GPU path");
    if (c.boundary != RGPU_BOUNDARY_SHEAR && c.boundary != RGPU_BOUNDARY_PERIODIC) return RGPU_OK;
    BoxCoef b;
    b.bx = c.root_size * (double)c.N_root_x;
    b.by = c.root_size * (double)c.N_root_y;
    b.bz = c.root_size * (double)c.N_root_z;
    b.shear = c.boundary == RGPU_BOUNDARY_SHEAR;
    b.offp1 = -fmod(-1.5 * c.OMEGA * b.bx * c.t + b.by / 2., b.by) - b.by / 2.;
    b.offm1 = -fmod(1.5 * c.OMEGA * b.bx * c.t - b.by / 2., b.by) + b.by / 2.;
    b.dvy = 3. / 2. * c.OMEGA * b.bx;
    boundary_wrap<<<grid_for(N, 256), 256, 0, s->stream>>>(s->p, N, b, s->d_status);
    g_launches++;
    return RGPU_OK;
}

// ----------------------------------------------------------------------------
// C ABI
// ----------------------------------------------------------------------------

extern "C" {

void rgpu_config_default(rgpu_config* c) {
    std::memset(c, 0, sizeof(*c));
    c->G = 1.0;
    c->OMEGA = 1.0;
    c->OMEGAZ = -1.0;
    c->root_size = -1.0;
    c->opening_angle2 = 0.25;
    c->coefficient_of_restitution = 1.0;
    c->N_active = -1;
    c->N_root_x = c->N_root_y = c->N_root_z = 1;
    c->gravity = RGPU_GRAVITY_BASIC;
    c->collision = RGPU_COLLISION_NONE;
    c->collision_resolve = RGPU_RESOLVE_HALT;
    c->boundary = RGPU_BOUNDARY_NONE;
    c->integrator = RGPU_INTEGRATOR_LEAPFROG;
    c->whfast_safe_mode = 1;
    c->exact_finish_time = 1;
    c->status = -1;
}

int rgpu_sim_create(rgpu_sim** out) {
    if (!out) return RGPU_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return RGPU_ERR_CUDA;
    }
    rgpu_sim* s = new (std::nothrow) rgpu_sim();
    if (!s) return RGPU_ERR_NOMEM;
    rgpu_config_default(&s->cfg);
    int rc = RGPU_OK;
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&s->d_status, sizeof(uint32_t)) != cudaSuccess ||
        cudaMemset(s->d_status, 0, sizeof(uint32_t)) != cudaSuccess ||
        cudaEventCreate(&s->ev0) != cudaSuccess || cudaEventCreate(&s->ev1) != cudaSuccess) {
        rc = RGPU_ERR_CUDA;
    }
    if (rc) { rgpu_sim_free(s); return rc; }
    *out = s;
    return RGPU_OK;
}

void rgpu_sim_free(rgpu_sim* s) {
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    tree_free(s);
    whfast_free(s);
    collide_free(s);
    direct_free(s);
    cudaFree(s->soa_block);
    cudaFree(s->jpos);
    cudaFree(s->jsplit);
    cudaFree(s->partial);
    cudaFree(s->stage);
    cudaFree(s->d_status);
    cudaFree(s->d_scalar);
    for (auto& e : s->kt_ev) cudaEventDestroy(e);
    cudaFree(s->flush_buf);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

const char* rgpu_sim_last_error(const rgpu_sim* s) { return s ? s->msg.c_str() : "null handle"; }

int rgpu_sim_configure(rgpu_sim* s, const rgpu_config* c) {
    if (!s || !c) return RGPU_ERR_ARG;
    if (c->gravity == RGPU_GRAVITY_TREE || c->gravity == RGPU_GRAVITY_TREE_SPLIT || c->collision == RGPU_COLLISION_TREE ||
        c->collision == RGPU_COLLISION_LINETREE) {
        if (c->root_size <= 0.0)
            return set_error(s, RGPU_ERR_ARG, "Set root_size to a finite value to use a tree based gravity or collision solver.");
    }
    if (c->N_root_x < 1 || c->N_root_y < 1 || c->N_root_z < 1) return set_error(s, RGPU_ERR_ARG, "N_root must be >= 1");
    if (c->N_ghost_x < 0 || c->N_ghost_y < 0 || c->N_ghost_z < 0) return set_error(s, RGPU_ERR_ARG, "N_ghost must be >= 0");
    if (c->integrator < 0 || c->integrator > 2) return set_error(s, RGPU_ERR_ARG, "unknown integrator");
    if (c->boundary < 0 || c->boundary > 3) return set_error(s, RGPU_ERR_ARG, "unknown boundary");
    if (c->collision != RGPU_COLLISION_NONE && c->collision != RGPU_COLLISION_DIRECT &&
        c->collision != RGPU_COLLISION_TREE && c->collision != RGPU_COLLISION_LINE &&
        c->collision != RGPU_COLLISION_LINETREE)
        return set_error(s, RGPU_ERR_UNSUPPORTED, "Collision routine not implemented.");
    if (c->collision_resolve < RGPU_RESOLVE_HALT || c->collision_resolve > RGPU_RESOLVE_NONE)
        return set_error(s, RGPU_ERR_UNSUPPORTED,
                         "collision_resolve: halt, hardsphere or none (resolvers that remove particles are not on the GPU path)");
    const bool integrator_changed = c->integrator != s->cfg.integrator;
    s->cfg = *c;
    if (integrator_changed) { s->did_modify = true; s->whfast_synchronized = true; }
    return RGPU_OK;
}

int rgpu_sim_get_config(const rgpu_sim* s, rgpu_config* c) {
    if (!s || !c) return RGPU_ERR_ARG;
    *c = s->cfg;
    return RGPU_OK;
}

size_t rgpu_sim_N(const rgpu_sim* s) { return s ? s->N : 0; }

int rgpu_sim_set_particles(rgpu_sim* s, const void* particles, size_t N, size_t stride) {
    if (!s || (N && !particles) || stride < 88 || (stride % 8) != 0) return set_error(s, RGPU_ERR_ARG, "bad particle buffer");
    if (N > (size_t)INT32_MAX / 2) return set_error(s, RGPU_ERR_CAPACITY, "too many particles");
    RGPU_TRY(ensure_capacity(s, N));
    s->N = N;
    s->did_modify = true;
    s->whfast_synchronized = true;
    if (!N) return RGPU_OK;
    RGPU_TRY(ensure_stage(s, N * stride));
    RGPU_CUDA(s, cudaMemcpyAsync(s->stage, particles, N * stride, cudaMemcpyHostToDevice, s->stream));
    aos_to_soa<<<grid_for(N, 256), 256, 0, s->stream>>>((const char*)s->stage, stride, (int)N, s->p);
    g_launches++;
    RGPU_CUDA(s, cudaGetLastError());
    return RGPU_OK;
}

int rgpu_sim_get_particles(rgpu_sim* s, void* particles, size_t N, size_t stride) {
    if (!s || (N && !particles) || stride < 88) return set_error(s, RGPU_ERR_ARG, "bad particle buffer");
    if (N != s->N) return set_error(s, RGPU_ERR_ARG, "particle count mismatch");
    if (!N) return RGPU_OK;
    RGPU_TRY(ensure_stage(s, N * 88));
    soa_to_aos88<<<grid_for(N, 256), 256, 0, s->stream>>>(s->p, (int)N, (double*)s->stage);
    g_launches++;
    if (stride == 88)
        RGPU_CUDA(s, cudaMemcpyAsync(particles, s->stage, N * 88, cudaMemcpyDeviceToHost, s->stream));
    else
        RGPU_CUDA(s, cudaMemcpy2DAsync(particles, stride, s->stage, 88, 88, N, cudaMemcpyDeviceToHost, s->stream));
    RGPU_CUDA(s, cudaStreamSynchronize(s->stream));
    return RGPU_OK;
}

int rgpu_update_acceleration(rgpu_sim* s) {
    if (!s) return RGPU_ERR_ARG;
    RGPU_TRY(update_acceleration(s));
    return read_status(s);
}

int rgpu_collision_search(rgpu_sim* s, rgpu_collision* out, size_t cap, size_t* n_found) {
    if (!s || !n_found || (cap && !out)) return set_error(s, RGPU_ERR_ARG, "bad collision buffer");
    *n_found = 0;
    switch (s->cfg.collision) {
        case RGPU_COLLISION_NONE: return RGPU_OK;
        case RGPU_COLLISION_DIRECT: return direct_collisions(s, out, cap, n_found, false);
        case RGPU_COLLISION_TREE: return tree_collisions(s, out, cap, n_found, false);
        case RGPU_COLLISION_LINE: return direct_collisions(s, out, cap, n_found, false, true);
        case RGPU_COLLISION_LINETREE: return tree_collisions(s, out, cap, n_found, false, true);
        default: return set_error(s, RGPU_ERR_UNSUPPORTED, "Collision routine not implemented.");
    }
}

int rgpu_steps(rgpu_sim* s, int64_t n) {
    if (!s || n < 0) return RGPU_ERR_ARG;
    for (int64_t k = 0; k < n; k++) {
        RGPU_TRY(archive_heartbeat(s));                  // src/simulation.c:507-508
        switch (s->cfg.integrator) {
            case RGPU_INTEGRATOR_LEAPFROG: RGPU_TRY(leapfrog_step(s)); break;
            case RGPU_INTEGRATOR_SEI: RGPU_TRY(sei_step(s, s->sei)); break;
            case RGPU_INTEGRATOR_WHFAST: RGPU_TRY(whfast_step(s)); break;
            default: return set_error(s, RGPU_ERR_ARG, "unknown integrator");
        }
        s->did_modify = false;
        s->dt_last_done = s->cfg.dt;
        s->steps_done++;
        RGPU_TRY(boundary_check(s));
        if (s->cfg.collision != RGPU_COLLISION_NONE) {
            size_t nf = 0;
            switch (s->cfg.collision) {
                case RGPU_COLLISION_DIRECT: RGPU_TRY(direct_collisions(s, nullptr, 0, &nf, true)); break;
                case RGPU_COLLISION_TREE: RGPU_TRY(tree_collisions(s, nullptr, 0, &nf, true)); break;
                case RGPU_COLLISION_LINE: RGPU_TRY(direct_collisions(s, nullptr, 0, &nf, true, true)); break;
                case RGPU_COLLISION_LINETREE: RGPU_TRY(tree_collisions(s, nullptr, 0, &nf, true, true)); break;
                default: return set_error(s, RGPU_ERR_UNSUPPORTED, "Collision routine not implemented.");
            }
            RGPU_TRY(resolve_collisions_device(s));
            if (s->cfg.status == 7) break;   // REB_STATUS_COLLISION from the halt resolver
        }
    }
    return read_status(s);
}

// Brings the integrator state to synchronized coordinates (reb_simulation_synchronize).
static int synchronize_state(rgpu_sim* s) {
    if (s->cfg.integrator == RGPU_INTEGRATOR_WHFAST) return whfast_synchronize(s);
    return RGPU_OK;
}

// reb_simulation_integrate (src/simulation.c:372-464) with the exit test of
// reb_check_exit (:291-354): with exact_finish_time the state is synchronized
// before the shortened last step, and dt returns to the last full step at the end.
int rgpu_integrate(rgpu_sim* s, double tmax) {
    if (!s) return RGPU_ERR_ARG;
    rgpu_config& c = s->cfg;
    if (c.dt == 0.0) return set_error(s, RGPU_ERR_ARG, "dt must be nonzero");
    c.status = -1;                                                  // REB_STATUS_RUNNING (:389-391)
    if (tmax != c.t) c.dt = std::copysign(c.dt, tmax > c.t ? 1.0 : -1.0);
    double last_full_dt = c.dt;
    s->dt_last_done = 0.;
    bool last_step = false;
    for (;;) {
        const double dtsign = std::copysign(1., c.dt);
        if (c.exact_finish_time) {
            if ((c.t + c.dt) * dtsign >= tmax * dtsign) {         // the next step would overshoot
                if (c.t == tmax) break;
                if (last_step) {
                    double tscale = 1e-12 * std::fabs(tmax);
                    if (tscale < 1e-200) tscale = 1e-12;
                    if (std::fabs(c.t - tmax) < tscale) break;
                    RGPU_TRY(synchronize_state(s));
                    c.dt = tmax - c.t;
                } else {
                    last_step = true;
                    RGPU_TRY(synchronize_state(s));
                    if (s->dt_last_done != 0.) last_full_dt = s->dt_last_done;
                    c.dt = tmax - c.t;
                }
            } else {
                last_step = false;
            }
        } else if (c.t * dtsign >= tmax * dtsign) {
            break;
        }
        const double t_before = c.t;
        RGPU_TRY(rgpu_steps(s, 1));
        if (c.status == 7) break;                                   // collision halt
        if (c.t == t_before) return set_error(s, RGPU_ERR_ARG, "dt too small to advance t");
    }
    RGPU_TRY(synchronize_state(s));
    if (c.exact_finish_time) c.dt = last_full_dt;
    RGPU_TRY(archive_heartbeat(s));                      // :459
    return read_status(s);
}

int rgpu_synchronize(rgpu_sim* s) {
    if (!s) return RGPU_ERR_ARG;
    if (s->cfg.integrator == RGPU_INTEGRATOR_WHFAST) RGPU_TRY(whfast_synchronize(s));
    return read_status(s);
}

int rgpu_energy(rgpu_sim* s, double* e) {
    if (!s || !e) return RGPU_ERR_ARG;
    if (s->cfg.integrator == RGPU_INTEGRATOR_WHFAST && !s->whfast_synchronized) {
        // the energy of the synchronized state; with safe_mode 0 the integrator keeps
        // its unsynchronized coordinates (keep_unsynchronized), so asking for the
        // energy does not change the trajectory
        const int keep = s->cfg.whfast_keep_unsynchronized;
        if (!s->cfg.whfast_safe_mode) s->cfg.whfast_keep_unsynchronized = 1;
        const int rc = whfast_synchronize(s);
        s->cfg.whfast_keep_unsynchronized = keep;
        RGPU_TRY(rc);
    }
    RGPU_TRY(direct_energy(s, e));
    return read_status(s);
}

int rgpu_sim_sync(rgpu_sim* s) {
    if (!s) return RGPU_ERR_ARG;
    RGPU_CUDA(s, cudaStreamSynchronize(s->stream));
    return read_status(s);
}

double rgpu_sim_last_kernel_ms(const rgpu_sim* s) {
    if (!s) return -1.0;
    float ms = -1.f;
    if (cudaEventSynchronize(s->ev1) != cudaSuccess) return -1.0;
    if (cudaEventElapsedTime(&ms, s->ev0, s->ev1) != cudaSuccess) { cudaGetLastError(); return -1.0; }
    return (double)ms;
}

int64_t rgpu_launch_count(void) { return g_launches.load(); }

int rgpu_sim_kernel_timer(rgpu_sim* s, int enable) {
    if (!s) return RGPU_ERR_ARG;
    s->ktimer_on = enable != 0;
    s->kt_ms = 0.;
    s->kt_count = 0;
    for (size_t k = 0; k < s->kt_pending.size(); k++) s->kt_pending[k] = 0;
    return RGPU_OK;
}

int rgpu_sim_kernel_time(rgpu_sim* s, double* total_ms, int64_t* launches) {
    if (!s || !total_ms || !launches) return RGPU_ERR_ARG;
    RGPU_CUDA(s, cudaStreamSynchronize(s->stream));
    for (size_t k = 0; k < s->kt_pending.size(); k++) ktimer_collect(s, k);
    *total_ms = s->kt_ms;
    *launches = s->kt_count;
    return RGPU_OK;
}

int rgpu_sim_time_steps(rgpu_sim* s, int64_t n, double* ms) {
    if (!s || !ms || n < 0) return RGPU_ERR_ARG;
    RGPU_CUDA(s, cudaEventRecord(s->ev0, s->stream));
    const int rc = rgpu_steps(s, n);
    RGPU_CUDA(s, cudaEventRecord(s->ev1, s->stream));
    RGPU_CUDA(s, cudaEventSynchronize(s->ev1));
    float f = 0.f;
    RGPU_CUDA(s, cudaEventElapsedTime(&f, s->ev0, s->ev1));
    *ms = f;
    return rc;
}

int rgpu_l2_flush(rgpu_sim* s, size_t bytes) {
    if (!s) return RGPU_ERR_ARG;
    if (bytes > s->flush_bytes) {
        cudaFree(s->flush_buf);
        s->flush_buf = nullptr;
        s->flush_bytes = 0;
        RGPU_CUDA(s, cudaMalloc(&s->flush_buf, bytes));
        s->flush_bytes = bytes;
    }
    RGPU_CUDA(s, cudaMemsetAsync(s->flush_buf, (int)(s->kt_count & 0xff), bytes, s->stream));
    return RGPU_OK;
}

}  // extern "C"
