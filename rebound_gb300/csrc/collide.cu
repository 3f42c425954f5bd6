// Direct collision search (src/collision.c:64-124), the LINE search (:125-196), and the post-search stage of
// reb_collision_search (src/collision.c:336-404): the rand_r shuffle of the pair
// list and the sequential resolve, hardsphere (src/collision.c:573-665) or halt.
//
// The search emits pairs in the reference's discovery order (ghost box, then
// projectile i, then target j), counted in one pass and written in a second
// after an exclusive scan.  The resolve stays on the host, as in the
// reference: pairs are few and strictly sequential (each bounce changes the
// velocities the next test reads); only the touched particles move between
// device and host.  Compiled with --fmad=false (exact pair tests).
#include "rgpu_internal.cuh"
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <unordered_map>
#include <vector>

namespace {

constexpr int kB = 128;

struct Ring {
    int n;
    double off[27][6];
};

// LINE = true: the LINE search (src/collision.c:125-196): pairs j > i whose straight
// paths over the last step (dt_last_done) come within the sum of the radii.
template <bool LINE>
__device__ __forceinline__ int direct_pairs_one(int g, int i, const Ring& ring, ParticlesSoA p, int N, double dtl,
                                                rgpu_collision* out, long long base) {
    const double* gb = ring.off[g];
    const double sx = gb[0] + p.x[i], sy = gb[1] + p.y[i], sz = gb[2] + p.z[i];
    const double svx = gb[3] + p.vx[i], svy = gb[4] + p.vy[i], svz = gb[5] + p.vz[i];
    const double r1 = p.r[i];
    int found = 0;
    for (int j = LINE ? i + 1 : 0; j < N; j++) {
        if (!LINE && i == j) continue;
        const double dx = sx - p.x[j], dy = sy - p.y[j], dz = sz - p.z[j];
        const double r2 = dx * dx + dy * dy + dz * dz;
        const double dvx = svx - p.vx[j], dvy = svy - p.vy[j], dvz = svz - p.vz[j];
        if (LINE) {
            const double dx2 = dx - dtl * dvx, dy2 = dy - dtl * dvy, dz2 = dz - dtl * dvz;   // at the start
            const double r2b = dx2 * dx2 + dy2 * dy2 + dz2 * dz2;
            const double tc = (dx * dvx + dy * dvy + dz * dvz) / (dvx * dvx + dvy * dvy + dvz * dvz);
            double rmin2 = r2 < r2b ? r2 : r2b;
            if (tc / dtl >= 0. && tc / dtl <= 1.) {
                const double dx3 = dx - tc * dvx, dy3 = dy - tc * dvy, dz3 = dz - tc * dvz;  // closest approach
                const double r3 = dx3 * dx3 + dy3 * dy3 + dz3 * dz3;
                rmin2 = rmin2 < r3 ? rmin2 : r3;
            }
            const double rsum = r1 + p.r[j];
            if (rmin2 > rsum * rsum) continue;
        } else {
            const double sr = r1 + p.r[j];
            if (r2 > sr * sr) continue;
            if (dvx * dx + dvy * dy + dvz * dz > 0) continue;
        }
        if (out) {
            rgpu_collision& o = out[base + found];
            o.p1 = (size_t)i; o.p2 = (size_t)j; o.ri = 0;
            for (int k = 0; k < 6; k++) o.gb[k] = gb[k];
        }
        found++;
    }
    return found;
}

template <bool LINE>
__global__ void direct_count(Ring ring, ParticlesSoA p, int N, double dtl, int* count) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)ring.n * N) return;
    const int g = (int)(t / N), i = (int)(t % N);
    count[t] = direct_pairs_one<LINE>(g, i, ring, p, N, dtl, nullptr, 0);
}

template <bool LINE>
__global__ void direct_write(Ring ring, ParticlesSoA p, int N, double dtl, const long long* off, rgpu_collision* out) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)ring.n * N) return;
    const int g = (int)(t / N), i = (int)(t % N);
    direct_pairs_one<LINE>(g, i, ring, p, N, dtl, out, off[t]);
}

__global__ void scan_counts(const int* __restrict__ cnt, long long n, long long* __restrict__ off) {
    __shared__ long long part[256];
    const long long per = (n + 255) / 256;
    const long long b0 = threadIdx.x * per;
    long long s = 0;
    for (long long k = 0; k < per; k++) if (b0 + k < n) s += cnt[b0 + k];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < 256; o <<= 1) {
        const long long v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    long long run = threadIdx.x ? part[threadIdx.x - 1] : 0;
    for (long long k = 0; k < per; k++) {
        if (b0 + k < n) { off[b0 + k] = run; run += cnt[b0 + k]; }
    }
    if (threadIdx.x == 255) off[n] = run;
}

// Gather / scatter the particles touched by the resolve.
__global__ void gather_touched(ParticlesSoA p, const int* __restrict__ ids, int n, double* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = ids[k];
    double* o = out + 8 * (size_t)k;
    o[0] = p.x[i]; o[1] = p.y[i]; o[2] = p.z[i]; o[3] = p.vx[i]; o[4] = p.vy[i]; o[5] = p.vz[i];
    o[6] = p.m[i]; o[7] = p.r[i];
}

__global__ void scatter_velocities(ParticlesSoA p, const int* __restrict__ ids, int n, const double* __restrict__ in) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = ids[k];
    const double* v = in + 8 * (size_t)k;
    p.vx[i] = v[3]; p.vy[i] = v[4]; p.vz[i] = v[5];
}

struct Body { double x, y, z, vx, vy, vz, m, r; };

// reb_collision_resolve_hardsphere (src/collision.c:573-665): the restitution
// coefficient is the constant eps, or eps_fn(eps_user, v) of the normal relative
// velocity when a callback is set; plog accumulates the y-momentum transferred
// to the outer particle (src/collision.c:655-662).
void hardsphere(Body& p1, Body& p2, const double gb[6], double eps, double (*eps_fn)(void*, double), void* eps_user,
                double minvel, int64_t& log_n, double& plog) {
    const double x21 = p1.x + gb[0] - p2.x, y21 = p1.y + gb[1] - p2.y, z21 = p1.z + gb[2] - p2.z;
    const double rp = p1.r + p2.r;
    const double oldvyouter = x21 > 0 ? p1.vy : p2.vy;
    if (rp * rp < x21 * x21 + y21 * y21 + z21 * z21) return;
    const double vx21 = p1.vx + gb[3] - p2.vx, vy21 = p1.vy + gb[4] - p2.vy, vz21 = p1.vz + gb[5] - p2.vz;
    if (vx21 * x21 + vy21 * y21 + vz21 * z21 > 0) return;
    const double th = atan2(z21, y21), sth = sin(th), cth = cos(th);
    const double vy21n = cth * vy21 + sth * vz21;
    const double y21n = cth * y21 + sth * z21;
    const double ph = atan2(y21n, x21), cph = cos(ph), sph = sin(ph);
    const double vx21nn = cph * vx21 + sph * vy21n;
    if (eps_fn) eps = eps_fn(eps_user, vx21nn);
    double dvx2 = -(1.0 + eps) * vx21nn;
    const double minr = (p1.r > p2.r) ? p2.r : p1.r;
    const double maxr = (p1.r < p2.r) ? p2.r : p1.r;
    double mindv = minr * minvel;
    const double rr = sqrt(x21 * x21 + y21 * y21 + z21 * z21);
    mindv *= 1. - (rr - maxr) / minr;
    if (mindv > maxr * minvel) mindv = maxr * minvel;
    if (dvx2 < mindv) dvx2 = mindv;
    const double dvx2n = cph * dvx2, dvy2n = sph * dvx2;
    const double dvy2nn = cth * dvy2n, dvz2nn = sth * dvy2n;
    const double p2pf = p1.m / (p1.m + p2.m);
    p2.vx -= p2pf * dvx2n; p2.vy -= p2pf * dvy2nn; p2.vz -= p2pf * dvz2nn;
    const double p1pf = p2.m / (p1.m + p2.m);
    p1.vx += p1pf * dvx2n; p1.vy += p1pf * dvy2nn; p1.vz += p1pf * dvz2nn;
    if (x21 > 0) plog += -fabs(x21) * (oldvyouter - p1.vy) * p1.m;
    else plog += -fabs(x21) * (oldvyouter - p2.vy) * p2.m;
    log_n++;
}

}  // namespace

int direct_collisions(rgpu_sim* s, rgpu_collision* out, size_t cap, size_t* n_found, bool device_only, bool line) {
    const int N = (int)s->N;
    *n_found = 0;
    s->n_pairs = 0;
    if (!N) return RGPU_OK;
    const rgpu_config& c = s->cfg;
    Ring ring;
    ring.n = 0;
    const int nx = c.N_ghost_x > 1 ? 1 : c.N_ghost_x, ny = c.N_ghost_y > 1 ? 1 : c.N_ghost_y,
              nz = c.N_ghost_z > 1 ? 1 : c.N_ghost_z;
    for (int gx = -nx; gx <= nx; gx++)
        for (int gy = -ny; gy <= ny; gy++)
            for (int gz = -nz; gz <= nz; gz++) ghostbox(c, gx, gy, gz, ring.off[ring.n++]);
    const long long nt = (long long)ring.n * N;
    if ((size_t)nt > s->pc_cap) {
        cudaFree(s->pc_count); cudaFree(s->pc_off);
        s->pc_count = nullptr; s->pc_off = nullptr; s->pc_cap = 0;
        RGPU_CUDA(s, cudaMalloc(&s->pc_count, sizeof(int) * nt));
        RGPU_CUDA(s, cudaMalloc(&s->pc_off, sizeof(long long) * (nt + 1)));
        s->pc_cap = (size_t)nt;
    }
    const unsigned grid = (unsigned)((nt + kB - 1) / kB);
    const double dtl = s->dt_last_done;
    if (line) direct_count<true><<<grid, kB, 0, s->stream>>>(ring, s->p, N, dtl, s->pc_count);
    else direct_count<false><<<grid, kB, 0, s->stream>>>(ring, s->p, N, dtl, s->pc_count);
    scan_counts<<<1, 256, 0, s->stream>>>(s->pc_count, nt, s->pc_off);
    g_launches += 2;
    long long total = 0;
    RGPU_CUDA(s, cudaMemcpyAsync(&total, s->pc_off + nt, sizeof(long long), cudaMemcpyDeviceToHost, s->stream));
    RGPU_CUDA(s, cudaStreamSynchronize(s->stream));
    if ((size_t)total > s->dp_cap) {
        cudaFree(s->dp_pairs);
        s->dp_pairs = nullptr;
        s->dp_cap = 0;
        const size_t want = std::max<size_t>(1024, 2 * (size_t)total);
        RGPU_CUDA(s, cudaMalloc(&s->dp_pairs, sizeof(rgpu_collision) * want));
        s->dp_cap = want;
    }
    if (total) {
        if (line) direct_write<true><<<grid, kB, 0, s->stream>>>(ring, s->p, N, dtl, s->pc_off, s->dp_pairs);
        else direct_write<false><<<grid, kB, 0, s->stream>>>(ring, s->p, N, dtl, s->pc_off, s->dp_pairs);
        g_launches++;
    }
    *n_found = (size_t)total;
    s->n_pairs = (size_t)total;
    s->dev_pairs = s->dp_pairs;
    if (device_only) return RGPU_OK;
    if ((size_t)total > cap) return set_error(s, RGPU_ERR_OVERFLOW, "collision buffer too small");
    if (total) RGPU_CUDA(s, cudaMemcpyAsync(out, s->dp_pairs, sizeof(rgpu_collision) * total, cudaMemcpyDeviceToHost, s->stream));
    RGPU_CUDA(s, cudaStreamSynchronize(s->stream));
    return read_status(s);
}

static int resolve_pairs(rgpu_sim* s);

// Host wall time of the resolve stage (shuffle, gather, hardsphere, scatter).
int resolve_collisions_device(rgpu_sim* s) {
    const size_t n = s->n_pairs;
    if (n == 0) return RGPU_OK;
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = resolve_pairs(s);
    s->resolve_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    s->resolve_calls++;
    return rc;
}

extern "C" int rgpu_sim_set_restitution_fn(rgpu_sim* s, double (*fn)(void*, double), void* user) {
    if (!s) return RGPU_ERR_ARG;
    s->eps_fn = fn;
    s->eps_user = user;
    return RGPU_OK;
}

extern "C" int rgpu_sim_resolve_time(rgpu_sim* s, double* ms, int64_t* calls) {
    if (!s || !ms || !calls) return RGPU_ERR_ARG;
    *ms = s->resolve_ms;
    *calls = s->resolve_calls;
    return RGPU_OK;
}

// Shuffle (src/collision.c:336-342) and resolve (:343-404) the pairs of the last search.
static int resolve_pairs(rgpu_sim* s) {
    rgpu_config& c = s->cfg;
    const size_t n = s->n_pairs;
    std::vector<rgpu_collision> pairs(n);
    RGPU_CUDA(s, cudaMemcpyAsync(pairs.data(), s->dev_pairs, sizeof(rgpu_collision) * n, cudaMemcpyDeviceToHost, s->stream));
    RGPU_CUDA(s, cudaStreamSynchronize(s->stream));
    for (size_t i = 0; i < n; i++) {
        const size_t nw = (size_t)rand_r(&c.rand_seed) % n;
        std::swap(pairs[i], pairs[nw]);
    }
    if (c.collision_resolve == RGPU_RESOLVE_NONE) return RGPU_OK;
    if (c.collision_resolve == RGPU_RESOLVE_HALT) {   // src/collision.c:667-672
        c.status = 7;
        return RGPU_OK;
    }
    // hardsphere: bring the touched particles to the host
    std::vector<int> ids;
    std::unordered_map<int, int> slot;
    for (const auto& q : pairs) {
        for (size_t v : {q.p1, q.p2}) {
            if (slot.emplace((int)v, (int)ids.size()).second) ids.push_back((int)v);
        }
    }
    const int nt = (int)ids.size();
    int* d_ids = nullptr;
    double* d_buf = nullptr;
    RGPU_CUDA(s, cudaMalloc(&d_ids, sizeof(int) * nt));
    const cudaError_t e2 = cudaMalloc(&d_buf, sizeof(double) * 8 * nt);
    if (e2 != cudaSuccess) { cudaFree(d_ids); return check_cuda(s, e2, "resolve buffer"); }
    std::vector<Body> b(nt);
    cudaMemcpyAsync(d_ids, ids.data(), sizeof(int) * nt, cudaMemcpyHostToDevice, s->stream);
    gather_touched<<<(nt + 127) / 128, 128, 0, s->stream>>>(s->p, d_ids, nt, d_buf);
    cudaMemcpyAsync(b.data(), d_buf, sizeof(double) * 8 * nt, cudaMemcpyDeviceToHost, s->stream);
    cudaStreamSynchronize(s->stream);
    for (const auto& q : pairs)
        hardsphere(b[slot[(int)q.p1]], b[slot[(int)q.p2]], q.gb, c.coefficient_of_restitution, s->eps_fn,
                   s->eps_user, c.minimum_collision_velocity, c.collisions_log_n, c.collisions_plog);
    cudaMemcpyAsync(d_buf, b.data(), sizeof(double) * 8 * nt, cudaMemcpyHostToDevice, s->stream);
    scatter_velocities<<<(nt + 127) / 128, 128, 0, s->stream>>>(s->p, d_ids, nt, d_buf);
    g_launches += 2;
    const cudaError_t e3 = cudaStreamSynchronize(s->stream);
    cudaFree(d_ids);
    cudaFree(d_buf);
    if (e3 != cudaSuccess) return check_cuda(s, e3, "resolve");
    return RGPU_OK;
}

void collide_free(rgpu_sim* s) {
    cudaFree(s->pc_count); cudaFree(s->pc_off); cudaFree(s->dp_pairs);
    s->pc_count = nullptr; s->pc_off = nullptr; s->dp_pairs = nullptr;
}
