// Octree gravity and tree collision search on sm_103a (src/tree.c,
// src/gravity.c:47-106, src/collision.c:197-269 and :422-503 of REBOUND 5.0.0).
//
// Build, GB300-style and without pointers:
//   1. keys: per particle, the root box and up to D octant digits found by
//      descending from the root centre with the reference's own comparisons
//      (p < centre) and centre updates (parent +/- w_child/2), so cell
//      membership is bit-identical to the reference's insertion tree;
//   2. a stable LSD radix sort of the 64-bit keys (8-bit digits, warp-match
//      ranking), particle indices carried along;
//   3. top-down, level by level: each internal cell (>= 2 particles) splits
//      its sorted range into its non-empty octants by binary search and
//      allocates its children contiguously, in octant order;
//   4. bottom-up mass and centre of mass, children summed in octant order with
//      the reference's expression order (no FMA contraction in this unit).
// The walk keeps the reference's order (ghost boxes, roots by index, octants
// 0..7, depth first) with an explicit stack, so accelerations are
// bit-identical to the reference's serial build.
#include "rgpu_internal.cuh"
#include "exactfp.cuh"
#include <algorithm>
#include <cmath>
#include <vector>

struct TreeBuffers {
    size_t cap = 0;                 // particles
    unsigned long long* keys = nullptr;
    unsigned long long* keys_alt = nullptr;
    int* idx = nullptr;
    int* idx_alt = nullptr;
    unsigned int* hist = nullptr;   // radix histograms [256][blocks]
    size_t hist_cap = 0;
    // cells (structure of arrays)
    size_t ccap = 0;
    double *cx = nullptr, *cy = nullptr, *cz = nullptr, *cw = nullptr;
    double* cw2 = nullptr;          // w * w, rounded as the walk's opening test computes it
    double *cm = nullptr, *cmx = nullptr, *cmy = nullptr, *cmz = nullptr;
    double *cqxx = nullptr, *cqxy = nullptr, *cqxz = nullptr, *cqyy = nullptr, *cqyz = nullptr;  // quadrupole
    int* cstart = nullptr;          // range in sorted order
    int* cend = nullptr;
    int* cfirst = nullptr;          // first child (children contiguous, octant order)
    int* cnchild = nullptr;
    int* cpt = nullptr;             // leaf: particle index; internal: -(count); empty root: INT_MIN
    int* cdepth = nullptr;
    unsigned long long* cpath = nullptr;
    int* counter = nullptr;         // device allocation counter
    std::vector<int> level_begin;   // host: cell index range per level
    int n_cells = 0;
    int D = 0;
    int n_root = 0;
    // collision output
    int* pair_count = nullptr;
    long long* pair_off = nullptr;
    rgpu_collision* pairs = nullptr;
    size_t pairs_cap = 0;
    double* r_top = nullptr;        // per-block top-2 radii, then the largest squared speed
    void* sweep = nullptr;          // split mode: per-root monopole records
    size_t sweep_cap = 0;
};

namespace {

constexpr int kB = 256;

struct BoxGeom {
    double root_size, bx, by, bz;
    int nx, ny, nz;
    int D;            // key depth
    int shift;        // 3 * D
};

// --- 1. keys --------------------------------------------------------------
__global__ void make_keys(ParticlesSoA p, int N, BoxGeom g, unsigned long long* keys, int* idx, uint32_t* status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double x = p.x[i], y = p.y[i], z = p.z[i];
    idx[i] = i;
    // src/tree.c:262-268 (outside box) and :66-69 (non-finite)
    if (fabs(x) > g.root_size * (double)g.nx / 2. || fabs(y) > g.root_size * (double)g.ny / 2. ||
        fabs(z) > g.root_size * (double)g.nz / 2.) {
        atomicOr(status, DEV_ERR_OUT_OF_BOX);
        keys[i] = ~0ull;
        return;
    }
    if (!isfinite(x) || !isfinite(y) || !isfinite(z)) {
        atomicOr(status, DEV_ERR_NONFINITE);
        keys[i] = ~0ull;
        return;
    }
    // root box, src/particle.c:119-126
    const int ri = ((int)floor((x + g.root_size * (double)g.nx / 2.) / g.root_size) + g.nx) % g.nx;
    const int rj = ((int)floor((y + g.root_size * (double)g.ny / 2.) / g.root_size) + g.ny) % g.ny;
    const int rk = ((int)floor((z + g.root_size * (double)g.nz / 2.) / g.root_size) + g.nz) % g.nz;
    const unsigned long long root = (unsigned long long)((rk * g.ny + rj) * g.nx + ri);
    // root cell centre, src/tree.c:87-98
    const int ci = ((int)floor((x + g.bx / 2.) / g.root_size)) % g.nx;
    const int cj = ((int)floor((y + g.by / 2.) / g.root_size)) % g.ny;
    const int ck = ((int)floor((z + g.bz / 2.) / g.root_size)) % g.nz;
    double cx = -g.bx / 2. + g.root_size * (0.5 + (double)ci);
    double cy = -g.by / 2. + g.root_size * (0.5 + (double)cj);
    double cz = -g.bz / 2. + g.root_size * (0.5 + (double)ck);
    double w = g.root_size;
    unsigned long long path = 0;
    for (int d = 0; d < g.D; d++) {
        int o = 0;
        if (x < cx) o += 1;                 // src/tree.c:136-142
        if (y < cy) o += 2;
        if (z < cz) o += 4;
        path = (path << 3) | (unsigned long long)o;
        const double wc = w / 2.;           // src/tree.c:100-103
        cx = cx + wc / 2. * ((o & 1) == 0 ? 1. : -1);
        cy = cy + wc / 2. * ((o & 2) == 0 ? 1. : -1);
        cz = cz + wc / 2. * ((o & 4) == 0 ? 1. : -1);
        w = wc;
    }
    keys[i] = (root << g.shift) | path;
}

// --- 2. stable LSD radix sort, 8-bit digits ----------------------------------
constexpr int kSortItems = 4;                      // elements per thread
constexpr int kSortTile = kB * kSortItems;

__global__ void radix_hist(const unsigned long long* __restrict__ keys, int N, int shift, unsigned int* hist, int nblk) {
    __shared__ unsigned int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile;
    for (int q = 0; q < kSortItems; q++) {
        const int i = base + q * kB + threadIdx.x;
        if (i < N) atomicAdd(&h[(keys[i] >> shift) & 255], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * nblk + blockIdx.x] = h[threadIdx.x];    // digit-major
}

// Exclusive scan of the digit-major histogram (one CTA; n = 256 * nblk).
__global__ void radix_scan(unsigned int* hist, int n) {
    __shared__ unsigned int part[kB];
    const int per = (n + kB - 1) / kB;
    const int b0 = threadIdx.x * per;
    unsigned int s = 0;
    for (int k = 0; k < per; k++) if (b0 + k < n) s += hist[b0 + k];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < kB; off <<= 1) {
        const unsigned int v = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned int run = threadIdx.x ? part[threadIdx.x - 1] : 0u;
    for (int k = 0; k < per; k++) {
        if (b0 + k < n) {
            const unsigned int v = hist[b0 + k];
            hist[b0 + k] = run;
            run += v;
        }
    }
}

// Stable scatter: elements of a tile keep their order within each digit.
// Each of the kSortItems rounds ranks 256 consecutive elements with
// __match_any_sync inside warps and per-warp digit counters across warps.
__global__ void radix_scatter(const unsigned long long* __restrict__ keys, const int* __restrict__ idx, int N,
                              int shift, const unsigned int* __restrict__ hist, int nblk,
                              unsigned long long* __restrict__ okeys, int* __restrict__ oidx) {
    __shared__ unsigned int base[256];
    __shared__ unsigned int wcount[kB / 32][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    base[threadIdx.x] = hist[threadIdx.x * nblk + blockIdx.x];
    for (int q = 0; q < kSortItems; q++) {
        const int i = blockIdx.x * kSortTile + q * kB + threadIdx.x;
        const bool live = i < N;
        const unsigned long long k = live ? keys[i] : 0ull;
        const unsigned d = live ? (unsigned)((k >> shift) & 255) : 256u + lane;   // dead lanes never match
        for (int w = 0; w < kB / 32; w++) wcount[w][threadIdx.x] = 0;
        __syncthreads();
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned lower = peers & ((1u << lane) - 1u);
        const int rank_in_warp = __popc(lower);
        if (live && lower == 0) wcount[warp][d] = __popc(peers);   // leader records the warp's count
        __syncthreads();
        if (live) {
            unsigned before = 0;
            for (int w = 0; w < warp; w++) before += wcount[w][d];
            const unsigned dst = base[d] + before + rank_in_warp;
            okeys[dst] = k;
            oidx[dst] = idx[i];
        }
        __syncthreads();
        // advance the per-digit base by this round's total
        unsigned tot = 0;
        for (int w = 0; w < kB / 32; w++) tot += wcount[w][threadIdx.x];
        __syncthreads();
        base[threadIdx.x] += tot;
        __syncthreads();
    }
}

// --- 3. cells ------------------------------------------------------------------
struct CellArrays {
    double *x, *y, *z, *w, *m, *mx, *my, *mz;
    double* w2;                               // w * w (the opening test's left side, same rounding)
    double *qxx, *qxy, *qxz, *qyy, *qyz;     // mass quadrupole (q_zz = -q_xx - q_yy)
    int *start, *end, *first, *nchild, *pt, *depth;
    unsigned long long* path;
};

__global__ void init_roots(CellArrays c, int n_root, BoxGeom g) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_root) return;
    const int ri = r % g.nx, rj = (r / g.nx) % g.ny, rk = r / (g.nx * g.ny);
    c.x[r] = -g.bx / 2. + g.root_size * (0.5 + (double)ri);
    c.y[r] = -g.by / 2. + g.root_size * (0.5 + (double)rj);
    c.z[r] = -g.bz / 2. + g.root_size * (0.5 + (double)rk);
    c.w[r] = g.root_size;
    c.w2[r] = g.root_size * g.root_size;
    c.start[r] = 0; c.end[r] = 0;
    c.first[r] = -1; c.nchild[r] = 0;
    c.pt[r] = INT_MIN;
    c.depth[r] = 0;
    c.path[r] = 0;
}

__global__ void root_ranges(const unsigned long long* __restrict__ keys, const int* __restrict__ idx, int N,
                            int shift, CellArrays c, int n_root) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const unsigned long long r = keys[i] >> shift;
    if (r >= (unsigned long long)n_root) return;          // invalid particle (status already set)
    if (i == 0 || (keys[i - 1] >> shift) != r) c.start[r] = i;
    if (i == N - 1 || (keys[i + 1] >> shift) != r) {
        c.end[r] = i + 1;
    }
}

__global__ void root_finish(const int* __restrict__ idx, CellArrays c, int n_root) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_root) return;
    const int n = c.end[r] - c.start[r];
    if (n <= 0) { c.pt[r] = INT_MIN; return; }
    c.pt[r] = n == 1 ? idx[c.start[r]] : -n;
}

__device__ __forceinline__ int digit_at(unsigned long long key, int depth, int D) {
    return (int)((key >> (3 * (D - depth))) & 7ull);
}

// Split each internal cell of one level into its non-empty octants.
__global__ void split_level(const unsigned long long* __restrict__ keys, const int* __restrict__ idx,
                            ParticlesSoA p, CellArrays c, int lvl_begin, int lvl_end, int D, int* counter,
                            int ccap, uint32_t* status) {
    const int cell = lvl_begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= lvl_end) return;
    const int s = c.start[cell], e = c.end[cell];
    if (e - s < 2) return;                                   // leaf or empty root
    const int d = c.depth[cell];
    if (d >= D) {
        // Key exhausted: equal paths.  Same coordinates is the reference's error
        // (src/tree.c:119-123); otherwise the device key is too short.
        const int a = idx[s], b = idx[s + 1];
        if (p.x[a] == p.x[b] && p.y[a] == p.y[b] && p.z[a] == p.z[b]) atomicOr(status, DEV_ERR_DUPLICATE);
        else atomicOr(status, DEV_ERR_TREE_DEPTH);
        return;
    }
    int bounds[9];
    bounds[0] = s;
    for (int o = 1; o < 8; o++) {                           // lower_bound of digit o in [s, e)
        int lo = bounds[o - 1], hi = e;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (digit_at(keys[mid], d + 1, D) < o) lo = mid + 1; else hi = mid;
        }
        bounds[o] = lo;
    }
    bounds[8] = e;
    int nc = 0;
    for (int o = 0; o < 8; o++) nc += bounds[o + 1] > bounds[o];
    const int first = atomicAdd(counter, nc);
    if (first + nc > ccap) { atomicOr(status, DEV_ERR_OVERFLOW); return; }
    c.first[cell] = first;
    c.nchild[cell] = nc;
    const double w = c.w[cell];
    int q = first;
    for (int o = 0; o < 8; o++) {
        const int cs = bounds[o], ce = bounds[o + 1];
        if (ce <= cs) continue;
        const double wc = w / 2.;
        c.w[q] = wc;
        c.w2[q] = wc * wc;
        c.x[q] = c.x[cell] + wc / 2. * ((o & 1) == 0 ? 1. : -1);
        c.y[q] = c.y[cell] + wc / 2. * ((o & 2) == 0 ? 1. : -1);
        c.z[q] = c.z[cell] + wc / 2. * ((o & 4) == 0 ? 1. : -1);
        c.start[q] = cs; c.end[q] = ce;
        c.first[q] = -1; c.nchild[q] = 0;
        c.pt[q] = (ce - cs == 1) ? idx[cs] : -(ce - cs);
        c.depth[q] = d + 1;
        c.path[q] = (c.path[cell] << 3) | (unsigned long long)o;
        q++;
    }
}

// --- 4. mass, centre of mass and (quad) the mass quadrupole, src/tree.c:147-207 ------
__global__ void reduce_level(ParticlesSoA p, CellArrays c, int lvl_begin, int lvl_end, int quad) {
    const int cell = lvl_begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= lvl_end) return;
    const int pt = c.pt[cell];
    if (quad) { c.qxx[cell] = 0.; c.qxy[cell] = 0.; c.qxz[cell] = 0.; c.qyy[cell] = 0.; c.qyz[cell] = 0.; }
    if (pt == INT_MIN) { c.m[cell] = 0.; c.mx[cell] = c.my[cell] = c.mz[cell] = 0.; return; }
    if (pt >= 0) {
        c.m[cell] = p.m[pt]; c.mx[cell] = p.x[pt]; c.my[cell] = p.y[pt]; c.mz[cell] = p.z[pt];
        return;
    }
    double m = 0., mx = 0., my = 0., mz = 0.;
    const int f = c.first[cell], n = c.nchild[cell];
    for (int k = 0; k < n; k++) {
        const double dm = c.m[f + k];
        mx += c.mx[f + k] * dm;
        my += c.my[f + k] * dm;
        mz += c.mz[f + k] * dm;
        m += dm;
    }
    if (m > 0) { mx /= m; my /= m; mz /= m; }
    c.m[cell] = m; c.mx[cell] = mx; c.my[cell] = my; c.mz[cell] = mz;
    if (!quad) return;
    // Hernquist (1987): the children's quadrupoles shifted to this cell's centre of
    // mass, accumulated in octant order (src/tree.c:180-198)
    double qxx = 0., qxy = 0., qxz = 0., qyy = 0., qyz = 0.;
    for (int k = 0; k < n; k++) {
        const double dm = c.m[f + k];
        const double qx = c.mx[f + k] - mx, qy = c.my[f + k] - my, qz = c.mz[f + k] - mz;
        const double qr2 = qx * qx + qy * qy + qz * qz;
        qxx += c.qxx[f + k] + dm * (3. * qx * qx - qr2);
        qxy += c.qxy[f + k] + dm * 3. * qx * qy;
        qxz += c.qxz[f + k] + dm * 3. * qx * qz;
        qyy += c.qyy[f + k] + dm * (3. * qy * qy - qr2);
        qyz += c.qyz[f + k] + dm * 3. * qy * qz;
    }
    c.qxx[cell] = qxx; c.qxy[cell] = qxy; c.qxz[cell] = qxz; c.qyy[cell] = qyy; c.qyz[cell] = qyz;
}

// --- 5. the walk -----------------------------------------------------------------
struct GhostArr {
    int n;
    double off[125][6];
};

constexpr int kStack = 192;

// Walk constants.  oa2_k: opening_angle2 = 2^oa2_k exactly (kNoPow2 otherwise),
// which turns the opening test into an integer comparison.
constexpr int kNoPow2 = 1 << 20;

struct WalkConst {
    double G, eps2, oa2;
    int oa2_k;
};

static int pow2_exponent(double v) {
    int e = 0;
    const double m = frexp(v, &e);
    return (v > 0. && m == 0.5 && e > -1000 && e < 1000) ? e - 1 : kNoPow2;
}

static WalkConst walk_const(const rgpu_config& cf, double eps2) {
    WalkConst w;
    w.G = cf.G;
    w.eps2 = eps2;
    w.oa2 = cf.opening_angle2;
    w.oa2_k = pow2_exponent(cf.opening_angle2);
    return w;
}

// Rare cases of the visit below in hardware FP64: operands or results outside
// the normal range (a zero displacement, a zero radius, subnormal or
// overflowing squares).  Kept out of line so that the common path issues no
// FP64 instruction for them.
__device__ __noinline__ double r2_fp64(double dx, double dy, double dz) { return dx * dx + dy * dy + dz * dz; }

__device__ __noinline__ double pf_fp64(double r2, double eps2, double G, double m) {
    const double rr = sqrt(r2 + eps2);
    return -G / (rr * rr * rr) * m;
}

__device__ __noinline__ int open_fp64(double w2, double oa2, double r2) { return w2 > oa2 * r2; }

// One root's subtree for particle i, shifted to (sx, sy, sz): the reference's
// depth-first descent and force sum (src/tree.c:275-328; QUAD adds the far-cell
// quadrupole term of src/tree.c:293-306).  Every FP64 operation of the visit is
// rounded exactly as the reference rounds it.  The squares, the two sums of r^2,
// the opening test, the square root, r^3 and the division run on the integer
// pipes (exactfp); the displacement, r^2 + eps^2, G m / r^3 and the three
// accumulations stay on the FP64 pipe, which then carries 11 of the visit's 22
// FP64 operations (the split that measured fastest: moving r^2 + eps^2 to the
// integer pipes, or r^3 or the sums of r^2 to the FP64 pipe, was slower).
template <bool QUAD>
__device__ __forceinline__ void walk_root(int r, int i, double sx, double sy, double sz, const CellArrays& c,
                                          const WalkConst& w, int* stack, double& ax, double& ay, double& az,
                                          uint32_t* status) {
    // The root itself is visited without a stack round trip; only opened cells
    // push their children.
    int sp = 0, q = r;
    for (;;) {
        {
            const double dx = sx - c.mx[q], dy = sy - c.my[q], dz = sz - c.mz[q];
            exactfp::u32 special = 0;
            double r2 = exactfp::add_pos_try(
                exactfp::add_pos_try(exactfp::sqr_try(dx, special), exactfp::sqr_try(dy, special), special),
                exactfp::sqr_try(dz, special), special);
            if (special) r2 = r2_fp64(dx, dy, dz);
            const int pt = c.pt[q];
            if (pt < 0) {
                const double w2 = c.w2[q];
                int open = w.oa2_k != kNoPow2 ? exactfp::gt_scaled_pow2(w2, r2, w.oa2_k) : -1;
                if (open < 0) open = open_fp64(w2, w.oa2, r2);
                if (open) {
                    const int f = c.first[q], n = c.nchild[q];
                    if (sp + n > kStack) { atomicOr(status, DEV_ERR_STACK); return; }
                    for (int k = n - 1; k >= 0; k--) stack[sp++] = f + k;
                    goto next;
                }
                if (QUAD) {
                    const double rr = exactfp::sqrt_rn(r2 + w.eps2);
                    const double pf = exactfp::div_rn(-w.G, rr * rr * rr) * c.m[q];
                    const double qxx = c.qxx[q], qxy = c.qxy[q], qxz = c.qxz[q], qyy = c.qyy[q], qyz = c.qyz[q];
                    const double qzz = -qxx - qyy;
                    double qpf = exactfp::div_rn(w.G, rr * rr * rr * rr * rr);
                    ax += qpf * (dx * qxx + dy * qxy + dz * qxz);
                    ay += qpf * (dx * qxy + dy * qyy + dz * qyz);
                    az += qpf * (dx * qxz + dy * qyz + dz * qzz);
                    const double mrr = dx * dx * qxx + dy * dy * qyy + dz * dz * qzz + 2. * dx * dy * qxy +
                                       2. * dx * dz * qxz + 2. * dy * dz * qyz;
                    qpf *= exactfp::div_rn(-5.0, 2.0 * rr * rr) * mrr;
                    ax += (qpf + pf) * dx; ay += (qpf + pf) * dy; az += (qpf + pf) * dz;
                    goto next;
                }
            } else if (pt == i) {
                goto next;
            }
            exactfp::u32 special2 = 0;
            const double s2 = r2 + w.eps2;
            const double rr = exactfp::sqrt_try(s2, special2);
            const double rr3 = exactfp::mul_try(exactfp::sqr_try(rr, special2), rr, special2);
            double pf = exactfp::div_try(-w.G, rr3, special2) * c.m[q];
            if (special2) pf = pf_fp64(r2, w.eps2, w.G, c.m[q]);
            ax += pf * dx; ay += pf * dy; az += pf * dz;
        }
    next:
        if (sp == 0) return;
        q = stack[--sp];
    }
}

// Threads take particles in key order (`order`, the sorted index array of the
// build), so a warp's 32 particles are neighbours in space: they see the same
// roots far or near and descend the same cells, which keeps the warp converged.
// Each particle's own sum keeps the reference's order, so results do not change.
template <bool QUAD>
__global__ void __launch_bounds__(128) walk_exact(ParticlesSoA p, int N, const int* __restrict__ order, CellArrays c,
                                                  int n_root, const GhostArr* __restrict__ gh, WalkConst w,
                                                  uint32_t* status) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    const int i = order[k];
    int stack[kStack];
    double ax = 0., ay = 0., az = 0.;
    const double px = p.x[i], py = p.y[i], pz = p.z[i];
    for (int g = 0; g < gh->n; g++) {
        const double sx = gh->off[g][0] + px, sy = gh->off[g][1] + py, sz = gh->off[g][2] + pz;
        for (int r = 0; r < n_root; r++) {
            if (c.pt[r] == INT_MIN) continue;
            walk_root<QUAD>(r, i, sx, sy, sz, c, w, stack, ax, ay, az, status);
        }
    }
    p.ax[i] = ax; p.ay[i] = ay; p.az[i] = az;
}

// --- split mode: near-window walk + far-root monopole sweep ----------------------------
// A root whose index differs from the shifted particle's (virtual) root index by
// more than K = ceil(1/theta) + 1 in any direction lies at least K-1 >= 1/theta
// root widths away, so the opening test w^2 > theta^2 r^2 (src/tree.c:285) fails
// for it and the reference uses exactly its monopole.  The split mode walks the
// window |offset| <= K with the reference's FP64 descent and sweeps all other
// roots as monopoles in a tiled kernel: FP64 displacement formed from two-float
// splits, FP32 force, compensated FP32 accumulation.
// Roots in pairs for the packed FP32x2 sweep (80 B): COM hi / lo two-float splits
// and G m of both roots, and for each root its index position (ix | iy << 11 |
// iz << 22) and its leaf particle (-1 for a cell or an empty root).  Empty roots
// and the partner of the last root of an odd count are massless.
struct __align__(16) RootPair {
    float4 a, b, c, d;   // (xh0, xh1, yh0, yh1), (zh0, zh1, Gm0, Gm1), (xl0, xl1, yl0, yl1), (zl0, zl1, 0, 0)
    int4 meta;           // pos0, pos1, leaf0, leaf1
};

__global__ void build_root_pairs(CellArrays c, int n_root, BoxGeom g, double G, RootPair* __restrict__ out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (n_root + 1) / 2) return;
    float xh[2], yh[2], zh[2], gm[2], xl[2], yl[2], zl[2];
    int pos[2], leaf[2];
    for (int k = 0; k < 2; k++) {
        const int r = 2 * q + k;
        const bool full = r < n_root && c.pt[r] != INT_MIN;
        const double mx = full ? c.mx[r] : 0., my = full ? c.my[r] : 0., mz = full ? c.mz[r] : 0.;
        xh[k] = (float)mx; yh[k] = (float)my; zh[k] = (float)mz;
        xl[k] = (float)(mx - (double)xh[k]); yl[k] = (float)(my - (double)yh[k]); zl[k] = (float)(mz - (double)zh[k]);
        gm[k] = full ? (float)(G * c.m[r]) : 0.f;
        const int rr = r < n_root ? r : 0;
        pos[k] = (rr % g.nx) | (((rr / g.nx) % g.ny) << 11) | ((rr / (g.nx * g.ny)) << 22);
        leaf[k] = (full && c.pt[r] >= 0) ? c.pt[r] : -1;
    }
    RootPair P;
    P.a = make_float4(xh[0], xh[1], yh[0], yh[1]);
    P.b = make_float4(zh[0], zh[1], gm[0], gm[1]);
    P.c = make_float4(xl[0], xl[1], yl[0], yl[1]);
    P.d = make_float4(zl[0], zl[1], 0.f, 0.f);
    P.meta = make_int4(pos[0], pos[1], leaf[0], leaf[1]);
    out[q] = P;
}

__device__ __forceinline__ void virtual_root(const BoxGeom& g, double sx, double sy, double sz, int& ix, int& iy,
                                             int& iz) {
    ix = (int)floor((sx + g.bx / 2.) / g.root_size);
    iy = (int)floor((sy + g.by / 2.) / g.root_size);
    iz = (int)floor((sz + g.bz / 2.) / g.root_size);
}

__global__ void __launch_bounds__(128) walk_near(ParticlesSoA p, int N, const int* __restrict__ order, CellArrays c,
                                                 BoxGeom geo, const GhostArr* __restrict__ gh, WalkConst w, int K,
                                                 uint32_t* status) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;      // particles in key order, as walk_exact
    if (k >= N) return;
    const int i = order[k];
    int stack[kStack];
    double ax = 0., ay = 0., az = 0.;
    const double px = p.x[i], py = p.y[i], pz = p.z[i];
    for (int g = 0; g < gh->n; g++) {
        const double sx = gh->off[g][0] + px, sy = gh->off[g][1] + py, sz = gh->off[g][2] + pz;
        int ixv, iyv, izv;
        virtual_root(geo, sx, sy, sz, ixv, iyv, izv);
        const int x0 = max(0, ixv - K), x1 = min(geo.nx - 1, ixv + K);
        const int y0 = max(0, iyv - K), y1 = min(geo.ny - 1, iyv + K);
        const int z0 = max(0, izv - K), z1 = min(geo.nz - 1, izv + K);
        for (int rk = z0; rk <= z1; rk++)
        for (int rj = y0; rj <= y1; rj++)
        for (int ri = x0; ri <= x1; ri++) {
            const int r = (rk * geo.ny + rj) * geo.nx + ri;
            if (c.pt[r] == INT_MIN) continue;
            walk_root<false>(r, i, sx, sy, sz, c, w, stack, ax, ay, az, status);
        }
    }
    p.ax[i] = ax; p.ay[i] = ay; p.az[i] = az;
}

constexpr int kSweepTile = 256;              // particles per CTA
constexpr int kSweepPairs = kSweepTile / 2;   // root pairs per shared-memory tile
constexpr int kSweepSub = 32;                 // root pairs summed in FP32 before a fold

// Far roots of every particle and ghost box: the packed FP32x2 pipe evaluates two
// roots per instruction (displacement from the two-float splits, r^2, G m / r^3,
// the accumulation); the roots of the particle's near window (walked exactly by
// walk_near) and its own leaf root contribute zero.  Terms are summed in FP32 over
// 32 root pairs and each sum is folded into a compensated FP32 pair.
__global__ void __launch_bounds__(kSweepTile) sweep_far(ParticlesSoA p, int N, const RootPair* __restrict__ roots,
                                                        int n_pair, BoxGeom geo, const GhostArr* __restrict__ gh,
                                                        double eps2, int K) {
    __shared__ RootPair tile[kSweepPairs];
    const int i = blockIdx.x * kSweepTile + threadIdx.x;
    const bool live = i < N;
    const double px = live ? p.x[i] : 0., py = live ? p.y[i] : 0., pz = live ? p.z[i] : 0.;
    const float ef = (float)eps2;
    const float2 e2 = make_float2(ef, ef);
    const unsigned span = 2u * (unsigned)K;
    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    for (int qt = 0; qt < n_pair; qt += kSweepPairs) {
        __syncthreads();
        if (threadIdx.x < kSweepPairs) {
            const int ql = qt + threadIdx.x;
            if (ql < n_pair) {
                tile[threadIdx.x] = roots[ql];
            } else {
                RootPair Z;
                Z.a = Z.b = Z.c = Z.d = make_float4(0.f, 0.f, 0.f, 0.f);
                Z.meta = make_int4(0, 0, -1, -1);
                tile[threadIdx.x] = Z;
            }
        }
        __syncthreads();
        const int nq = min(kSweepPairs, n_pair - qt);
        for (int g = 0; g < gh->n; g++) {
            const double gx = gh->off[g][0] + px, gy = gh->off[g][1] + py, gz = gh->off[g][2] + pz;
            int ixv, iyv, izv;
            virtual_root(geo, gx, gy, gz, ixv, iyv, izv);
            const int bx = ixv - K, by = iyv - K, bz = izv - K;    // near window corner
            const float hx = (float)gx, hy = (float)gy, hz = (float)gz;
            const float lx = (float)(gx - (double)hx), ly = (float)(gy - (double)hy), lz = (float)(gz - (double)hz);
            const float2 nxh = make_float2(-hx, -hx), nyh = make_float2(-hy, -hy), nzh = make_float2(-hz, -hz);
            const float2 nxl = make_float2(-lx, -lx), nyl = make_float2(-ly, -ly), nzl = make_float2(-lz, -lz);
            for (int qs = 0; qs < nq; qs += kSweepSub) {
                const int qe = min(nq, qs + kSweepSub);
                float2 ax = make_float2(0.f, 0.f), ay = ax, az = ax;
#pragma unroll 4
                for (int q = qs; q < qe; q++) {
                    const RootPair J = tile[q];
                    const float2 dx = __fadd2_rn(__fadd2_rn(make_float2(J.a.x, J.a.y), nxh),
                                                 __fadd2_rn(make_float2(J.c.x, J.c.y), nxl));
                    const float2 dy = __fadd2_rn(__fadd2_rn(make_float2(J.a.z, J.a.w), nyh),
                                                 __fadd2_rn(make_float2(J.c.z, J.c.w), nyl));
                    const float2 dz = __fadd2_rn(__fadd2_rn(make_float2(J.b.x, J.b.y), nzh),
                                                 __fadd2_rn(make_float2(J.d.x, J.d.y), nzl));
                    const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __ffma2_rn(dz, dz, e2)));
                    const float2 ri = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
                    float2 s = __fmul2_rn(__fmul2_rn(ri, ri), __fmul2_rn(make_float2(J.b.z, J.b.w), ri));
                    // near window: every index within K of the virtual root's
                    const int p0 = J.meta.x, p1 = J.meta.y;
                    const bool near0 = (unsigned)((p0 & 2047) - bx) <= span && (unsigned)(((p0 >> 11) & 2047) - by) <= span &&
                                       (unsigned)((p0 >> 22) - bz) <= span;
                    const bool near1 = (unsigned)((p1 & 2047) - bx) <= span && (unsigned)(((p1 >> 11) & 2047) - by) <= span &&
                                       (unsigned)((p1 >> 22) - bz) <= span;
                    s.x = (near0 || J.meta.z == i || J.b.z == 0.f) ? 0.f : s.x;
                    s.y = (near1 || J.meta.w == i || J.b.w == 0.f) ? 0.f : s.y;
                    ax = __ffma2_rn(s, dx, ax);
                    ay = __ffma2_rn(s, dy, ay);
                    az = __ffma2_rn(s, dz, az);
                }
                const float tx = ax.x + ax.y, ty = ay.x + ay.y, tz = az.x + az.y;
                float t, y;
                y = tx - cx; t = sx + y; cx = (t - sx) - y; sx = t;
                y = ty - cy; t = sy + y; cy = (t - sy) - y; sy = t;
                y = tz - cz; t = sz + y; cz = (t - sz) - y; sz = t;
            }
        }
    }
    if (!live) return;
    p.ax[i] += (double)sx - (double)cx;
    p.ay[i] += (double)sy - (double)cy;
    p.az[i] += (double)sz - (double)cz;
}

// --- collision search (src/collision.c:197-269, :422-503) ----------------------------
// Roots farther than the search radius from the shifted particle cannot pass the
// descent test r < r1 + r2nd + (sqrt(3)/2) w, so each particle scans only the
// window of root boxes around it (index order preserved, same pair set and order).
// LINE = true: the LINETREE search (src/collision.c:270-330, 506-572), which tests
// the straight paths of the last step (dt_last_done) instead of the overlap now and
// descends while r < r1 + dt |v1| + maxdrift + (sqrt(3)/2) w.
template <bool LINE>
__device__ __forceinline__ int tree_pairs_one(int i, ParticlesSoA p, CellArrays c, BoxGeom g,
                                              const GhostArr* __restrict__ gh, int nring, double r2nd, double rmax,
                                              double dtl, double vmax2, rgpu_collision* out, long long base,
                                              int* stack, uint32_t* status) {
    const double p1x = p.x[i], p1y = p.y[i], p1z = p.z[i];
    const double p1vx = p.vx[i], p1vy = p.vy[i], p1vz = p.vz[i], p1r = p.r[i];
    double maxdrift = 0., p1r_dtv = 0.;
    if (LINE) {
        maxdrift = dtl * sqrt(vmax2);
        p1r_dtv = p1r + dtl * sqrt(p1vx * p1vx + p1vy * p1vy + p1vz * p1vz);
    }
    int found = 0;
    for (int g0 = 0; g0 < nring; g0++) {
        const double* gb = gh->off[g0];
        const double sx = gb[0] + p1x, sy = gb[1] + p1y, sz = gb[2] + p1z;
        const double svx = gb[3] + p1vx, svy = gb[4] + p1vy, svz = gb[5] + p1vz;
        // A root can only contribute if its cell centre is within the descent radius
        // of the shifted particle or, for a one-particle root, if that particle can
        // pass the pair test (for LINE: the end-of-step distance is at most the
        // radii plus the relative path length |dt| (|v1 + v_gb| + v_max)).
        double reach;
        if (LINE) {
            const double adt = fabs(dtl);
            const double desc = fabs(p1r_dtv) + fabs(maxdrift) + 0.8660254037844387 * g.root_size;
            const double leaf = p1r + rmax + adt * (sqrt(svx * svx + svy * svy + svz * svz) + sqrt(vmax2));
            reach = fmax(desc, leaf) * (1. + 1e-12);
        } else {
            reach = p1r + fmax(rmax, r2nd + 0.8660254037844387 * g.root_size);
        }
        const int K = (int)ceil(reach / g.root_size) + 2;
        const int ixv = (int)floor((sx + g.bx / 2.) / g.root_size);
        const int iyv = (int)floor((sy + g.by / 2.) / g.root_size);
        const int izv = (int)floor((sz + g.bz / 2.) / g.root_size);
        const int x0 = max(0, ixv - K), x1 = min(g.nx - 1, ixv + K);
        const int y0 = max(0, iyv - K), y1 = min(g.ny - 1, iyv + K);
        const int z0 = max(0, izv - K), z1 = min(g.nz - 1, izv + K);
        for (int rk = z0; rk <= z1; rk++)
        for (int rj = y0; rj <= y1; rj++)
        for (int ri = x0; ri <= x1; ri++) {
            const int r = (rk * g.ny + rj) * g.nx + ri;
            if (c.pt[r] == INT_MIN) continue;
            int sp = 0;
            stack[sp++] = r;
            while (sp > 0) {
                const int q = stack[--sp];
                const int pt = c.pt[q];
                if (pt >= 0) {
                    if (pt == i) continue;
                    const double dx = sx - p.x[pt], dy = sy - p.y[pt], dz = sz - p.z[pt];
                    const double r2 = dx * dx + dy * dy + dz * dz;
                    const double dvx = svx - p.vx[pt], dvy = svy - p.vy[pt], dvz = svz - p.vz[pt];
                    if (LINE) {
                        const double dx2 = dx - dtl * dvx, dy2 = dy - dtl * dvy, dz2 = dz - dtl * dvz;
                        const double r2b = dx2 * dx2 + dy2 * dy2 + dz2 * dz2;
                        const double tc = (dx * dvx + dy * dvy + dz * dvz) / (dvx * dvx + dvy * dvy + dvz * dvz);
                        double rmin2 = r2 < r2b ? r2 : r2b;
                        if (tc / dtl >= 0. && tc / dtl <= 1.) {
                            const double dx3 = dx - tc * dvx, dy3 = dy - tc * dvy, dz3 = dz - tc * dvz;
                            const double r3 = dx3 * dx3 + dy3 * dy3 + dz3 * dz3;
                            rmin2 = rmin2 < r3 ? rmin2 : r3;
                        }
                        const double rsum = p1r + p.r[pt];
                        if (rmin2 > rsum * rsum) continue;
                    } else {
                        const double rp = p1r + p.r[pt];
                        if (r2 > rp * rp) continue;
                        if (dvx * dx + dvy * dy + dvz * dz > 0) continue;
                    }
                    if (out) {
                        rgpu_collision& o = out[base + found];
                        o.p1 = (size_t)i; o.p2 = (size_t)pt; o.ri = (size_t)r;
                        for (int k = 0; k < 6; k++) o.gb[k] = gb[k];
                    }
                    found++;
                } else {
                    const double dx = sx - c.x[q], dy = sy - c.y[q], dz = sz - c.z[q];
                    const double r2 = dx * dx + dy * dy + dz * dz;
                    const double rp = LINE ? p1r_dtv + maxdrift + 0.86602540378443 * c.w[q]
                                           : p1r + r2nd + 0.86602540378443 * c.w[q];
                    if (r2 < rp * rp) {
                        const int f = c.first[q], n = c.nchild[q];
                        if (sp + n > kStack) { atomicOr(status, DEV_ERR_STACK); return found; }
                        for (int k = n - 1; k >= 0; k--) stack[sp++] = f + k;
                    }
                }
            }
        }
    }
    return found;
}

// Largest squared speed of the particles (src/collision.c:273-277), as the bits of
// a non-negative double so that an integer atomicMax orders them.
__global__ void max_speed2(ParticlesSoA p, int N, unsigned long long* out) {
    __shared__ double part[kB];
    double l = 0.;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const double v2 = p.vx[i] * p.vx[i] + p.vy[i] * p.vy[i] + p.vz[i] * p.vz[i];
        l = l > v2 ? l : v2;
    }
    part[threadIdx.x] = l;
    __syncthreads();
    for (int w = kB / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) part[threadIdx.x] = fmax(part[threadIdx.x], part[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicMax(out, (unsigned long long)__double_as_longlong(part[0]));
}

template <bool LINE>
// Both pair kernels take particles in key order (`order`), like the walks; counts
// and output offsets stay indexed by particle, so the list keeps the reference's
// particle-major discovery order.
__global__ void __launch_bounds__(128) tree_pairs_count(ParticlesSoA p, int N, const int* __restrict__ order,
                                                        CellArrays c, BoxGeom g,
                                                        const GhostArr* __restrict__ gh, int nring, const double* r2nd,
                                                        double dtl, const unsigned long long* vmax2, int* count,
                                                        uint32_t* status) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    const int i = order[k];
    int stack[kStack];
    count[i] = tree_pairs_one<LINE>(i, p, c, g, gh, nring, r2nd[0], r2nd[1], dtl,
                                    LINE ? __longlong_as_double((long long)*vmax2) : 0., nullptr, 0, stack, status);
}

template <bool LINE>
__global__ void __launch_bounds__(128) tree_pairs_write(ParticlesSoA p, int N, const int* __restrict__ order,
                                                        CellArrays c, BoxGeom g,
                                                        const GhostArr* __restrict__ gh, int nring, const double* r2nd,
                                                        double dtl, const unsigned long long* vmax2,
                                                        const long long* off, rgpu_collision* out, uint32_t* status) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    const int i = order[k];
    int stack[kStack];
    tree_pairs_one<LINE>(i, p, c, g, gh, nring, r2nd[0], r2nd[1], dtl,
                         LINE ? __longlong_as_double((long long)*vmax2) : 0., out, off[i], stack, status);
}

// Second-largest radius (src/simulation.c:718-800): the second element of the
// radii sorted in descending order, which does not depend on traversal order.
__global__ void top2_radii(const double* __restrict__ r, int N, double* out) {
    __shared__ double a1[kB], a2[kB];
    double l1 = -1.0, l2 = -1.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const double v = r[i];
        if (v > l1) { l2 = l1; l1 = v; } else if (v > l2) { l2 = v; }
    }
    a1[threadIdx.x] = l1; a2[threadIdx.x] = l2;
    __syncthreads();
    for (int w = kB / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            const double b1 = a1[threadIdx.x + w], b2 = a2[threadIdx.x + w];
            double x1 = a1[threadIdx.x], x2 = a2[threadIdx.x];
            // merge two top-2 lists
            if (b1 > x1) { x2 = fmax(x1, b2); x1 = b1; } else { x2 = fmax(x2, b1); }
            a1[threadIdx.x] = x1; a2[threadIdx.x] = x2;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) { out[2 * blockIdx.x] = a1[0]; out[2 * blockIdx.x + 1] = a2[0]; }
}

__global__ void top2_final(double* v, int nb, int N) {
    double x1 = -1.0, x2 = -1.0;
    for (int b = 0; b < nb; b++) {
        const double b1 = v[2 * b], b2 = v[2 * b + 1];
        if (b1 > x1) { x2 = fmax(x1, b2); x1 = b1; } else { x2 = fmax(x2, b1); }
    }
    v[0] = N >= 2 ? x2 : 0.0;   // reference: 0 when there is no second particle
    v[1] = x1;                  // largest radius (bounds the leaf-root reach)
}

__global__ void exclusive_scan_counts(const int* __restrict__ cnt, int N, long long* __restrict__ off) {
    // one CTA, sequential per thread chunk + block scan
    __shared__ long long part[kB];
    const int per = (N + kB - 1) / kB;
    const int b0 = threadIdx.x * per;
    long long s = 0;
    for (int k = 0; k < per; k++) if (b0 + k < N) s += cnt[b0 + k];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < kB; o <<= 1) {
        const long long v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    long long run = threadIdx.x ? part[threadIdx.x - 1] : 0;
    for (int k = 0; k < per; k++) {
        if (b0 + k < N) { off[b0 + k] = run; run += cnt[b0 + k]; }
    }
    if (threadIdx.x == kB - 1) off[N] = run;
}

// --- host side -------------------------------------------------------------------------
CellArrays arrays(TreeBuffers* t) {
    return CellArrays{t->cx, t->cy, t->cz, t->cw, t->cm, t->cmx, t->cmy, t->cmz, t->cw2,
                      t->cqxx, t->cqxy, t->cqxz, t->cqyy, t->cqyz, t->cstart, t->cend, t->cfirst, t->cnchild, t->cpt, t->cdepth, t->cpath};
}

void free_cells(TreeBuffers* t) {
    double* d[] = {t->cx, t->cy, t->cz, t->cw, t->cm, t->cmx, t->cmy, t->cmz, t->cw2,
                   t->cqxx, t->cqxy, t->cqxz, t->cqyy, t->cqyz};
    for (double* q : d) cudaFree(q);
    t->cqxx = t->cqxy = t->cqxz = t->cqyy = t->cqyz = nullptr;
    int* n[] = {t->cstart, t->cend, t->cfirst, t->cnchild, t->cpt, t->cdepth};
    for (int* q : n) cudaFree(q);
    cudaFree(t->cpath);
    t->cx = t->cy = t->cz = t->cw = t->cm = t->cmx = t->cmy = t->cmz = t->cw2 = nullptr;
    t->cstart = t->cend = t->cfirst = t->cnchild = t->cpt = t->cdepth = nullptr;
    t->cpath = nullptr;
    t->ccap = 0;
}

int alloc_cells(rgpu_sim* s, TreeBuffers* t, size_t ccap) {
    free_cells(t);
    double** d[] = {&t->cx, &t->cy, &t->cz, &t->cw, &t->cm, &t->cmx, &t->cmy, &t->cmz, &t->cw2,
                    &t->cqxx, &t->cqxy, &t->cqxz, &t->cqyy, &t->cqyz};
    for (double** q : d) RGPU_CUDA(s, cudaMalloc(q, sizeof(double) * ccap));
    int** n[] = {&t->cstart, &t->cend, &t->cfirst, &t->cnchild, &t->cpt, &t->cdepth};
    for (int** q : n) RGPU_CUDA(s, cudaMalloc(q, sizeof(int) * ccap));
    RGPU_CUDA(s, cudaMalloc(&t->cpath, sizeof(unsigned long long) * ccap));
    t->ccap = ccap;
    return RGPU_OK;
}

int ensure_tree(rgpu_sim* s) {
    if (!s->tree) s->tree = new TreeBuffers();
    TreeBuffers* t = s->tree;
    if (t->cap < s->cap) {
        cudaFree(t->keys); cudaFree(t->keys_alt); cudaFree(t->idx); cudaFree(t->idx_alt);
        cudaFree(t->pair_count); cudaFree(t->pair_off);
        t->keys = t->keys_alt = nullptr; t->idx = t->idx_alt = nullptr; t->pair_count = nullptr; t->pair_off = nullptr;
        RGPU_CUDA(s, cudaMalloc(&t->keys, sizeof(unsigned long long) * s->cap));
        RGPU_CUDA(s, cudaMalloc(&t->keys_alt, sizeof(unsigned long long) * s->cap));
        RGPU_CUDA(s, cudaMalloc(&t->idx, sizeof(int) * s->cap));
        RGPU_CUDA(s, cudaMalloc(&t->idx_alt, sizeof(int) * s->cap));
        RGPU_CUDA(s, cudaMalloc(&t->pair_count, sizeof(int) * s->cap));
        RGPU_CUDA(s, cudaMalloc(&t->pair_off, sizeof(long long) * (s->cap + 1)));
        t->cap = s->cap;
    }
    if (!t->counter) RGPU_CUDA(s, cudaMalloc(&t->counter, sizeof(int)));
    if (!t->r_top) RGPU_CUDA(s, cudaMalloc(&t->r_top, sizeof(double) * (2 * 1024 + 1)));   // + max speed^2
    return RGPU_OK;
}

BoxGeom geometry(const rgpu_config& c, int* n_root) {
    BoxGeom g;
    g.root_size = c.root_size;
    g.nx = c.N_root_x; g.ny = c.N_root_y; g.nz = c.N_root_z;
    g.bx = c.root_size * (double)c.N_root_x;
    g.by = c.root_size * (double)c.N_root_y;
    g.bz = c.root_size * (double)c.N_root_z;
    *n_root = g.nx * g.ny * g.nz;
    int bits = 1;
    while ((1ll << bits) < (long long)*n_root) bits++;
    g.D = std::min(21, (64 - bits) / 3);
    g.shift = 3 * g.D;
    return g;
}

GhostArr* g_ghosts = nullptr;

int upload_ghosts(rgpu_sim* s, int nx, int ny, int nz) {
    GhostArr h;
    h.n = 0;
    for (int gx = -nx; gx <= nx; gx++)
        for (int gy = -ny; gy <= ny; gy++)
            for (int gz = -nz; gz <= nz; gz++) {
                if (h.n >= 125) return set_error(s, RGPU_ERR_UNSUPPORTED, "more than 125 ghost boxes");
                ghostbox(s->cfg, gx, gy, gz, h.off[h.n]);
                h.n++;
            }
    if (!g_ghosts) RGPU_CUDA(s, cudaMalloc(&g_ghosts, sizeof(GhostArr)));
    RGPU_CUDA(s, cudaMemcpyAsync(g_ghosts, &h, sizeof(GhostArr), cudaMemcpyHostToDevice, s->stream));
    return RGPU_OK;
}

// Build the tree for the current particle positions.
int build_tree_once(rgpu_sim* s, bool* overflow) {
    *overflow = false;
    RGPU_TRY(ensure_tree(s));
    TreeBuffers* t = s->tree;
    const int N = (int)s->N;
    int n_root = 0;
    const BoxGeom g = geometry(s->cfg, &n_root);
    t->D = g.D;
    t->n_root = n_root;
    const size_t want = (size_t)n_root + 4 * (size_t)N + 64;
    if (t->ccap < want) RGPU_TRY(alloc_cells(s, t, want));
    cudaStream_t st = s->stream;
    make_keys<<<grid_for(N, kB), kB, 0, st>>>(s->p, N, g, t->keys, t->idx, s->d_status);
    g_launches++;
    // radix sort over the used key bits
    const int used_bits = g.shift + 1 + (int)std::log2((double)std::max(1, n_root));
    const int nblk = (N + kSortTile - 1) / kSortTile;
    if ((size_t)256 * nblk > t->hist_cap) {
        cudaFree(t->hist);
        t->hist = nullptr;
        RGPU_CUDA(s, cudaMalloc(&t->hist, sizeof(unsigned int) * 256 * nblk));
        t->hist_cap = (size_t)256 * nblk;
    }
    for (int shift = 0; shift < std::min(64, used_bits + 1); shift += 8) {
        radix_hist<<<nblk, kB, 0, st>>>(t->keys, N, shift, t->hist, nblk);
        radix_scan<<<1, kB, 0, st>>>(t->hist, 256 * nblk);
        radix_scatter<<<nblk, kB, 0, st>>>(t->keys, t->idx, N, shift, t->hist, nblk, t->keys_alt, t->idx_alt);
        g_launches += 3;
        std::swap(t->keys, t->keys_alt);
        std::swap(t->idx, t->idx_alt);
    }
    CellArrays c = arrays(t);
    init_roots<<<grid_for(n_root, kB), kB, 0, st>>>(c, n_root, g);
    root_ranges<<<grid_for(N, kB), kB, 0, st>>>(t->keys, t->idx, N, g.shift, c, n_root);
    root_finish<<<grid_for(n_root, kB), kB, 0, st>>>(t->idx, c, n_root);
    g_launches += 3;
    // levels, top-down
    t->level_begin.assign(1, 0);
    t->level_begin.push_back(n_root);
    int next = n_root;
    RGPU_CUDA(s, cudaMemcpyAsync(t->counter, &next, sizeof(int), cudaMemcpyHostToDevice, st));
    for (int d = 0; d <= g.D; d++) {
        const int b = t->level_begin[d], e = t->level_begin[d + 1];
        if (e <= b) break;
        split_level<<<grid_for(e - b, kB), kB, 0, st>>>(t->keys, t->idx, s->p, c, b, e, g.D, t->counter,
                                                        (int)t->ccap, s->d_status);
        g_launches++;
        RGPU_CUDA(s, cudaMemcpyAsync(&next, t->counter, sizeof(int), cudaMemcpyDeviceToHost, st));
        RGPU_CUDA(s, cudaStreamSynchronize(st));
        if (next > (int)t->ccap) {
            *overflow = true;
            uint32_t zero = 0;   // clear the overflow bit; the caller rebuilds with more cells
            cudaMemcpyAsync(s->d_status, &zero, sizeof(zero), cudaMemcpyHostToDevice, st);
            return RGPU_OK;
        }
        t->level_begin.push_back(next);
    }
    t->n_cells = next;
    // bottom-up reduction
    const int nl = (int)t->level_begin.size() - 1;
    for (int d = nl - 1; d >= 0; d--) {
        const int b = t->level_begin[d], e = t->level_begin[d + 1];
        if (e > b) {
            reduce_level<<<grid_for(e - b, kB), kB, 0, st>>>(s->p, c, b, e, s->cfg.tree_quadrupole != 0);
            g_launches++;
        }
    }
    RGPU_CUDA(s, cudaGetLastError());
    return RGPU_OK;
}

int build_tree(rgpu_sim* s) {
    for (int attempt = 0; attempt < 6; attempt++) {
        bool overflow = false;
        RGPU_TRY(build_tree_once(s, &overflow));
        if (!overflow) return RGPU_OK;
        RGPU_TRY(alloc_cells(s, s->tree, 2 * s->tree->ccap));
    }
    return set_error(s, RGPU_ERR_OVERFLOW, "tree cell capacity exceeded");
}

}  // namespace

int tree_accel(rgpu_sim* s) {
    const int N = (int)s->N;
    if (!N) return RGPU_OK;
    RGPU_TRY(boundary_check(s));                       // src/gravity.c:62-64
    RGPU_TRY(build_tree(s));
    RGPU_TRY(read_status(s));
    const rgpu_config& cf = s->cfg;
    RGPU_TRY(upload_ghosts(s, cf.N_ghost_x, cf.N_ghost_y, cf.N_ghost_z));
    TreeBuffers* t = s->tree;
    const double eps2 = cf.softening * cf.softening;
    if (cf.gravity != RGPU_GRAVITY_TREE_SPLIT) {
        ktimer_begin(s);
        if (cf.tree_quadrupole)
            walk_exact<true><<<grid_for(N, 128), 128, 0, s->stream>>>(s->p, N, t->idx, arrays(t), t->n_root, g_ghosts,
                                                                      walk_const(cf, eps2), s->d_status);
        else
            walk_exact<false><<<grid_for(N, 128), 128, 0, s->stream>>>(s->p, N, t->idx, arrays(t), t->n_root, g_ghosts,
                                                                       walk_const(cf, eps2), s->d_status);
        ktimer_end(s);
        g_launches++;
        RGPU_CUDA(s, cudaGetLastError());
        return RGPU_OK;
    }
    // Split mode: near-window walk (reference semantics) + far-root monopole sweep.
    if (cf.tree_quadrupole)
        return set_error(s, RGPU_ERR_UNSUPPORTED, "the split tree mode sums far roots as monopoles (no quadrupole)");
    if (!(cf.opening_angle2 > 0.))
        return set_error(s, RGPU_ERR_ARG, "split tree mode needs opening_angle2 > 0");
    const int K = (int)ceil(1.0 / sqrt(cf.opening_angle2)) + 1;
    int n_root = 0;
    const BoxGeom geo = geometry(cf, &n_root);
    const int n_pair = (n_root + 1) / 2;
    if ((size_t)n_pair > t->sweep_cap) {
        cudaFree(t->sweep);
        t->sweep = nullptr;
        t->sweep_cap = 0;
        RGPU_CUDA(s, cudaMalloc(&t->sweep, sizeof(RootPair) * n_pair));
        t->sweep_cap = (size_t)n_pair;
    }
    RootPair* sw = (RootPair*)t->sweep;
    build_root_pairs<<<grid_for(n_pair, kB), kB, 0, s->stream>>>(arrays(t), n_root, geo, cf.G, sw);
    walk_near<<<grid_for(N, 128), 128, 0, s->stream>>>(s->p, N, t->idx, arrays(t), geo, g_ghosts,
                                                        walk_const(cf, eps2), K, s->d_status);
    ktimer_begin(s);
    sweep_far<<<grid_for(N, kSweepTile), kSweepTile, 0, s->stream>>>(s->p, N, sw, n_pair, geo, g_ghosts, eps2, K);
    ktimer_end(s);
    g_launches += 3;
    RGPU_CUDA(s, cudaGetLastError());
    return RGPU_OK;
}

int tree_collisions(rgpu_sim* s, rgpu_collision* out, size_t cap, size_t* n_found, bool device_only, bool line) {
    const int N = (int)s->N;
    *n_found = 0;
    if (!N) return RGPU_OK;
    RGPU_TRY(build_tree(s));
    RGPU_TRY(read_status(s));
    TreeBuffers* t = s->tree;
    const rgpu_config& cf = s->cfg;
    // inner ring of ghost boxes only (src/collision.c:207-210)
    const int nx = cf.N_ghost_x > 1 ? 1 : cf.N_ghost_x, ny = cf.N_ghost_y > 1 ? 1 : cf.N_ghost_y,
              nz = cf.N_ghost_z > 1 ? 1 : cf.N_ghost_z;
    RGPU_TRY(upload_ghosts(s, nx, ny, nz));
    const int nring = (2 * nx + 1) * (2 * ny + 1) * (2 * nz + 1);
    int n_root = 0;
    const BoxGeom g = geometry(cf, &n_root);
    const int nb = std::min(1024, (int)grid_for(N, kB));
    top2_radii<<<nb, kB, 0, s->stream>>>(s->p.r, N, t->r_top);
    top2_final<<<1, 1, 0, s->stream>>>(t->r_top, nb, N);
    CellArrays c = arrays(t);
    unsigned long long* vmax2 = reinterpret_cast<unsigned long long*>(t->r_top + 2 * 1024);
    if (line) {
        RGPU_CUDA(s, cudaMemsetAsync(vmax2, 0, sizeof(double), s->stream));
        max_speed2<<<nb, kB, 0, s->stream>>>(s->p, N, vmax2);
        g_launches++;
    }
    const double dtl = s->dt_last_done;
    if (line)
        tree_pairs_count<true><<<grid_for(N, 128), 128, 0, s->stream>>>(s->p, N, t->idx, c, g, g_ghosts, nring, t->r_top,
                                                                        dtl, vmax2, t->pair_count, s->d_status);
    else
        tree_pairs_count<false><<<grid_for(N, 128), 128, 0, s->stream>>>(s->p, N, t->idx, c, g, g_ghosts, nring, t->r_top,
                                                                         dtl, vmax2, t->pair_count, s->d_status);
    exclusive_scan_counts<<<1, kB, 0, s->stream>>>(t->pair_count, N, t->pair_off);
    g_launches += 4;
    long long total = 0;
    RGPU_CUDA(s, cudaMemcpyAsync(&total, t->pair_off + N, sizeof(long long), cudaMemcpyDeviceToHost, s->stream));
    RGPU_CUDA(s, cudaStreamSynchronize(s->stream));
    RGPU_TRY(read_status(s));
    if ((size_t)total > t->pairs_cap) {
        cudaFree(t->pairs);
        t->pairs = nullptr;
        t->pairs_cap = 0;
        const size_t want = std::max<size_t>(1024, (size_t)total * 2);
        RGPU_CUDA(s, cudaMalloc(&t->pairs, sizeof(rgpu_collision) * want));
        t->pairs_cap = want;
    }
    if (total) {
        if (line)
            tree_pairs_write<true><<<grid_for(N, 128), 128, 0, s->stream>>>(s->p, N, t->idx, c, g, g_ghosts, nring, t->r_top,
                                                                            dtl, vmax2, t->pair_off, t->pairs,
                                                                            s->d_status);
        else
            tree_pairs_write<false><<<grid_for(N, 128), 128, 0, s->stream>>>(s->p, N, t->idx, c, g, g_ghosts, nring,
                                                                             t->r_top, dtl, vmax2, t->pair_off,
                                                                             t->pairs, s->d_status);
        g_launches++;
    }
    *n_found = (size_t)total;
    s->n_pairs = (size_t)total;
    s->dev_pairs = t->pairs;
    if (device_only) return RGPU_OK;
    if ((size_t)total > cap) return set_error(s, RGPU_ERR_OVERFLOW, "collision buffer too small");
    if (total) RGPU_CUDA(s, cudaMemcpyAsync(out, t->pairs, sizeof(rgpu_collision) * total, cudaMemcpyDeviceToHost, s->stream));
    RGPU_CUDA(s, cudaStreamSynchronize(s->stream));
    return read_status(s);
}

void tree_free(rgpu_sim* s) {
    if (!s->tree) return;
    TreeBuffers* t = s->tree;
    free_cells(t);
    cudaFree(t->keys); cudaFree(t->keys_alt); cudaFree(t->idx); cudaFree(t->idx_alt);
    cudaFree(t->hist); cudaFree(t->counter); cudaFree(t->pair_count); cudaFree(t->pair_off);
    cudaFree(t->pairs); cudaFree(t->r_top); cudaFree(t->sweep);
    delete t;
    s->tree = nullptr;
}

// Export cells in depth-first order (root index, then octants) for membership parity.
extern "C" int rgpu_tree_export(rgpu_sim* s, void* out_cells, size_t cap, size_t* n_out) {
    if (!s || !n_out) return RGPU_ERR_ARG;
    *n_out = 0;
    if (!s->N) return RGPU_OK;
    if (s->cfg.root_size <= 0) return set_error(s, RGPU_ERR_ARG, "root_size must be set");
    RGPU_TRY(build_tree(s));
    RGPU_TRY(read_status(s));
    TreeBuffers* t = s->tree;
    const int nc = t->n_cells;
    std::vector<double> x(nc), y(nc), z(nc), w(nc), m(nc), mx(nc), my(nc), mz(nc);
    std::vector<int> first(nc), nch(nc), pt(nc), depth(nc);
    std::vector<unsigned long long> path(nc);
    cudaStreamSynchronize(s->stream);
    cudaMemcpy(x.data(), t->cx, 8 * nc, cudaMemcpyDeviceToHost);
    cudaMemcpy(y.data(), t->cy, 8 * nc, cudaMemcpyDeviceToHost);
    cudaMemcpy(z.data(), t->cz, 8 * nc, cudaMemcpyDeviceToHost);
    cudaMemcpy(w.data(), t->cw, 8 * nc, cudaMemcpyDeviceToHost);
    cudaMemcpy(m.data(), t->cm, 8 * nc, cudaMemcpyDeviceToHost);
    cudaMemcpy(mx.data(), t->cmx, 8 * nc, cudaMemcpyDeviceToHost);
    cudaMemcpy(my.data(), t->cmy, 8 * nc, cudaMemcpyDeviceToHost);
    cudaMemcpy(mz.data(), t->cmz, 8 * nc, cudaMemcpyDeviceToHost);
    cudaMemcpy(first.data(), t->cfirst, 4 * nc, cudaMemcpyDeviceToHost);
    cudaMemcpy(nch.data(), t->cnchild, 4 * nc, cudaMemcpyDeviceToHost);
    cudaMemcpy(pt.data(), t->cpt, 4 * nc, cudaMemcpyDeviceToHost);
    cudaMemcpy(depth.data(), t->cdepth, 4 * nc, cudaMemcpyDeviceToHost);
    RGPU_CUDA(s, cudaMemcpy(path.data(), t->cpath, 8 * (size_t)nc, cudaMemcpyDeviceToHost));
    // record layout: int32 root, int32 depth, uint64 path, 8 doubles, int64 pt (88 bytes)
    struct Rec { int32_t root, depth; uint64_t path; double x, y, z, w, m, mx, my, mz; int64_t pt; };
    Rec* o = (Rec*)out_cells;
    size_t n = 0;
    std::vector<int> stack;
    for (int r = 0; r < t->n_root; r++) {
        if (pt[r] == INT_MIN) continue;
        stack.assign(1, r);
        while (!stack.empty()) {
            const int q = stack.back();
            stack.pop_back();
            if (o && n < cap) o[n] = Rec{r, depth[q], path[q], x[q], y[q], z[q], w[q], m[q], mx[q], my[q], mz[q], (int64_t)pt[q]};
            n++;
            for (int k = nch[q] - 1; k >= 0; k--) stack.push_back(first[q] + k);
        }
    }
    *n_out = n;
    return n > cap ? RGPU_ERR_OVERFLOW : RGPU_OK;
}
