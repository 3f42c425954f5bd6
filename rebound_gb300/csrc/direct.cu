// Direct-summation gravity on sm_103a: REB_GRAVITY_BASIC and COMPENSATED
// (src/gravity.c:167-531 of REBOUND 5.0.0) plus the GB300 mixed-precision forms.
//
// Layout: one thread per i-particle, CTAs of 256 threads; the j-range is cut
// into `splits` chunks (grid.y) so that small N still fills 152 SMs, and the
// CTA count is chosen close to a multiple of the SM count.  j-data is staged
// through shared memory in tiles of 256 bodies as packed (x, y, z, G*m)
// doubles (MIXED_SPLIT: two float4 per body, the (hi, lo) single-precision
// split of each coordinate).  All threads of a warp read the same j-body, so
// the shared loads are broadcasts.
//
// GB300 executes FP64 arithmetic on a narrow pipe (about 1/64 of the FP32
// rate), so the FP64 kernel minimises FP64 instructions:
//   displacement 3 DADD, r^2 3 DFMA, G m / r^3 6, accumulate 3 DFMA = 15
// per pair (all format conversions run on the integer pipe).  BASIC sums each
// 256-body tile with FMAs and folds the tile sums in with Kahan compensation,
// so its error does not grow with N (the plain sequential sum of 262,144 terms
// is off by up to ~3e-14 relative).
// 1/r^3 is seeded in FP32 (MUFU rsqrt) from an integer truncation of r^2 and
// corrected in FP64 with the binomial series
//   (1-h)^(-3/2) = 1 + 3/2 h + 15/8 h^2 + O(h^3),   h = 1 - r^2 y0^2,
// |h| < 2^-21, so the dropped 35/16 h^3 term is below 2^-62.
#include "rgpu_internal.cuh"
#include "fixpair.cuh"
#include <algorithm>
#include <cmath>
#include <vector>

namespace {

constexpr int kBlock = 256;   // threads per CTA = i-particles per CTA = j-tile size

enum Mode { kBasic = 0, kComp = 1, kMixed = 2, kMixedSplit = 3 };
// How m/r^3 is evaluated in the FP64 modes.
enum RinvVariant { kRinvLib = 0, kRinvSeries = 1, kRinvSeriesF32 = 2, kRinvSeriesInt = 3 };

// --- exact bit-level conversions on the integer pipe --------------------------
// Positive double -> float by truncating the mantissa; valid for v in [2^-126, 2^128).
__device__ __forceinline__ float trunc_pos_to_float(double v) {
    const unsigned lo = (unsigned)__double2loint(v);
    const unsigned hi = (unsigned)__double2hiint(v);
    // (sign|exp11|mant20 : mant32) << 3 keeps the low 9 exponent bits and the
    // top 23 mantissa bits; subtracting (1023-127) << 23 rebiases the exponent.
    return __uint_as_float(__funnelshift_l(lo, hi, 3) - 0xC0000000u);
}
// Signed double -> float by truncation; |v| < 2^-126 gives 0.  Valid for |v| < 2^128.
__device__ __forceinline__ float trunc_to_float(double v) {
    const unsigned lo = (unsigned)__double2loint(v);
    const unsigned hi = (unsigned)__double2hiint(v);
    const unsigned mag = (__funnelshift_l(lo, hi, 3) - 0xC0000000u) & 0x7FFFFFFFu;
    const unsigned f = ((hi & 0x7FFFFFFFu) < 0x38100000u) ? 0u : (mag | (hi & 0x80000000u));
    return __uint_as_float(f);
}
// Signed double -> float rounded to nearest (ties away from zero); |v| < 2^-126 gives 0.
__device__ __forceinline__ float round_to_float(double v) {
    const unsigned lo = (unsigned)__double2loint(v);
    const unsigned hi = (unsigned)__double2hiint(v);
    const unsigned mag = ((__funnelshift_l(lo, hi, 3) - 0xC0000000u) + ((lo >> 28) & 1u)) & 0x7FFFFFFFu;
    const unsigned f = ((hi & 0x7FFFFFFFu) < 0x38100000u) ? 0u : (mag | (hi & 0x80000000u));
    return __uint_as_float(f);
}
// Positive normal float -> double, exactly (0 maps to 2^-127, harmless where used).
__device__ __forceinline__ double exact_to_double(float f) {
    const unsigned b = __float_as_uint(f);
    return __hiloint2double((int)((b >> 3) + 0x38000000u), (int)(b << 29));
}
constexpr unsigned kHiMin = 0x38100000u;   // high word of 2^-126
constexpr unsigned kHiMax = 0x47E00000u;   // high word of 2^127

// m * r2^(-3/2) in FP64.
template <int RV>
__device__ __forceinline__ double m_rinv3(double r2, double m) {
    if (RV == kRinvLib) {
        const double ri = rsqrt(r2);
        return m * ri * ri * ri;
    }
    const unsigned hi = (unsigned)__double2hiint(r2);
    if (hi - kHiMin <= kHiMax - kHiMin) {
        const float y0f = rsqrtf(trunc_pos_to_float(r2));
        const double y0 = exact_to_double(y0f);
        const double y2 = y0 * y0;                        // exact (48-bit product)
        const double h = fma(-r2, y2, 1.0);               // |h| < 2^-21
        const double my3 = (m * y2) * y0;
        double c;
        if (RV == kRinvSeriesF32) {
            const float hf = (float)h;
            c = fma(h, 1.5, (double)(1.875f * hf * hf));   // 15/8 h^2 needs ~11 bits
        } else if (RV == kRinvSeriesInt) {
            // The same with both conversions on the integer pipe (GB300 runs cvt
            // on the FP64 pipe): 15/8 h^2 < 2^-40 needs only ~11 correct bits.
            const float hf = trunc_to_float(h);
            c = fma(h, 1.5, exact_to_double(1.875f * hf * hf));
        } else {
            c = h * fma(h, 1.875, 1.5);
        }
        return fma(my3, c, my3);
    }
    const double ri = rsqrt(r2);                          // outside the FP32 exponent range
    return m * ri * ri * ri;
}

struct GhostList {
    int n;
    double off[125][3];
};

// --- Fixed-point positions for the integer-pipe pair forms ---------------------
// Positions are held as 64-bit fixed point with scale 2^s, s chosen per force
// evaluation so the largest |coordinate| is below 2^61 (differences then fit in
// int64) and eps^2 2^2s below 2^124.  Every coordinate with |x| >= 2^-8 max|x|
// is representable exactly, so the integer difference rounded once to double
// equals the FP64 subtraction bit for bit; smaller coordinates are rounded to
// the 2^-s grid (an absolute error below 2^-61 max|x|).
struct __align__(32) FixBody {
    long long x, y, z;
    double gm;
};

// Per-evaluation scale words, written by pack_fix and read by every pair thread.
struct __align__(16) FixScale {
    unsigned long long dmax;               // max |coordinate| as double bits (atomicMax target)
    int shift;                             // s
    int two_s;                             // 2 s
    unsigned long long e0, e1, e2;         // eps^2 2^2s = e0 + e1 2^32 + e2 2^62 (e0 < 2^32, e1 < 2^30)
};
static_assert(sizeof(FixScale) <= 256 * 2 * sizeof(float4), "FixScale lives in the jsplit buffer (>= 256 bodies)");

__global__ void max_abs_coord(ParticlesSoA p, int N, unsigned long long* __restrict__ out) {
    __shared__ double red[256];
    double m = 0.;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
        m = fmax(m, fmax(fabs(p.x[i]), fmax(fabs(p.y[i]), fabs(p.z[i]))));
    red[threadIdx.x] = m;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicMax(out, (unsigned long long)__double_as_longlong(red[0]));  // positive doubles order as integers
}

__global__ void pack_fix(ParticlesSoA p, int N, double G, double eps2, FixScale* __restrict__ sc,
                         FixBody* __restrict__ out) {
    const double mx = __longlong_as_double((long long)sc->dmax);
    int s = (mx > 0. && isfinite(mx)) ? 60 - ilogb(mx) : 60;
    if (eps2 > 0. && isfinite(eps2)) s = min(s, (123 - ilogb(eps2)) >> 1);
    s = min(s, 1022);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        unsigned long long hi = 0, lo = 0;
        if (eps2 > 0. && isfinite(eps2)) {
            int ee;
            const double fr = frexp(eps2, &ee);                        // eps2 = fr 2^ee, fr in [0.5, 1)
            const unsigned long long m53 = (unsigned long long)scalbn(fr, 53);
            const int sh = ee - 53 + 2 * s;                             // eps2 2^2s = m53 2^sh < 2^124
            if (sh >= 64) { hi = m53 << (sh - 64); }
            else if (sh > 0) { hi = m53 >> (64 - sh); lo = m53 << sh; }
            else if (sh > -64) { lo = m53 >> (-sh); }
        }
        sc->shift = s;
        sc->two_s = 2 * s;
        sc->e0 = lo & 0xFFFFFFFFull;
        sc->e1 = (lo >> 32) & 0x3FFFFFFFull;
        sc->e2 = (lo >> 62) | (hi << 2);
    }
    if (i >= N) return;
    FixBody b;
    b.x = __double2ll_rn(scalbn(p.x[i], s));
    b.y = __double2ll_rn(scalbn(p.y[i], s));
    b.z = __double2ll_rn(scalbn(p.z[i], s));
    b.gm = G * p.m[i];
    out[i] = b;
}

struct DirectArgs {
    const double4_32a* __restrict__ jpos;      // (x, y, z, G*m)
    const float4* __restrict__ jsplit;     // 2 per body: (xh, yh, zh, Gm_f), (xl, yl, zl, 0)
    int N;                                 // i-range [0, N)
    int Na;                                // active particles
    int tp;                                // testparticle_type
    int ign;                               // gravity_ignore_terms
    double eps2;
    int splits;
    double* __restrict__ ax;               // direct output (splits == 1)
    double* __restrict__ ay;
    double* __restrict__ az;
    double* __restrict__ partial;          // [split][3][cap] (splits > 1)
    size_t cap;
    const FixScale* __restrict__ fix;      // non-null: jpos holds FixBody records (FIX kernels)
};

// j-range of particle i (src/gravity.c:215-233 and :258-277): active
// particles also feel test particles when testparticle_type == 1.
__device__ __forceinline__ int j_end_of(const DirectArgs& a, int i) {
    return (a.tp && i < a.Na) ? a.N : a.Na;
}

__device__ __forceinline__ bool pair_skipped(const DirectArgs& a, int i, int j) {
    if (a.ign == 1) return (i == 0 && j == 1) || (i == 1 && j == 0);
    if (a.ign == 2) return i == 0 || j == 0;
    return false;
}

// FIX: 0 = FP64 positions; 1 = fixed-point positions, displacement converted on
// the integer pipe (exactly the FP64 subtraction), FP64 r^2 and m/r^3; 2 =
// fixed-point positions, displacement and (r^2+eps^2)^(-3/2) on the integer
// pipes (fixpair::limbs_to_double, fixpair::rinv3_limbs), FP64 only for
// G m f and the accumulation.
template <int MODE, bool GENERAL, int RV, bool CVT, int FIX = 0>
__global__ void __launch_bounds__(kBlock) direct_kernel(DirectArgs a, const GhostList* __restrict__ ghosts) {
    __shared__ double4_32a tile[(MODE == kMixedSplit) ? 1 : kBlock];
    __shared__ float4 tile_s[(MODE == kMixedSplit) ? 2 * kBlock : 1];
    const int i = blockIdx.x * kBlock + threadIdx.x;
    const bool live = i < a.N;
    const int jmax_cta = (a.tp && (int)(blockIdx.x * kBlock) < a.Na) ? a.N : a.Na;
    const int chunk = (((jmax_cta + a.splits - 1) / a.splits) + kBlock - 1) / kBlock * kBlock;
    const int j0 = blockIdx.y * chunk;
    const int j1 = min(jmax_cta, j0 + chunk);
    const int jend_i = live ? j_end_of(a, i) : 0;

    double xi = 0., yi = 0., zi = 0.;
    if (live) {
        const double4_32a p = a.jpos[i];
        xi = p.x; yi = p.y; zi = p.z;
    }
    // FIX: the records are FixBody bit patterns; the displacement is the int64
    // difference converted once (exactly the FP64 subtraction, see FixBody).
    const long long xfi = __double_as_longlong(xi), yfi = __double_as_longlong(yi), zfi = __double_as_longlong(zi);
    int ebias = 0, two_s = 0;
    float sc_hi = 0.f, sc_lo = 0.f;                 // 2^(32 - s), 2^-s (MIXED)
    unsigned long long e0 = 0, e1 = 0, e2 = 0;
    if (FIX) {
        ebias = 1086 - a.fix->shift;
        if (MODE == kMixed) {
            sc_hi = __uint_as_float((unsigned)max(1, min(254, 127 + 32 - a.fix->shift)) << 23);
            sc_lo = __uint_as_float((unsigned)max(1, min(254, 127 - a.fix->shift)) << 23);
        }
        two_s = a.fix->two_s;
        e0 = a.fix->e0;
        e1 = a.fix->e1;
        e2 = a.fix->e2;
    }
    double sx = 0., sy = 0., sz = 0., cx = 0., cy = 0., cz = 0.;
    float fsx = 0.f, fsy = 0.f, fsz = 0.f, fcx = 0.f, fcy = 0.f, fcz = 0.f;
    const float eps2f = (float)a.eps2;
    const int ng = GENERAL ? ghosts->n : 1;

    for (int jt = j0; jt < j1; jt += kBlock) {
        const int jl = jt + threadIdx.x;
        __syncthreads();
        if (MODE == kMixedSplit) {
            tile_s[2 * threadIdx.x] = jl < j1 ? a.jsplit[2 * jl] : make_float4(0.f, 0.f, 0.f, 0.f);
            tile_s[2 * threadIdx.x + 1] = jl < j1 ? a.jsplit[2 * jl + 1] : make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
            tile[threadIdx.x] = jl < j1 ? a.jpos[jl] : make_double4_32a(0., 0., 0., 0.);
        }
        __syncthreads();
        const int nt = min(kBlock, j1 - jt);
        for (int g = 0; g < ng; g++) {
            // BASIC: FMA-accumulate this tile, then fold the tile sum into the running
            // total with Kahan compensation (error O(tile) instead of O(N) terms).
            double tx = 0., ty = 0., tz = 0.;
            // The reference shifts particle i by the ghost offset: dx_ref = (gb + x_i) - x_j;
            // here d = x_j - (gb + x_i) and the force is +s*d.
            double gxi = xi, gyi = yi, gzi = zi;
            if (GENERAL) {
                gxi = ghosts->off[g][0] + xi; gyi = ghosts->off[g][1] + yi; gzi = ghosts->off[g][2] + zi;
            }
            float xih = 0.f, yih = 0.f, zih = 0.f, xil = 0.f, yil = 0.f, zil = 0.f;
            if (MODE == kMixedSplit) {
                xih = (float)gxi; yih = (float)gyi; zih = (float)gzi;
                xil = (float)(gxi - (double)xih); yil = (float)(gyi - (double)yih); zil = (float)(gzi - (double)zih);
            }
#pragma unroll 4
            for (int k = 0; k < nt; k++) {
                const int j = jt + k;
                bool skip = (j == i);
                if (GENERAL) skip = skip || j >= jend_i || pair_skipped(a, i, j);
                if (MODE == kBasic || MODE == kComp) {
                    const double4_32a q = tile[k];
                    double dx, dy, dz, s;
                    if (FIX == 2) {
                        unsigned xh, xl, yh, yl, zh, zl, sx_, sy_, sz_;
                        fixpair::sub_abs(__double_as_longlong(q.x), xfi, xh, xl, sx_);
                        fixpair::sub_abs(__double_as_longlong(q.y), yfi, yh, yl, sy_);
                        fixpair::sub_abs(__double_as_longlong(q.z), zfi, zh, zl, sz_);
                        dx = fixpair::limbs_to_double(xh, xl, sx_, ebias - 1);
                        dy = fixpair::limbs_to_double(yh, yl, sy_, ebias - 1);
                        dz = fixpair::limbs_to_double(zh, zl, sz_, ebias - 1);
                        // COMPENSATED is FP64-bound (Kahan terms): G m folded into the integer
                        // factor saves its DMUL; BASIC is integer-bound: the DMUL is cheaper there.
                        if (MODE == kComp)
                            s = fixpair::rinv3m_limbs<true>(xh, xl, yh, yl, zh, zl, e0, e1, e2, two_s,
                                                            (unsigned long long)__double_as_longlong(q.w));
                        else
                            s = q.w * fixpair::rinv3_limbs<true>(xh, xl, yh, yl, zh, zl, e0, e1, e2, two_s);
                    } else if (FIX) {
                        unsigned long long sgx, sgy, sgz;
                        const unsigned long long ux = fixpair::abs64(__double_as_longlong(q.x) - xfi, &sgx);
                        const unsigned long long uy = fixpair::abs64(__double_as_longlong(q.y) - yfi, &sgy);
                        const unsigned long long uz = fixpair::abs64(__double_as_longlong(q.z) - zfi, &sgz);
                        dx = fixpair::abs_to_double(ux, sgx, ebias);
                        dy = fixpair::abs_to_double(uy, sgy, ebias);
                        dz = fixpair::abs_to_double(uz, sgz, ebias);
                        const double r2 = fma(dx, dx, fma(dy, dy, fma(dz, dz, a.eps2)));
                        s = m_rinv3<RV>(r2, q.w);
                    } else {
                        dx = q.x - gxi; dy = q.y - gyi; dz = q.z - gzi;
                        const double r2 = fma(dx, dx, fma(dy, dy, fma(dz, dz, a.eps2)));
                        s = m_rinv3<RV>(r2, q.w);
                    }
                    s = skip ? 0.0 : s;
                    if (MODE == kBasic) {
                        tx = fma(s, dx, tx); ty = fma(s, dy, ty); tz = fma(s, dz, tz);
                    } else {
                        // Kahan per component (src/gravity.c:325-343).
                        double t, y;
                        y = s * dx - cx; t = sx + y; cx = (t - sx) - y; sx = t;
                        y = s * dy - cy; t = sy + y; cy = (t - sy) - y; sy = t;
                        y = s * dz - cz; t = sz + y; cz = (t - sz) - y; sz = t;
                    }
                } else {
                    float dxf, dyf, dzf, mf;
                    if (MODE == kMixed && FIX) {
                        // the exact displacement D (int64, from the fixed-point positions) to float
                        // as hi 2^32 + lo with two 32-bit conversions and one FFMA (<= 1.5 ulp)
                        const double4_32a q = tile[k];
                        const long long Dx = __double_as_longlong(q.x) - xfi;
                        const long long Dy = __double_as_longlong(q.y) - yfi;
                        const long long Dz = __double_as_longlong(q.z) - zfi;
                        dxf = fmaf(__int2float_rn((int)(Dx >> 32)), sc_hi, __uint2float_rn((unsigned)Dx) * sc_lo);
                        dyf = fmaf(__int2float_rn((int)(Dy >> 32)), sc_hi, __uint2float_rn((unsigned)Dy) * sc_lo);
                        dzf = fmaf(__int2float_rn((int)(Dz >> 32)), sc_hi, __uint2float_rn((unsigned)Dz) * sc_lo);
                        mf = round_to_float(q.w);
                    } else if (MODE == kMixed) {
                        const double4_32a q = tile[k];
                        const double dx = q.x - gxi, dy = q.y - gyi, dz = q.z - gzi;   // FP64 displacement
                        if (CVT) { dxf = (float)dx; dyf = (float)dy; dzf = (float)dz; mf = (float)q.w; }
                        else { dxf = round_to_float(dx); dyf = round_to_float(dy); dzf = round_to_float(dz); mf = round_to_float(q.w); }
                    } else {
                        const float4 h = tile_s[2 * k], l = tile_s[2 * k + 1];
                        // The FP64 displacement from the two-float split: the hi difference is
                        // exact whenever it cancels (Sterbenz), the lo difference carries the rest.
                        dxf = (h.x - xih) + (l.x - xil);
                        dyf = (h.y - yih) + (l.y - yil);
                        dzf = (h.z - zih) + (l.z - zil);
                        mf = h.w;
                    }
                    const float r2 = fmaf(dxf, dxf, fmaf(dyf, dyf, fmaf(dzf, dzf, eps2f)));
                    const float ri = rsqrtf(r2);
                    float s = mf * ri * ri * ri;
                    s = skip ? 0.f : s;
                    // Compensated FP32-pair accumulation (Kahan).
                    float t, y;
                    y = fmaf(s, dxf, -fcx); t = fsx + y; fcx = (t - fsx) - y; fsx = t;
                    y = fmaf(s, dyf, -fcy); t = fsy + y; fcy = (t - fsy) - y; fsy = t;
                    y = fmaf(s, dzf, -fcz); t = fsz + y; fcz = (t - fsz) - y; fsz = t;
                }
            }
            if (MODE == kBasic) {
                double t, y;
                y = tx - cx; t = sx + y; cx = (t - sx) - y; sx = t;
                y = ty - cy; t = sy + y; cy = (t - sy) - y; sy = t;
                y = tz - cz; t = sz + y; cz = (t - sz) - y; sz = t;
            }
        }
    }
    if (!live) return;
    if (MODE == kMixed || MODE == kMixedSplit) {
        sx = (double)fsx - (double)fcx; sy = (double)fsy - (double)fcy; sz = (double)fsz - (double)fcz;
    } else {
        sx -= cx; sy -= cy; sz -= cz;
    }
    if (a.splits == 1) {
        a.ax[i] = sx; a.ay[i] = sy; a.az[i] = sz;
    } else {
        double* P = a.partial + (size_t)blockIdx.y * 3 * a.cap;
        P[i] = sx; P[a.cap + i] = sy; P[2 * a.cap + i] = sz;
    }
}

// Sum the j-split partials in split order (deterministic).  COMPENSATED
// carries TwoSum error terms across the split boundaries.
template <bool COMP>
__global__ void reduce_partials(const double* __restrict__ P, int splits, size_t cap, int N,
                                double* __restrict__ ax, double* __restrict__ ay, double* __restrict__ az) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    double out[3];
    for (int c = 0; c < 3; c++) {
        double s = 0., e = 0.;
        for (int k = 0; k < splits; k++) {
            const double v = P[(size_t)k * 3 * cap + (size_t)c * cap + i];
            if (COMP) {
                const double t = s + v;
                const double bp = t - s;
                e += (s - (t - bp)) + (v - bp);
                s = t;
            } else {
                s += v;
            }
        }
        out[c] = s + e;
    }
    ax[i] = out[0]; ay[i] = out[1]; az[i] = out[2];
}

// Pack (x, y, z, G*m) and, when requested, the float split used by MIXED_SPLIT.
__global__ void pack_j(ParticlesSoA p, int N, double G, double4_32a* __restrict__ jpos, float4* __restrict__ jsplit) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double x = p.x[i], y = p.y[i], z = p.z[i], gm = G * p.m[i];
    jpos[i] = make_double4_32a(x, y, z, gm);
    if (jsplit) {
        const float xh = (float)x, yh = (float)y, zh = (float)z;
        jsplit[2 * i] = make_float4(xh, yh, zh, (float)gm);
        jsplit[2 * i + 1] = make_float4((float)(x - (double)xh), (float)(y - (double)yh), (float)(z - (double)zh), 0.f);
    }
}

// Potential energy (src/tools.c:120-131, unsoftened): phi_i = sum_{j<Na, j!=i}
// G m_j / r_ij; E_pot = -(1/2) sum_{i<Na} m_i phi_i - sum_{Na<=i<Ni} m_i phi_i
// (active pairs appear twice in the gather, active-test pairs once).
__global__ void __launch_bounds__(kBlock) potential_kernel(const double4_32a* __restrict__ jpos, const double* __restrict__ m,
                                                           int Na, int Ni, double* __restrict__ out_block) {
    __shared__ double4_32a tile[kBlock];
    __shared__ double red[kBlock];
    const int i = blockIdx.x * kBlock + threadIdx.x;
    const bool live = i < Ni;
    const double4_32a pi = live ? jpos[i] : make_double4_32a(0., 0., 0., 0.);
    double phi = 0.;
    for (int jt = 0; jt < Na; jt += kBlock) {
        __syncthreads();
        const int jl = jt + threadIdx.x;
        tile[threadIdx.x] = jl < Na ? jpos[jl] : make_double4_32a(0., 0., 0., 0.);
        __syncthreads();
        const int nt = min(kBlock, Na - jt);
        for (int k = 0; k < nt; k++) {
            const double4_32a q = tile[k];
            const double dx = pi.x - q.x, dy = pi.y - q.y, dz = pi.z - q.z;
            const double term = q.w / sqrt(dx * dx + dy * dy + dz * dz);
            phi += (jt + k == i) ? 0.0 : term;
        }
    }
    red[threadIdx.x] = live ? -(i < Na ? 0.5 : 1.0) * m[i] * phi : 0.0;
    __syncthreads();
    for (int w = kBlock / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out_block[blockIdx.x] = red[0];
}

__global__ void kinetic_kernel(ParticlesSoA p, int Ni, double* __restrict__ out_block) {
    __shared__ double red[kBlock];
    const int i = blockIdx.x * kBlock + threadIdx.x;
    red[threadIdx.x] = i < Ni ? 0.5 * p.m[i] * (p.vx[i] * p.vx[i] + p.vy[i] * p.vy[i] + p.vz[i] * p.vz[i]) : 0.0;
    __syncthreads();
    for (int w = kBlock / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out_block[blockIdx.x] = red[0];
}

int sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

// Number of j-splits: enough CTAs to fill the GPU, and a CTA count close to a
// multiple of the SM count so the last wave is not ragged.
int choose_splits(int nbi, int jmax) {
    const int nsm = sm_count();
    const int per_sm = 6;
    const int smax_j = jmax > 0 ? (jmax + kBlock - 1) / kBlock : 1;   // at least one tile per split
    int smin = (nsm * per_sm + nbi - 1) / nbi;
    smin = smin < 1 ? 1 : (smin > smax_j ? smax_j : smin);
    int best = smin;
    double best_cost = 1e30;
    for (int s = smin; s <= smin + 48 && s <= smax_j; s++) {
        const double work = (double)nbi * s;
        const double ragged = std::ceil(work / nsm) / (work / nsm);
        const double cost = ragged * (1.0 + 0.002 * s);
        if (cost < best_cost) { best_cost = cost; best = s; }
    }
    return best;
}

GhostList* g_ghost_dev = nullptr;
int g_rinv_variant = kRinvSeriesInt;
bool g_mixed_cvt = false;
int g_disp_mode = 2;

template <int MODE, bool GEN>
void launch_mode(dim3 grid, cudaStream_t st, const DirectArgs& a) {
    if constexpr ((MODE == kBasic || MODE == kComp) && !GEN) {
        if (a.fix) {
            if (g_disp_mode == 1)
                direct_kernel<MODE, false, kRinvSeriesInt, true, 1><<<grid, kBlock, 0, st>>>(a, g_ghost_dev);
            else
                direct_kernel<MODE, false, kRinvSeriesInt, true, 2><<<grid, kBlock, 0, st>>>(a, g_ghost_dev);
            return;
        }
    }
    if constexpr (MODE == kMixed && !GEN) {
        if (a.fix) {
            direct_kernel<kMixed, false, kRinvSeries, false, 1><<<grid, kBlock, 0, st>>>(a, g_ghost_dev);
            return;
        }
    }
    if (MODE == kBasic || MODE == kComp) {
        switch (g_rinv_variant) {
            case kRinvLib: direct_kernel<MODE, GEN, kRinvLib, true><<<grid, kBlock, 0, st>>>(a, g_ghost_dev); break;
            case kRinvSeriesF32: direct_kernel<MODE, GEN, kRinvSeriesF32, true><<<grid, kBlock, 0, st>>>(a, g_ghost_dev); break;
            case kRinvSeries: direct_kernel<MODE, GEN, kRinvSeries, true><<<grid, kBlock, 0, st>>>(a, g_ghost_dev); break;
            default: direct_kernel<MODE, GEN, kRinvSeriesInt, true><<<grid, kBlock, 0, st>>>(a, g_ghost_dev); break;
        }
    } else if (MODE == kMixed && !g_mixed_cvt) {
        direct_kernel<MODE, GEN, kRinvSeries, false><<<grid, kBlock, 0, st>>>(a, g_ghost_dev);
    } else {
        direct_kernel<MODE, GEN, kRinvSeries, true><<<grid, kBlock, 0, st>>>(a, g_ghost_dev);
    }
}

}  // namespace

extern "C" int rgpu_set_kernel_variant(int rinv_variant, int mixed_cvt) {
    if (rinv_variant < 0 || rinv_variant > 3) return RGPU_ERR_ARG;
    g_rinv_variant = rinv_variant;
    g_mixed_cvt = mixed_cvt != 0;
    return RGPU_OK;
}

extern "C" int rgpu_set_displacement_mode(int mode) {
    if (mode < 0 || mode > 2) return RGPU_ERR_ARG;
    g_disp_mode = mode;
    return RGPU_OK;
}

int ensure_partial(rgpu_sim* s, size_t splits) {
    const size_t need = splits * 3 * s->cap;
    if (need <= s->partial_cap) return RGPU_OK;
    if (s->partial) cudaFree(s->partial);
    s->partial = nullptr;
    s->partial_cap = 0;
    RGPU_CUDA(s, cudaMalloc(&s->partial, need * sizeof(double)));
    s->partial_cap = need;
    return RGPU_OK;
}

int direct_accel(rgpu_sim* s, int gravity) {
    const int N = (int)s->N;
    if (N == 0) return RGPU_OK;
    const rgpu_config& c = s->cfg;
    const int Na = (int)n_active(s);
    int mode = kBasic;
    if (gravity == RGPU_GRAVITY_COMPENSATED) mode = kComp;
    else if (gravity == RGPU_GRAVITY_MIXED) mode = kMixed;
    else if (gravity == RGPU_GRAVITY_MIXED_SPLIT) mode = kMixedSplit;

    // Ghost boxes apply to BASIC and the mixed forms; COMPENSATED has none
    // (src/gravity.c:284-531).
    GhostList gl;
    gl.n = 0;
    const bool ghosts = mode != kComp && (c.N_ghost_x || c.N_ghost_y || c.N_ghost_z);
    if (ghosts) {
        for (int gx = -c.N_ghost_x; gx <= c.N_ghost_x; gx++)
            for (int gy = -c.N_ghost_y; gy <= c.N_ghost_y; gy++)
                for (int gz = -c.N_ghost_z; gz <= c.N_ghost_z; gz++) {
                    if (gl.n >= 125) return set_error(s, RGPU_ERR_UNSUPPORTED, "more than 125 ghost boxes");
                    double gb[6];
                    ghostbox(c, gx, gy, gz, gb);
                    gl.off[gl.n][0] = gb[0]; gl.off[gl.n][1] = gb[1]; gl.off[gl.n][2] = gb[2];
                    gl.n++;
                }
    }
    const bool general = ghosts || Na != N || c.testparticle_type || c.gravity_ignore_terms;
    if (general) {
        if (!g_ghost_dev) RGPU_CUDA(s, cudaMalloc(&g_ghost_dev, sizeof(GhostList)));
        if (!ghosts) { gl.n = 1; gl.off[0][0] = gl.off[0][1] = gl.off[0][2] = 0.; }
        RGPU_CUDA(s, cudaMemcpyAsync(g_ghost_dev, &gl, sizeof(GhostList), cudaMemcpyHostToDevice, s->stream));
    }

    // BASIC, COMPENSATED and MIXED without ghosts or pair exclusions form the
    // displacement on the integer pipe from fixed-point positions; the scale
    // words (FixScale) live in the jsplit buffer, which only MIXED_SPLIT uses.
    const bool fix = g_disp_mode != 0 && (mode == kBasic || mode == kComp || mode == kMixed) && !general;
    FixScale* fsc = nullptr;
    if (fix) {
        fsc = reinterpret_cast<FixScale*>(s->jsplit);
        RGPU_CUDA(s, cudaMemsetAsync(&fsc->dmax, 0, sizeof(unsigned long long), s->stream));
        max_abs_coord<<<std::min<int>(grid_for(N, 256), 2 * 152), 256, 0, s->stream>>>(s->p, N, &fsc->dmax);
        pack_fix<<<grid_for(N, 256), 256, 0, s->stream>>>(s->p, N, c.G, c.softening * c.softening, fsc,
                                                          reinterpret_cast<FixBody*>(s->jpos));
        g_launches += 2;
    } else {
        pack_j<<<grid_for(N, 256), 256, 0, s->stream>>>(s->p, N, c.G, s->jpos, mode == kMixedSplit ? s->jsplit : nullptr);
        g_launches++;
    }

    const int nbi = (N + kBlock - 1) / kBlock;
    const int jmax = c.testparticle_type ? N : Na;
    const int splits = choose_splits(nbi, jmax);
    if (splits > 1) RGPU_TRY(ensure_partial(s, (size_t)splits));

    DirectArgs a{};
    a.jpos = s->jpos; a.jsplit = s->jsplit;
    a.N = N; a.Na = Na; a.tp = c.testparticle_type; a.ign = c.gravity_ignore_terms;
    a.eps2 = c.softening * c.softening;
    a.splits = splits;
    a.ax = s->p.ax; a.ay = s->p.ay; a.az = s->p.az;
    a.partial = s->partial; a.cap = s->cap;
    a.fix = fsc;
    const dim3 grid(nbi, splits);

    ktimer_begin(s);
    switch (mode) {
        case kBasic: general ? launch_mode<kBasic, true>(grid, s->stream, a) : launch_mode<kBasic, false>(grid, s->stream, a); break;
        case kComp: general ? launch_mode<kComp, true>(grid, s->stream, a) : launch_mode<kComp, false>(grid, s->stream, a); break;
        case kMixed: general ? launch_mode<kMixed, true>(grid, s->stream, a) : launch_mode<kMixed, false>(grid, s->stream, a); break;
        default: general ? launch_mode<kMixedSplit, true>(grid, s->stream, a) : launch_mode<kMixedSplit, false>(grid, s->stream, a); break;
    }
    g_launches++;
    ktimer_end(s);
    RGPU_CUDA(s, cudaGetLastError());
    if (splits > 1) {
        if (mode == kComp)
            reduce_partials<true><<<grid_for(N, 256), 256, 0, s->stream>>>(s->partial, splits, s->cap, N, s->p.ax, s->p.ay, s->p.az);
        else
            reduce_partials<false><<<grid_for(N, 256), 256, 0, s->stream>>>(s->partial, splits, s->cap, N, s->p.ax, s->p.ay, s->p.az);
        g_launches++;
    }
    return RGPU_OK;
}

int direct_energy(rgpu_sim* s, double* e) {
    const int N = (int)s->N;
    *e = 0.;
    if (N == 0) return RGPU_OK;
    const int Na = (int)n_active(s);
    const int Ni = s->cfg.testparticle_type == 0 ? Na : N;
    const int nb = grid_for(Ni > 0 ? Ni : 1, kBlock);
    std::vector<double> hk(nb), hp(nb);
    double* d = nullptr;
    RGPU_CUDA(s, cudaMalloc(&d, sizeof(double) * 2 * nb));
    pack_j<<<grid_for(N, 256), 256, 0, s->stream>>>(s->p, N, s->cfg.G, s->jpos, nullptr);
    kinetic_kernel<<<nb, kBlock, 0, s->stream>>>(s->p, Ni, d);
    potential_kernel<<<nb, kBlock, 0, s->stream>>>(s->jpos, s->p.m, Na, Ni, d + nb);
    g_launches += 3;
    cudaMemcpyAsync(hk.data(), d, sizeof(double) * nb, cudaMemcpyDeviceToHost, s->stream);
    cudaMemcpyAsync(hp.data(), d + nb, sizeof(double) * nb, cudaMemcpyDeviceToHost, s->stream);
    const cudaError_t err = cudaStreamSynchronize(s->stream);
    cudaFree(d);
    if (err != cudaSuccess) return check_cuda(s, err, "energy");
    double ek = 0., ep = 0.;
    for (int b = 0; b < nb; b++) { ek += hk[b]; ep += hp[b]; }
    *e = ek + ep;
    return RGPU_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free direct summation.
//
// Some callers cannot allocate device memory at the moment they need forces:
// a host framework that owns every device allocation through its own pool, a
// REBOUND build embedded in a process whose allocator is locked down, or code
// running where cudaMalloc is not allowed.  rgpu_direct_accel_noalloc takes the
// caller's device arrays for inputs and outputs and keeps its scratch (the
// packed j-bodies, their float split and the j-split partial sums) in the
// file-scope device array below, which every GPU that loads the library holds
// until the process exits.
//
// Sizes: at most kNoAllocMaxN particles; the j-range is cut into at most
// kNoAllocMaxSplits chunks.  Every scratch slot the reduction reads is written
// earlier in the same call, so nothing needs clearing between calls.  All
// calls share the one array: calls that overlap on the GPU (different streams,
// or different host threads) race on it and must be serialised by the caller.
// ---------------------------------------------------------------------------
#include <mutex>

namespace {

constexpr int kNoAllocMaxN = 65536;
constexpr int kNoAllocMaxSplits = 4;
constexpr size_t kNoAllocJpos = (size_t)kNoAllocMaxN * sizeof(double4_32a);       // 2 MiB
constexpr size_t kNoAllocJsplit = (size_t)kNoAllocMaxN * 2 * sizeof(float4);     // 2 MiB
constexpr size_t kNoAllocPartial = (size_t)kNoAllocMaxSplits * 3 * kNoAllocMaxN * sizeof(double);  // 6 MiB
constexpr size_t kNoAllocBytes = kNoAllocJpos + kNoAllocJsplit + kNoAllocPartial;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kNoAllocMaxDevices = 64;
void* g_noalloc_addr[kNoAllocMaxDevices] = {nullptr};
std::mutex g_noalloc_mu;

// Device address of the scratch array on the current device.  Host code cannot
// use the symbol itself (it names a host-side shadow); the address is looked
// up once per device with that device current.
int noalloc_scratch(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return RGPU_ERR_CUDA; }
    if (dev < 0 || dev >= kNoAllocMaxDevices) return RGPU_ERR_CAPACITY;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) { cudaGetLastError(); return RGPU_ERR_CUDA; }
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return RGPU_OK;
}

}  // namespace

extern "C" int rgpu_direct_accel_noalloc(const double* x, const double* y, const double* z, const double* m,
                                         double* ax, double* ay, double* az, int64_t n, double G,
                                         double softening, int gravity, void* stream) {
    if (n < 0 || (n > 0 && (!x || !y || !z || !m || !ax || !ay || !az))) return RGPU_ERR_ARG;
    if (n > kNoAllocMaxN) return RGPU_ERR_CAPACITY;
    int mode;
    switch (gravity) {
        case RGPU_GRAVITY_BASIC: mode = kBasic; break;
        case RGPU_GRAVITY_COMPENSATED: mode = kComp; break;
        case RGPU_GRAVITY_MIXED: mode = kMixed; break;
        case RGPU_GRAVITY_MIXED_SPLIT: mode = kMixedSplit; break;
        default: return RGPU_ERR_ARG;
    }
    void* base = nullptr;
    const int rc = noalloc_scratch(&base);      // first call on a device: symbol lookup
    if (rc) return rc;
    if (n == 0) return RGPU_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int N = (int)n;
    double4_32a* jpos = (double4_32a*)base;
    float4* jsplit = (float4*)((char*)base + kNoAllocJpos);
    double* partial = (double*)((char*)base + kNoAllocJpos + kNoAllocJsplit);

    ParticlesSoA p{};
    p.x = const_cast<double*>(x); p.y = const_cast<double*>(y); p.z = const_cast<double*>(z);
    p.m = const_cast<double*>(m);
    pack_j<<<grid_for(N, 256), 256, 0, st>>>(p, N, G, jpos, mode == kMixedSplit ? jsplit : nullptr);
    const int nbi = (N + kBlock - 1) / kBlock;
    int splits = choose_splits(nbi, N);
    if (splits > kNoAllocMaxSplits) splits = kNoAllocMaxSplits;
    DirectArgs a{};
    a.jpos = jpos; a.jsplit = jsplit;
    a.N = N; a.Na = N; a.tp = 0; a.ign = 0;
    a.eps2 = softening * softening;
    a.splits = splits;
    a.ax = ax; a.ay = ay; a.az = az;
    a.partial = partial; a.cap = (size_t)kNoAllocMaxN;
    const dim3 grid(nbi, splits);
    switch (mode) {
        case kBasic: launch_mode<kBasic, false>(grid, st, a); break;
        case kComp: launch_mode<kComp, false>(grid, st, a); break;
        case kMixed: launch_mode<kMixed, false>(grid, st, a); break;
        default: launch_mode<kMixedSplit, false>(grid, st, a); break;
    }
    if (splits > 1) {
        if (mode == kComp)
            reduce_partials<true><<<grid_for(N, 256), 256, 0, st>>>(partial, splits, (size_t)kNoAllocMaxN, N, ax, ay, az);
        else
            reduce_partials<false><<<grid_for(N, 256), 256, 0, st>>>(partial, splits, (size_t)kNoAllocMaxN, N, ax, ay, az);
    }
    g_launches += splits > 1 ? 3 : 2;
    return cudaGetLastError() == cudaSuccess ? RGPU_OK : RGPU_ERR_CUDA;
}
