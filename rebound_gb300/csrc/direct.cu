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

// Per-evaluation scale words, written by pack_fix and read by every pair thread,
// and the counters of the exactness guard (see "Exactness guard" below).
struct __align__(16) FixScale {
    unsigned long long dmax;               // max |coordinate| as double bits (atomicMax target)
    int shift;                             // s
    int two_s;                             // 2 s
    unsigned long long e0, e1, e2;         // eps^2 2^2s = e0 + e1 2^32 + e2 2^62 (e0 < 2^32, e1 < 2^30)
    int n_inexact;                         // bodies with a coordinate off the 2^-s grid
    int n_redo;                            // particles whose force is recomputed in FP64
    int all;                               // 1: every particle is recomputed in FP64
    int eps_off;                           // eps^2 is not exact on the 2^-2s grid
    float delta;                           // bound on the FP32 displacement error of the bound kernels
};

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

// Blocks of pack_fix and fix_scatter: 256 bodies each.
constexpr int kGuardBlock = 256;

// Fixed-point records of every body.  With `err` set (BASIC / COMPENSATED) it
// also writes, for the exactness guard, each body's rounding error
// |x - X 2^-s| (Euclidean, rounded up to float; +inf for a non-finite body),
// its FP32 position and G m, and the number of inexact bodies of each
// 256-body block (bcnt).
__global__ void __launch_bounds__(kGuardBlock) pack_fix(ParticlesSoA p, int N, double G, double eps2,
                                                        FixScale* __restrict__ sc, FixBody* __restrict__ out,
                                                        float* __restrict__ err, float4* __restrict__ fpos,
                                                        int* __restrict__ bcnt) {
    const double mx = __longlong_as_double((long long)sc->dmax);
    int s = (mx > 0. && isfinite(mx)) ? 60 - ilogb(mx) : 60;
    if (eps2 > 0. && isfinite(eps2)) s = min(s, (123 - ilogb(eps2)) >> 1);
    s = min(s, 1022);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool inexact = false;
    if (i < N) {
        const double x = p.x[i], y = p.y[i], z = p.z[i];
        FixBody b;
        b.x = __double2ll_rn(scalbn(x, s));
        b.y = __double2ll_rn(scalbn(y, s));
        b.z = __double2ll_rn(scalbn(z, s));
        b.gm = G * p.m[i];
        out[i] = b;
        if (err) {
            // x - X 2^-s is exact: X converts back exactly (below 2^53 as an integer,
            // above it x 2^s already was one) and x lies within half a grid step of it.
            const double rx = x - scalbn((double)b.x, -s);
            const double ry = y - scalbn((double)b.y, -s);
            const double rz = z - scalbn((double)b.z, -s);
            const double e = sqrt(fma(rx, rx, fma(ry, ry, rz * rz))) * (1.0 + 0x1p-20);
            const float ef = e <= 3.0e38 ? (float)e : __int_as_float(0x7f800000);   // NaN / overflow -> +inf
            err[i] = ef;
            fpos[i] = make_float4((float)x, (float)y, (float)z, (float)b.gm);
            inexact = ef != 0.f;
        }
    }
    if (bcnt) {
        __shared__ int wsum[kGuardBlock / 32];
        const unsigned bal = __ballot_sync(0xffffffffu, inexact);
        if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = __popc(bal);
        __syncthreads();
        if (threadIdx.x == 0) {
            int t = 0;
            for (int w = 0; w < kGuardBlock / 32; w++) t += wsum[w];
            bcnt[blockIdx.x] = t;
        }
    }
    if (i == 0) {
        sc->n_inexact = 0;
        sc->n_redo = 0;
        sc->all = 0;
        sc->delta = isfinite(mx) ? (float)scalbn(mx, -20) : __int_as_float(0x7f800000);
        unsigned long long hi = 0, lo = 0;
        bool eps_off = false;
        if (eps2 > 0. && isfinite(eps2)) {
            int ee;
            const double fr = frexp(eps2, &ee);                        // eps2 = fr 2^ee, fr in [0.5, 1)
            const unsigned long long m53 = (unsigned long long)scalbn(fr, 53);
            const int sh = ee - 53 + 2 * s;                             // eps2 2^2s = m53 2^sh < 2^124
            if (sh >= 64) { hi = m53 << (sh - 64); }
            else if (sh > 0) { hi = m53 >> (64 - sh); lo = m53 << sh; }
            else if (sh > -64) { lo = m53 >> (-sh); }
            // eps^2 off the 2^-2s grid (a softening below ~2^-31 max|x|): r^2 + eps^2 is
            // then not exact and the guard sends every particle to the FP64 kernel
            eps_off = sh <= -64 || (sh < 0 && (m53 & ((1ull << (-sh)) - 1ull)) != 0ull);
        }
        sc->eps_off = eps_off ? 1 : 0;
        sc->shift = s;
        sc->two_s = 2 * s;
        sc->e0 = lo & 0xFFFFFFFFull;
        sc->e1 = (lo >> 32) & 0x3FFFFFFFull;
        sc->e2 = (lo >> 62) | (hi << 2);
    }
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
    // the exactness guard sent every particle to the FP64 recomputation
    if ((MODE == kBasic || MODE == kComp) && FIX && a.fix->all) return;
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

// --- Mixed-precision pair kernel (MIXED, MIXED_SPLIT; all particles active, no
// ghost boxes) --------------------------------------------------------------------
// Each coordinate is held as a two-float split x = xh + xl (xh = (float)x, xl =
// (float)(x - xh), exact), so the displacement (xh_j - xh_i) + (xl_j - xl_i) is
// the FP64 displacement to ~2^-48 of the coordinates before its final rounding
// to FP32 (the high difference is exact whenever it cancels).  r^2, rsqrt and
// G m / r^3 are FP32.  The arithmetic runs on Blackwell's packed FP32x2 FMA pipe
// (__fadd2_rn / __ffma2_rn / __fmul2_rn): every lane evaluates two j-bodies per
// instruction, 9 packed instructions for the displacements, 3 for r^2, 3 for
// G m / r^3 and 3 for the accumulation per two pairs, plus one MUFU rsqrt per
// pair.  Pair terms are summed in FP32 over 32 j-pairs (64 terms) and each such
// sum is folded into the per-particle accumulator: FP64 (MIXED, the FP64
// accumulation of the mixed form) or a compensated FP32 pair (MIXED_SPLIT).
// j-bodies are stored in pairs, 64 B each: (xh0, xh1, yh0, yh1),
// (zh0, zh1, Gm0, Gm1), (xl0, xl1, yl0, yl1), (zl0, zl1, 0, 0).
struct __align__(16) SplitPair {
    float4 a, b, c, d;
};

__global__ void pack_split2(ParticlesSoA p, int N, double G, SplitPair* __restrict__ out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (N + 1) / 2) return;
    float xh[2], yh[2], zh[2], gm[2], xl[2], yl[2], zl[2];
    for (int k = 0; k < 2; k++) {
        const int i = 2 * q + k;
        if (i < N) {
            const double x = p.x[i], y = p.y[i], z = p.z[i];
            xh[k] = (float)x; yh[k] = (float)y; zh[k] = (float)z;
            xl[k] = (float)(x - (double)xh[k]); yl[k] = (float)(y - (double)yh[k]); zl[k] = (float)(z - (double)zh[k]);
            gm[k] = (float)(G * p.m[i]);
        } else {   // the partner of the last body of an odd N: massless, at the origin
            xh[k] = yh[k] = zh[k] = xl[k] = yl[k] = zl[k] = gm[k] = 0.f;
        }
    }
    SplitPair P;
    P.a = make_float4(xh[0], xh[1], yh[0], yh[1]);
    P.b = make_float4(zh[0], zh[1], gm[0], gm[1]);
    P.c = make_float4(xl[0], xl[1], yl[0], yl[1]);
    P.d = make_float4(zl[0], zl[1], 0.f, 0.f);
    out[q] = P;
}

constexpr int kSubPairs = 32;   // j-pairs summed in FP32 before a fold

// MUFU reciprocal square root with subnormal inputs flushed to zero: one
// instruction (rsqrtf adds the scaling that keeps subnormal inputs exact).
// Used where the argument is at least eps^2 > 0.
__device__ __forceinline__ float rsqrt_ftz(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// ACC: 0 = compensated FP32 pair (MIXED_SPLIT), 1 = FP64 (MIXED).  SOFT: eps^2 > 0,
// so the self pair (d = 0) contributes exactly 0 and needs no test.
template <int ACC, bool SOFT>
__global__ void __launch_bounds__(kBlock) direct_split2(DirectArgs a, const SplitPair* __restrict__ jp) {
    __shared__ SplitPair tile[kBlock / 2];
    const int i = blockIdx.x * kBlock + threadIdx.x;
    const bool live = i < a.N;
    const int chunk = (((a.N + a.splits - 1) / a.splits) + kBlock - 1) / kBlock * kBlock;
    const int j0 = blockIdx.y * chunk;
    const int j1 = min(a.N, j0 + chunk);

    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    SplitPair P;
    P.a = P.b = P.c = P.d = z4;
    if (live) P = jp[i >> 1];
    const bool odd = i & 1;
    const float xh = odd ? P.a.y : P.a.x, yh = odd ? P.a.w : P.a.z, zh = odd ? P.b.y : P.b.x;
    const float xl = odd ? P.c.y : P.c.x, yl = odd ? P.c.w : P.c.z, zl = odd ? P.d.y : P.d.x;
    const float2 nxh = make_float2(-xh, -xh), nyh = make_float2(-yh, -yh), nzh = make_float2(-zh, -zh);
    const float2 nxl = make_float2(-xl, -xl), nyl = make_float2(-yl, -yl), nzl = make_float2(-zl, -zl);
    const float ef = (float)a.eps2;
    const float2 e2 = make_float2(ef, ef);

    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;   // ACC 0
    double dx64 = 0., dy64 = 0., dz64 = 0.;                               // ACC 1

    for (int jt = j0; jt < j1; jt += kBlock) {
        const int nj = min(kBlock, j1 - jt);
        const int nq = (nj + 1) >> 1;
        __syncthreads();
        {
            const float4* src = reinterpret_cast<const float4*>(jp + (jt >> 1));
            float4* dst = reinterpret_cast<float4*>(tile);
            for (int u = threadIdx.x; u < 2 * kBlock; u += kBlock) dst[u] = u < 4 * nq ? src[u] : z4;
        }
        __syncthreads();
        for (int qs = 0; qs < nq; qs += kSubPairs) {
            const int qe = min(nq, qs + kSubPairs);
            float2 ax = make_float2(0.f, 0.f), ay = ax, az = ax;
#pragma unroll 4
            for (int q = qs; q < qe; q++) {
                const SplitPair J = tile[q];
                const float2 dx = __fadd2_rn(__fadd2_rn(make_float2(J.a.x, J.a.y), nxh),
                                             __fadd2_rn(make_float2(J.c.x, J.c.y), nxl));
                const float2 dy = __fadd2_rn(__fadd2_rn(make_float2(J.a.z, J.a.w), nyh),
                                             __fadd2_rn(make_float2(J.c.z, J.c.w), nyl));
                const float2 dz = __fadd2_rn(__fadd2_rn(make_float2(J.b.x, J.b.y), nzh),
                                             __fadd2_rn(make_float2(J.d.x, J.d.y), nzl));
                const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __ffma2_rn(dz, dz, e2)));
                const float2 ri = SOFT ? make_float2(rsqrt_ftz(r2.x), rsqrt_ftz(r2.y))
                                       : make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
                float2 s = __fmul2_rn(__fmul2_rn(ri, ri), __fmul2_rn(make_float2(J.b.z, J.b.w), ri));
                if (!SOFT) {
                    const int j = jt + 2 * q;
                    s.x = (j == i || j >= j1) ? 0.f : s.x;
                    s.y = (j + 1 == i || j + 1 >= j1) ? 0.f : s.y;
                }
                ax = __ffma2_rn(s, dx, ax);
                ay = __ffma2_rn(s, dy, ay);
                az = __ffma2_rn(s, dz, az);
            }
            const float tx = ax.x + ax.y, ty = ay.x + ay.y, tz = az.x + az.y;
            if (ACC == 1) {
                dx64 += (double)tx;
                dy64 += (double)ty;
                dz64 += (double)tz;
            } else {
                float t, y;
                y = tx - cx; t = sx + y; cx = (t - sx) - y; sx = t;
                y = ty - cy; t = sy + y; cy = (t - sy) - y; sy = t;
                y = tz - cz; t = sz + y; cz = (t - sz) - y; sz = t;
            }
        }
    }
    if (!live) return;
    double ox, oy, oz;
    if (ACC == 1) {
        ox = dx64; oy = dy64; oz = dz64;
    } else {
        ox = (double)sx - (double)cx; oy = (double)sy - (double)cy; oz = (double)sz - (double)cz;
    }
    if (a.splits == 1) {
        a.ax[i] = ox; a.ay[i] = oy; a.az[i] = oz;
    } else {
        double* Pp = a.partial + (size_t)blockIdx.y * 3 * a.cap;
        Pp[i] = ox; Pp[a.cap + i] = oy; Pp[2 * a.cap + i] = oz;
    }
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

// --- Exactness guard for the fixed-point forms ---------------------------------
// A coordinate below 2^-8 max|x| has bits under the 2^-s grid and is rounded to
// it (error e_b <= 2^-s-1 per component), so a pair of bodies can be displaced
// by up to |e_i| + |e_j| from where the FP64 subtraction puts them.  The force
// G m d / (d^2 + eps^2)^(3/2) has a Jacobian of norm at most
// 2 G m / (r^2 + eps^2)^(3/2) (r the smallest distance on the segment between
// the two displacements), so the fixed-point force on particle i is off by at
// most
//     B_i = 2 sum_j s_ij (|e_i| + |e_j|) = 2 (|e_i| S_i + T_i),
//     S_i = sum_j s_ij,   T_i = sum_j s_ij |e_j|,   s_ij >= G m_j / (r^2 + eps^2)^(3/2),
// where s_ij is evaluated in FP32 at the distance lowered by a bound on its
// FP32 error (delta = 2^-20 max|x|), so it is an upper bound.  S_i is needed
// only for inexact i and T_i only runs over inexact j, so on the inputs this
// kernel is built for (a Plummer sphere: about 6 % of the bodies inexact) the
// two bound sums cost a few percent of the FP64 pair kernel.  Every particle
// with B_i > kGuardTau |a_i| (or a non-finite a_i or B_i) is recomputed by an
// FP64 kernel (the FP64 subtraction, as the reference forms it); more than a
// quarter of the bodies inexact, or eps^2 off the grid, sends every particle
// there and the fixed-point kernel returns at once.  Everything is decided on
// the device from counters in FixScale; the host launches a fixed sequence.
// Results are deterministic: the inexact list is compacted in index order,
// each bound and each recomputed force is summed by one thread in a fixed order.
constexpr double kGuardTau = 5e-15;
constexpr int kGuardSplitMax = 16;         // j-chunks of the S_i sums

// Exclusive scan of the per-block inexact counts (one CTA of 1024 threads);
// sets n_inexact and the all-FP64 switch.
__global__ void __launch_bounds__(1024) fix_scan(int* __restrict__ bcnt, int nb, int N, FixScale* __restrict__ sc) {
    __shared__ int wtot[32];
    __shared__ int carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += 1024) {
        const int k = base + threadIdx.x;
        const int v = k < nb ? bcnt[k] : 0;
        int x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wtot[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int t = wtot[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            wtot[lane] = t;
        }
        __syncthreads();
        const int excl = carry + (warp ? wtot[warp - 1] : 0) + x - v;
        if (k < nb) bcnt[k] = excl;
        __syncthreads();
        if (threadIdx.x == 1023) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        sc->n_inexact = carry;
        sc->n_redo = 0;
        sc->all = (sc->eps_off || (long long)carry * 4 > (long long)N) ? 1 : 0;
    }
}

// The inexact bodies in index order.
__global__ void __launch_bounds__(kGuardBlock) fix_scatter(const float* __restrict__ err, const int* __restrict__ boff,
                                                           int N, const FixScale* __restrict__ sc, int* __restrict__ list) {
    if (sc->all) return;
    __shared__ int wsum[kGuardBlock / 32];
    const int i = blockIdx.x * kGuardBlock + threadIdx.x;
    const bool inexact = i < N && err[i] != 0.f;
    const unsigned bal = __ballot_sync(0xffffffffu, inexact);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wsum[warp] = __popc(bal);
    __syncthreads();
    int off = boff[blockIdx.x];
    for (int w = 0; w < warp; w++) off += wsum[w];
    if (inexact) list[off + __popc(bal & ((1u << lane) - 1u))] = i;
}

// Upper bound on G m_j / (r^2 + eps^2)^(3/2) for two j-bodies at once (packed
// FP32x2), from FP32 displacements.  R = sqrt(r_f^2 + eps^2) is within delta of
// its exact value (the map r -> sqrt(r^2 + eps^2) is 1-Lipschitz and the FP32
// distance r_f is within delta of the exact one), so the term is at most
// G m / (R - delta)^3 = G m y^3 / (1 - delta y)^3 <= G m y^3 (1 + 4 delta y) for
// delta y <= 1/8 (y = 1/R; the FP32 rounding of r^2 and rsqrt stays inside the
// 5 % slack of the final bound).  t4 = 4 delta y is returned for the range check.
__device__ __forceinline__ float2 s_upper2(float2 dx, float2 dy, float2 dz, float2 gm, float2 e2, float2 d4, float2& t4) {
    const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __ffma2_rn(dz, dz, e2)));
    const float2 y = make_float2(rsqrt_ftz(r2.x), rsqrt_ftz(r2.y));   // a flushed r^2 gives +inf: flagged
    t4 = __fmul2_rn(d4, y);
    const float2 s0 = __fmul2_rn(__fmul2_rn(y, y), __fmul2_rn(gm, y));
    return __ffma2_rn(t4, s0, s0);
}

// Pair-layout tile of FP32 positions for the bound kernels: j-bodies 2q, 2q+1
// as (x0, x1, y0, y1), (z0, z1, g0, g1), (e0, e1, id0, id1) with g = G m and, in
// the T kernel, e = the body's rounding error and id its index.
struct __align__(16) BoundPair {
    float4 a, b, c;
};

// Accumulate one tile's two-body terms into S (W = false) or T (W = true: the
// terms weighted by e).  The pair holding particle `self` is excluded; `tm`
// collects the largest 4 delta y of the included pairs.
template <bool W>
__device__ __forceinline__ void bound_tile(const BoundPair* __restrict__ tile, int nj, int qself_or_idx, bool by_index,
                                           int self, float2 nx, float2 ny, float2 nz, float2 e2, float2 d4,
                                           float2& acc, float& tm) {
    const int nq = (nj + 1) >> 1;
#pragma unroll 4
    for (int q = 0; q < nq; q++) {
        const BoundPair J = tile[q];
        const float2 dx = __fadd2_rn(make_float2(J.a.x, J.a.y), nx);
        const float2 dy = __fadd2_rn(make_float2(J.a.z, J.a.w), ny);
        const float2 dz = __fadd2_rn(make_float2(J.b.x, J.b.y), nz);
        float2 t4;
        float2 su = s_upper2(dx, dy, dz, make_float2(J.b.z, J.b.w), e2, d4, t4);
        bool x0, x1;   // excluded halves
        if (by_index) {
            x0 = __float_as_int(J.c.z) == self;
            x1 = __float_as_int(J.c.w) == self;
        } else {
            x0 = q == qself_or_idx && !(self & 1);
            x1 = q == qself_or_idx && (self & 1);
        }
        x1 = x1 || 2 * q + 1 >= nj;   // the empty half of an odd tile's last pair
        su.x = x0 ? 0.f : su.x;
        su.y = x1 ? 0.f : su.y;
        tm = fmaxf(tm, fmaxf(x0 ? 0.f : t4.x, x1 ? 0.f : t4.y));
        acc = W ? __ffma2_rn(su, make_float2(J.c.x, J.c.y), acc) : __fadd2_rn(acc, su);
    }
}

// S_i for the inexact particles: chunk y of the j-range per work item, written
// to spart[y][i] (+inf when a pair left the range of the bound).
__global__ void __launch_bounds__(kBlock) fix_bound_S(const float4* __restrict__ fpos, const int* __restrict__ list,
                                                      const FixScale* __restrict__ sc, int N, float eps2f, int ny,
                                                      float* __restrict__ spart, size_t cap) {
    if (sc->all) return;
    __shared__ BoundPair tile[kBlock / 2];
    const int ni = sc->n_inexact;
    const int nbi = (ni + kBlock - 1) / kBlock;
    const int chunk = ((N + ny - 1) / ny + kBlock - 1) / kBlock * kBlock;
    const float d4f = 4.f * sc->delta;
    const float2 d4 = make_float2(d4f, d4f), e2 = make_float2(eps2f, eps2f);
    for (int w = blockIdx.x; w < nbi * ny; w += gridDim.x) {
        const int b = w % nbi, y = w / nbi;
        const int pos = b * kBlock + threadIdx.x;
        const int i = pos < ni ? list[pos] : -1;
        const float4 pi = i >= 0 ? fpos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float2 nx = make_float2(-pi.x, -pi.x), nyv = make_float2(-pi.y, -pi.y), nz = make_float2(-pi.z, -pi.z);
        const int j0 = y * chunk, j1 = min(N, j0 + chunk);
        float2 S = make_float2(0.f, 0.f);
        float tm = 0.f;
        for (int jt = j0; jt < j1; jt += kBlock) {
            __syncthreads();
            {
                const int jl = jt + threadIdx.x;
                const float4 q = jl < j1 ? fpos[jl] : make_float4(0.f, 0.f, 0.f, 0.f);
                float* t = reinterpret_cast<float*>(&tile[threadIdx.x >> 1]);
                const int h = threadIdx.x & 1;
                t[0 + h] = q.x; t[2 + h] = q.y; t[4 + h] = q.z; t[6 + h] = q.w;
            }
            __syncthreads();
            const int d = i - jt;   // self inside this tile when 0 <= d < kBlock
            bound_tile<false>(tile, min(kBlock, j1 - jt), (d >= 0 && d < kBlock) ? (d >> 1) : -1, false, d, nx, nyv,
                              nz, e2, d4, S, tm);
        }
        if (i >= 0) {
            const float Sv = S.x + S.y;
            spart[(size_t)y * cap + i] = tm <= 0.5f ? Sv : __int_as_float(0x7f800000);
        }
    }
}

// T_i over the inexact bodies for every particle, the bound B_i, and the list
// of particles to recompute.
__global__ void __launch_bounds__(kBlock) fix_bound_flag(const float4* __restrict__ fpos, const float* __restrict__ err,
                                                         const int* __restrict__ list, FixScale* __restrict__ sc, int N,
                                                         float eps2f, int ny, const float* __restrict__ spart, size_t cap,
                                                         const double* __restrict__ ax, const double* __restrict__ ay,
                                                         const double* __restrict__ az, int* __restrict__ redo) {
    if (sc->all) return;
    const int ni = sc->n_inexact;
    if (ni == 0) return;                  // every coordinate on the grid: the fixed-point sums are exact
    __shared__ BoundPair tile[kBlock / 2];
    const float d4f = 4.f * sc->delta;
    const float2 d4 = make_float2(d4f, d4f), e2 = make_float2(eps2f, eps2f);
    const int nb = (N + kBlock - 1) / kBlock;
    for (int b = blockIdx.x; b < nb; b += gridDim.x) {
        const int i = b * kBlock + threadIdx.x;
        const bool live = i < N;
        const float4 pi = live ? fpos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float2 nx = make_float2(-pi.x, -pi.x), ny2 = make_float2(-pi.y, -pi.y), nz = make_float2(-pi.z, -pi.z);
        float2 T = make_float2(0.f, 0.f);
        float tm = 0.f;
        for (int jt = 0; jt < ni; jt += kBlock) {
            __syncthreads();
            {
                const int k = jt + threadIdx.x;
                float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
                float e = 0.f;
                int j = -1;
                if (k < ni) { j = list[k]; q = fpos[j]; e = err[j]; }
                float* t = reinterpret_cast<float*>(&tile[threadIdx.x >> 1]);
                const int h = threadIdx.x & 1;
                t[0 + h] = q.x; t[2 + h] = q.y; t[4 + h] = q.z; t[6 + h] = q.w;
                t[8 + h] = e; t[10 + h] = __int_as_float(j);
            }
            __syncthreads();
            bound_tile<true>(tile, min(kBlock, ni - jt), -1, true, i, nx, ny2, nz, e2, d4, T, tm);
        }
        if (live) {
            const float Ei = err[i];
            float S = 0.f;
            if (Ei != 0.f)
                for (int y = 0; y < ny; y++) S += spart[(size_t)y * cap + i];
            // 2 (|e_i| S_i + T_i) with 5 % slack for the FP32 evaluation
            double B = 2.1 * ((double)Ei * (double)S + (double)(T.x + T.y));
            if (!(tm <= 0.5f)) B = __longlong_as_double(0x7ff0000000000000ll);
            const double amag = sqrt(ax[i] * ax[i] + ay[i] * ay[i] + az[i] * az[i]);
            if (!(B <= kGuardTau * amag)) redo[atomicAdd(&sc->n_redo, 1)] = i;
        }
    }
}

// FP64 pair term of the recomputation: the FP64 subtraction (src/gravity.c:215-233),
// r^2 and m/r^3 as in the FP64 kernel.
__device__ __forceinline__ double redo_term(double xj, double yj, double zj, double gmj, double xi, double yi,
                                            double zi, double eps2, double& dx, double& dy, double& dz) {
    dx = xj - xi; dy = yj - yi; dz = zj - zi;
    const double r2 = fma(dx, dx, fma(dy, dy, fma(dz, dz, eps2)));
    return m_rinv3<kRinvSeriesInt>(r2, gmj);
}

// Short recomputation lists (kRedoWarpMax particles or fewer): one warp per
// (particle, j-chunk), the lanes striding over the chunk's bodies (all lanes
// busy however few particles there are), Kahan sums per lane combined across
// the warp in a fixed order; chunk sums go to part[(c * 3 + comp) * nr + p].
constexpr int kRedoWarpMax = 2048;

struct WarpSplit {
    int nr, J, chunk;
};
__device__ __forceinline__ WarpSplit warp_split(const FixScale* sc, int N, int target) {
    WarpSplit w;
    w.nr = sc->all ? 0 : sc->n_redo;
    if (w.nr > kRedoWarpMax) w.nr = 0;
    const int maxJ = max(1, (N + 63) / 64);          // at least two bodies per lane
    int J = w.nr ? (target + w.nr - 1) / w.nr : 1;
    w.J = max(1, min(J, maxJ));
    w.chunk = ((N + w.J - 1) / w.J + 31) / 32 * 32;
    return w;
}

// (s, c) + (t, d) for Kahan pairs, as a TwoSum of the sums plus the compensations.
__device__ __forceinline__ void kahan_merge(double& s, double& c, double t, double d) {
    const double u = s + t;
    const double bp = u - s;
    const double e = (s - (u - bp)) + (t - bp);
    s = u;
    c = c + d - e;
}

template <int MODE>
__global__ void __launch_bounds__(kBlock) fix_redo_warp(ParticlesSoA p, int N, double G, double eps2,
                                                        const FixScale* __restrict__ sc, const int* __restrict__ redo,
                                                        int target, double* __restrict__ part) {
    const WarpSplit ws = warp_split(sc, N, target);
    if (ws.nr == 0) return;
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (kBlock / 32);
    for (int w = blockIdx.x * (kBlock / 32) + (threadIdx.x >> 5); w < ws.nr * ws.J; w += warps) {
        const int pidx = w % ws.nr, c = w / ws.nr;
        const int i = redo[pidx];
        const double xi = p.x[i], yi = p.y[i], zi = p.z[i];
        const int j0 = c * ws.chunk, j1 = min(N, j0 + ws.chunk);
        double s[3] = {0., 0., 0.}, k[3] = {0., 0., 0.};     // Kahan sum and compensation
        for (int j = j0 + lane; j < j1; j += 32) {
            double dx, dy, dz;
            double f = redo_term(p.x[j], p.y[j], p.z[j], G * p.m[j], xi, yi, zi, eps2, dx, dy, dz);
            f = (j == i) ? 0.0 : f;
            const double v[3] = {f * dx, f * dy, f * dz};
            for (int q = 0; q < 3; q++) {
                const double y = v[q] - k[q];
                const double t = s[q] + y;
                k[q] = (t - s[q]) - y;
                s[q] = t;
            }
        }
        // fixed-order butterfly over the lanes
        for (int o = 16; o > 0; o >>= 1)
            for (int q = 0; q < 3; q++) {
                const double t = __shfl_down_sync(0xffffffffu, s[q], o);
                const double d = __shfl_down_sync(0xffffffffu, k[q], o);
                kahan_merge(s[q], k[q], t, d);
            }
        if (lane == 0)
            for (int q = 0; q < 3; q++) part[((size_t)c * 3 + q) * ws.nr + pidx] = s[q] - k[q];
    }
    (void)MODE;
}

__global__ void fix_redo_warp_reduce(const double* __restrict__ part, const FixScale* __restrict__ sc,
                                     const int* __restrict__ redo, int N, int target,
                                     double* __restrict__ ax, double* __restrict__ ay, double* __restrict__ az) {
    const WarpSplit ws = warp_split(sc, N, target);
    if (ws.nr == 0) return;
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x / 32);
    for (int pidx = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); pidx < ws.nr; pidx += warps) {
        double s[3] = {0., 0., 0.}, k[3] = {0., 0., 0.};
        for (int c = lane; c < ws.J; c += 32)
            for (int q = 0; q < 3; q++) kahan_merge(s[q], k[q], part[((size_t)c * 3 + q) * ws.nr + pidx], 0.);
        for (int o = 16; o > 0; o >>= 1)
            for (int q = 0; q < 3; q++) {
                const double t = __shfl_down_sync(0xffffffffu, s[q], o);
                const double d = __shfl_down_sync(0xffffffffu, k[q], o);
                kahan_merge(s[q], k[q], t, d);
            }
        if (lane == 0) {
            const int i = redo[pidx];
            ax[i] = s[0] - k[0]; ay[i] = s[1] - k[1]; az[i] = s[2] - k[2];
        }
    }
}

// Long recomputation lists (more than kRedoWarpMax particles, or every particle):
// 256-particle blocks against shared-memory tiles of j-bodies, the j-range cut
// into J chunks so that about `target` work items exist.
struct RedoSplit {
    int nr, nb, J, chunk;
    size_t stride;
};
__device__ __forceinline__ RedoSplit redo_split(const FixScale* sc, int N, int target) {
    RedoSplit r;
    r.nr = sc->all ? N : sc->n_redo;
    if (!sc->all && r.nr <= kRedoWarpMax) r.nr = 0;
    r.nb = (r.nr + kBlock - 1) / kBlock;
    const int ntile = (N + kBlock - 1) / kBlock;
    int J = r.nb ? (target + r.nb - 1) / r.nb : 1;
    J = max(1, min(J, ntile));
    r.J = J;
    r.chunk = (ntile + J - 1) / J * kBlock;
    r.stride = (size_t)r.nb * kBlock;
    return r;
}

// BASIC sums each 256-body tile with FMAs and folds it with Kahan compensation,
// COMPENSATED compensates every term (src/gravity.c:325-343).  One chunk's
// sums go to part[c][3][pos].
template <int MODE>
__global__ void __launch_bounds__(kBlock) fix_redo(ParticlesSoA p, int N, double G, double eps2,
                                                   const FixScale* __restrict__ sc, const int* __restrict__ redo,
                                                   int target, double* __restrict__ part) {
    const RedoSplit rs = redo_split(sc, N, target);
    if (rs.nr == 0) return;
    const bool all = sc->all != 0;
    __shared__ double4_32a tile[kBlock];
    for (int w = blockIdx.x; w < rs.nb * rs.J; w += gridDim.x) {
        const int b = w % rs.nb, c = w / rs.nb;
        const int pos = b * kBlock + threadIdx.x;
        const int i = pos < rs.nr ? (all ? pos : redo[pos]) : -1;
        double xi = 0., yi = 0., zi = 0.;
        if (i >= 0) { xi = p.x[i]; yi = p.y[i]; zi = p.z[i]; }
        const int j0 = c * rs.chunk, j1 = min(N, j0 + rs.chunk);
        double sx = 0., sy = 0., sz = 0., cx = 0., cy = 0., cz = 0.;
        for (int jt = j0; jt < j1; jt += kBlock) {
            __syncthreads();
            const int jl = jt + threadIdx.x;
            tile[threadIdx.x] = jl < j1 ? make_double4_32a(p.x[jl], p.y[jl], p.z[jl], G * p.m[jl])
                                        : make_double4_32a(0., 0., 0., 0.);
            __syncthreads();
            const int nt = min(kBlock, j1 - jt);
            double tx = 0., ty = 0., tz = 0.;
            for (int k = 0; k < nt; k++) {
                const double4_32a q = tile[k];
                double dx, dy, dz;
                double s = redo_term(q.x, q.y, q.z, q.w, xi, yi, zi, eps2, dx, dy, dz);
                s = (jt + k == i) ? 0.0 : s;
                if (MODE == kBasic) {
                    tx = fma(s, dx, tx); ty = fma(s, dy, ty); tz = fma(s, dz, tz);
                } else {
                    double t, y;
                    y = s * dx - cx; t = sx + y; cx = (t - sx) - y; sx = t;
                    y = s * dy - cy; t = sy + y; cy = (t - sy) - y; sy = t;
                    y = s * dz - cz; t = sz + y; cz = (t - sz) - y; sz = t;
                }
            }
            if (MODE == kBasic) {
                double t, y;
                y = tx - cx; t = sx + y; cx = (t - sx) - y; sx = t;
                y = ty - cy; t = sy + y; cy = (t - sy) - y; sy = t;
                y = tz - cz; t = sz + y; cz = (t - sz) - y; sz = t;
            }
        }
        if (i >= 0) {
            double* P = part + (size_t)c * 3 * rs.stride;
            P[pos] = sx - cx; P[rs.stride + pos] = sy - cy; P[2 * rs.stride + pos] = sz - cz;
        }
    }
}

// Sum the recomputation's chunks in chunk order (TwoSum carries) into a[i].
__global__ void fix_redo_reduce(const double* __restrict__ part, const FixScale* __restrict__ sc,
                                const int* __restrict__ redo, int N, int target,
                                double* __restrict__ ax, double* __restrict__ ay, double* __restrict__ az) {
    const RedoSplit rs = redo_split(sc, N, target);
    const bool all = sc->all != 0;
    for (int pos = blockIdx.x * blockDim.x + threadIdx.x; pos < rs.nr; pos += gridDim.x * blockDim.x) {
        const int i = all ? pos : redo[pos];
        double out[3];
        for (int comp = 0; comp < 3; comp++) {
            double s = 0., e = 0.;
            for (int c = 0; c < rs.J; c++) {
                const double v = part[((size_t)c * 3 + comp) * rs.stride + pos];
                const double t = s + v;
                const double bp = t - s;
                e += (s - (t - bp)) + (v - bp);
                s = t;
            }
            out[comp] = s + e;
        }
        ax[i] = out[0]; ay[i] = out[1]; az[i] = out[2];
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

// MIXED / MIXED_SPLIT without ghost boxes or pair exclusions: the packed
// FP32x2 kernel over j-bodies packed by pack_split2.
void launch_split2(int mode, dim3 grid, cudaStream_t st, const DirectArgs& a, const SplitPair* jp) {
    const bool soft = (float)a.eps2 >= 1.17549435e-38f;   // eps^2 a normal float: r^2 never subnormal
    if (mode == kMixed) {
        if (soft) direct_split2<1, true><<<grid, kBlock, 0, st>>>(a, jp);
        else direct_split2<1, false><<<grid, kBlock, 0, st>>>(a, jp);
    } else {
        if (soft) direct_split2<0, true><<<grid, kBlock, 0, st>>>(a, jp);
        else direct_split2<0, false><<<grid, kBlock, 0, st>>>(a, jp);
    }
}

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

// Device buffers of the exactness guard, sized for `cap` particles.
struct FixGuard {
    size_t cap = 0;
    void* block = nullptr;      // one allocation holding everything below
    FixScale* sc = nullptr;
    float* err = nullptr;       // [cap] rounding error per body
    float4* fpos = nullptr;     // [cap] FP32 position and G m
    int* list = nullptr;        // [cap] inexact bodies in index order
    int* redo = nullptr;        // [cap] particles recomputed in FP64
    int* bcnt = nullptr;        // [cap / 256 + 1] per-block counts, then offsets
    float* spart = nullptr;     // [kGuardSplitMax][cap] S_i chunk sums
    double* rpart = nullptr;    // recomputation chunk sums
    size_t rpart_len = 0;
};

// Work items of the FP64 recomputation: tiled (about two per resident CTA) and
// warp-per-particle (about two per resident warp), and the grid of both.
static int redo_target() { return sm_count() * 8; }
static int redo_warp_target() { return sm_count() * 64; }
static int redo_grid() { return sm_count() * 4; }

static int ensure_fixguard(rgpu_sim* s) {
    if (s->fixg && s->fixg->cap >= s->cap) return RGPU_OK;
    direct_free(s);
    FixGuard* g = new FixGuard();
    const size_t cap = s->cap;
    const size_t nb = cap / kGuardBlock + 1;
    g->rpart_len = std::max((size_t)(redo_target() + nb) * 3 * kBlock,
                            (size_t)(redo_warp_target() + kRedoWarpMax) * 3);
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t bytes = al(sizeof(FixScale)) + al(cap * 4) + al(cap * 16) + 2 * al(cap * 4) + al(nb * 4) +
                         al(kGuardSplitMax * cap * 4) + al(g->rpart_len * 8);
    if (cudaMalloc(&g->block, bytes) != cudaSuccess) {
        delete g;
        return check_cuda(s, cudaGetLastError(), "cudaMalloc exactness guard");
    }
    char* q = (char*)g->block;
    g->sc = (FixScale*)q; q += al(sizeof(FixScale));
    g->err = (float*)q; q += al(cap * 4);
    g->fpos = (float4*)q; q += al(cap * 16);
    g->list = (int*)q; q += al(cap * 4);
    g->redo = (int*)q; q += al(cap * 4);
    g->bcnt = (int*)q; q += al(nb * 4);
    g->spart = (float*)q; q += al(kGuardSplitMax * cap * 4);
    g->rpart = (double*)q;
    g->cap = cap;
    s->fixg = g;
    return RGPU_OK;
}

void direct_free(rgpu_sim* s) {
    if (!s->fixg) return;
    cudaFree(s->fixg->block);
    delete s->fixg;
    s->fixg = nullptr;
}

extern "C" int rgpu_sim_guard_stats(rgpu_sim* s, int64_t* n_inexact, int64_t* n_redo) {
    if (!s || !n_inexact || !n_redo) return RGPU_ERR_ARG;
    *n_inexact = -1;
    *n_redo = -1;
    if (!s->fixg) return RGPU_OK;
    FixScale h;
    RGPU_CUDA(s, cudaMemcpyAsync(&h, s->fixg->sc, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
    RGPU_CUDA(s, cudaStreamSynchronize(s->stream));
    *n_inexact = h.n_inexact;
    *n_redo = h.all ? (int64_t)s->N : h.n_redo;
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

    // BASIC and COMPENSATED without ghosts or pair exclusions form the pair on the
    // integer pipes from fixed-point positions; MIXED and MIXED_SPLIT without them
    // run the packed FP32x2 kernel over two-float splits.
    const bool fix = g_disp_mode != 0 && (mode == kBasic || mode == kComp) && !general;
    const bool split2 = (mode == kMixed || mode == kMixedSplit) && !general;
    // BASIC and COMPENSATED promise the FP64 result: the exactness guard checks
    // the grid rounding and recomputes the particles it could affect.
    const bool guard = fix;
    FixScale* fsc = nullptr;
    FixGuard* fg = nullptr;
    const int nbg = (int)grid_for(N, kGuardBlock);
    if (fix) {
        RGPU_TRY(ensure_fixguard(s));
        fg = s->fixg;
        fsc = fg->sc;
        RGPU_CUDA(s, cudaMemsetAsync(&fsc->dmax, 0, sizeof(unsigned long long), s->stream));
        max_abs_coord<<<std::min<int>(grid_for(N, 256), 2 * 152), 256, 0, s->stream>>>(s->p, N, &fsc->dmax);
        pack_fix<<<nbg, kGuardBlock, 0, s->stream>>>(s->p, N, c.G, c.softening * c.softening, fsc,
                                                     reinterpret_cast<FixBody*>(s->jpos), guard ? fg->err : nullptr,
                                                     guard ? fg->fpos : nullptr, guard ? fg->bcnt : nullptr);
        g_launches += 2;
        if (guard) {
            fix_scan<<<1, 1024, 0, s->stream>>>(fg->bcnt, nbg, N, fsc);
            fix_scatter<<<nbg, kGuardBlock, 0, s->stream>>>(fg->err, fg->bcnt, N, fsc, fg->list);
            g_launches += 2;
        }
    } else if (split2) {
        pack_split2<<<grid_for((N + 1) / 2, 256), 256, 0, s->stream>>>(s->p, N, c.G,
                                                                      reinterpret_cast<SplitPair*>(s->jsplit));
        g_launches++;
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
    if (split2) launch_split2(mode, grid, s->stream, a, reinterpret_cast<const SplitPair*>(s->jsplit));
    else switch (mode) {
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
    if (guard) {
        const float eps2f = (float)(c.softening * c.softening) * (1.f - 0x1p-22f);
        const int ny = std::max(1, std::min(kGuardSplitMax, (int)grid_for(N, kBlock)));
        const int persist = std::min<int>(sm_count() * 8, (int)grid_for(N, kBlock) * ny);
        fix_bound_S<<<persist, kBlock, 0, s->stream>>>(fg->fpos, fg->list, fsc, N, eps2f, ny, fg->spart, fg->cap);
        fix_bound_flag<<<std::min<int>(sm_count() * 8, (int)grid_for(N, kBlock)), kBlock, 0, s->stream>>>(
            fg->fpos, fg->err, fg->list, fsc, N, eps2f, ny, fg->spart, fg->cap, s->p.ax, s->p.ay, s->p.az, fg->redo);
        const double eps2 = c.softening * c.softening;
        // short lists: a warp per (particle, chunk); long lists: 256-particle tiles
        if (mode == kComp) {
            fix_redo_warp<kComp><<<redo_grid(), kBlock, 0, s->stream>>>(s->p, N, c.G, eps2, fsc, fg->redo,
                                                                       redo_warp_target(), fg->rpart);
            fix_redo<kComp><<<redo_grid(), kBlock, 0, s->stream>>>(s->p, N, c.G, eps2, fsc, fg->redo, redo_target(),
                                                                  fg->rpart);
        } else {
            fix_redo_warp<kBasic><<<redo_grid(), kBlock, 0, s->stream>>>(s->p, N, c.G, eps2, fsc, fg->redo,
                                                                        redo_warp_target(), fg->rpart);
            fix_redo<kBasic><<<redo_grid(), kBlock, 0, s->stream>>>(s->p, N, c.G, eps2, fsc, fg->redo, redo_target(),
                                                                   fg->rpart);
        }
        fix_redo_warp_reduce<<<64, 256, 0, s->stream>>>(fg->rpart, fsc, fg->redo, N, redo_warp_target(), s->p.ax,
                                                        s->p.ay, s->p.az);
        fix_redo_reduce<<<std::min<int>(sm_count() * 4, (int)grid_for(N, 256)), 256, 0, s->stream>>>(
            fg->rpart, fsc, fg->redo, N, redo_target(), s->p.ax, s->p.ay, s->p.az);
        g_launches += 6;
        RGPU_CUDA(s, cudaGetLastError());
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
    const bool split2 = mode == kMixed || mode == kMixedSplit;
    if (split2) pack_split2<<<grid_for((N + 1) / 2, 256), 256, 0, st>>>(p, N, G, reinterpret_cast<SplitPair*>(jsplit));
    else pack_j<<<grid_for(N, 256), 256, 0, st>>>(p, N, G, jpos, nullptr);
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
        default: launch_split2(mode, grid, st, a, reinterpret_cast<const SplitPair*>(jsplit)); break;
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
