// Pair-force factor 1/(r^2 + eps^2)^(3/2) from 64-bit fixed-point displacements,
// computed on the integer pipes.  GB300 runs FP64 at ~1/64 of its FP32 rate but
// keeps two full-width integer pipes (ALU and IMAD) that issue alongside the
// FP64 unit, so the pair kernel moves everything except the final products
// onto them:
//
//   1. r^2 + eps^2 exactly, as a 128-bit integer (sum of the squared int64
//      displacements plus eps^2 on the same 2^-2s grid);
//   2. an FP32 seed y0 ~ (r^2)^(-1/2) from the leading 24 bits (MUFU rsqrt);
//   3. the residual h = 1 - r^2 y0^2 in 2^-62 fixed point (exact enough: the
//      seed error makes |h| < 2^-20, so h is needed to ~2^-55 absolute);
//   4. (r^2)^(-3/2) = y0^3 (1 - h)^(-3/2) = y0^3 (1 + 3/2 h + 15/8 h^2 + O(h^3)),
//      the binomial series, with y0^3 formed exactly (72-bit product) and the
//      product y0^3 (1 + c) taken as a 64x64 high multiply;
//   5. one rounding to double.
//
// Relative error of the result: the final rounding (2^-53) plus a few 2^-59
// from truncated low bits and the O(h^3) tail (measured against 80-bit extended
// precision over 3e6 random cases: at most 1.04 half-ulps).  The helpers compile
// for the host too, so their arithmetic can be checked on a CPU.
#pragma once
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define FIX_HD __host__ __device__ __forceinline__
#else
#define FIX_HD inline
#endif

namespace fixpair {

typedef unsigned long long u64;
typedef unsigned int u32;
typedef unsigned __int128 u128;

FIX_HD int clz64(u64 v) {
#ifdef __CUDA_ARCH__
    return __clzll((long long)v);
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}

FIX_HD u64 wide(u32 a, u32 b) { return (u64)a * b; }

FIX_HD u32 mulhi32(u32 a, u32 b) {
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return (u32)(((u64)a * b) >> 32);
#endif
}

FIX_HD u64 mulhi64(u64 a, u64 b) {
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return (u64)(((u128)a * b) >> 64);
#endif
}

FIX_HD double bits_double(u64 b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double d;
    memcpy(&d, &b, 8);
    return d;
#endif
}

FIX_HD float bits_float(u32 b) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float f;
    memcpy(&f, &b, 4);
    return f;
#endif
}

FIX_HD u32 float_bits(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    u32 b;
    memcpy(&b, &f, 4);
    return b;
#endif
}

// |v| of a two's-complement int64 and its sign mask (all ones when negative).
FIX_HD u64 abs64(long long v, u64* sign) {
    const u64 s = (u64)(v >> 63);
    *sign = s;
    return ((u64)v ^ s) - s;
}

// sign * a * 2^-s as a double (sign: all-ones mask when negative), round to
// nearest even; ebias = 1086 - s.  Callers keep s <= 1022 so nonzero results are
// normal numbers.
FIX_HD double abs_to_double(u64 a, u64 sign, int ebias) {
    const int lz = clz64(a);                                         // 64 when a == 0
    const u64 n = a << (lz & 63);                                    // bit 63 set
    const u64 r = n + 0x3FFull + ((n >> 11) & 1ull);                 // half an ulp, ties to even
    const int carry = r < n;                                         // rounded up to 2^64
    const u64 frac = carry ? 0ull : ((r >> 11) & 0xFFFFFFFFFFFFFull);
    const u64 e = (u64)(ebias - lz + carry);
    const u64 bits = (e << 52) | frac | (sign << 63);
    return a ? bits_double(bits) : 0.0;
}

// Seed y0 ~ x^(-1/2) for x in [1, 4) given as float bits.  The device uses the
// hardware approximation (relative error below 2^-21); the host uses the
// correctly rounded value, optionally perturbed by a caller-given factor to
// exercise the seed-error range.
#ifndef FIXPAIR_HOST_SEED
#define FIXPAIR_HOST_SEED(x) (1.0f / sqrtf(x))
#endif
FIX_HD float seed_rsqrt(float x) {
#ifdef __CUDA_ARCH__
    return rsqrtf(x);
#else
    return FIXPAIR_HOST_SEED(x);
#endif
}

// ---------------------------------------------------------------------------
// Limb forms: the same arithmetic arranged for 32-bit integer instructions.

FIX_HD int clz32(u32 v) {
#ifdef __CUDA_ARCH__
    return __clz((int)v);
#else
    return v ? __builtin_clz(v) : 32;
#endif
}

// (hi << n) | (lo >> (32 - n)) for n in [0, 31].
FIX_HD u32 shf_l(u32 lo, u32 hi, int n) {
#ifdef __CUDA_ARCH__
    return __funnelshift_l(lo, hi, n);
#else
    return n ? (hi << n) | (lo >> (32 - n)) : hi;
#endif
}

// (lo >> n) | (hi << (32 - n)) for n in [0, 31].
FIX_HD u32 shf_r(u32 lo, u32 hi, int n) {
#ifdef __CUDA_ARCH__
    return __funnelshift_r(lo, hi, n);
#else
    return n ? (lo >> n) | (hi << (32 - n)) : lo;
#endif
}

FIX_HD u32 shl_clamp(u32 v, int n) {   // v << n, 0 for n >= 32
#ifdef __CUDA_ARCH__
    return __funnelshift_lc(0u, v, n);
#else
    return n >= 32 ? 0u : v << n;
#endif
}

// |xj - xi| of two int64 fixed-point coordinates as 32-bit limbs, and the sign
// of the difference (all ones when negative).
FIX_HD void sub_abs(long long xj, long long xi, u32& ah, u32& al, u32& sg) {
    const long long d = xj - xi;
    const u64 m = (u64)(d >> 63);
    const u64 a = ((u64)d ^ m) - m;
    ah = (u32)(a >> 32);
    al = (u32)a;
    sg = (u32)m;
}

// Multi-word sums below are written as multiply-accumulate chains (the IMAD
// pipe) rather than add/compare carry chains (the ALU pipe): the two pipes
// issue side by side and the ALU pipe is the one the pair kernel saturates.
FIX_HD u64 mad_wide(u32 a, u32 b, u64 c) { return (u64)a * b + c; }

// sign * (ah 2^32 + al) 2^-s as a double, rounded to nearest (ties away from
// zero: one add on the assembled bits); ebias1 = 1085 - s (the biased exponent
// minus one).  Callers keep s <= 1022 so nonzero results are normal numbers.
FIX_HD double limbs_to_double(u32 ah, u32 al, u32 sg, int ebias1) {
    const bool big = ah != 0;
    const u32 c = big ? ah : al;
    const int lz = clz32(c);                                         // 32 when c == 0
    const u32 x = shl_clamp(al, lz);
    const u32 th = big ? shf_l(al, ah, lz) : x;                      // leading 32 bits, bit 31 set (0 when c == 0)
    const u32 tl = big ? x : 0u;
    const int e1 = (big ? ebias1 : ebias1 - 32) - lz;
    const u32 hi = ((u32)e1 << 20) + (th >> 11);
    const u32 lo = shf_l(tl, th, 21);
    const u64 r = (((u64)hi << 32) | lo) + ((tl >> 10) & 1u);
    const u32 keep = c ? 0xFFFFFFFFu : 0u;
    const u32 rh = ((u32)(r >> 32) & keep) | (sg & 0x80000000u);
    return bits_double(((u64)rh << 32) | (u32)r);                    // lo is already 0 when c == 0
}

// The factor (r^2 + eps^2)^(-3/2) from the limbs of |dx|, |dy|, |dz| (< 2^62
// each), with eps^2 2^2s pre-split as e0 + e1 2^32 + e2 2^62 (e0 < 2^32,
// e1 < 2^30, e2 < 2^62), as F 2^(e3 - 59) with F in [2^58, 2^62).  Returns false
// for a zero radius.  UNIFORM: all 32 lanes of the warp call it together (lets
// the common normalisation take a warp-uniform branch).
template <bool UNIFORM>
FIX_HD bool rinv3_core(u32 xh, u32 xl, u32 yh, u32 yl, u32 zh, u32 zl, u64 e0, u64 e1, u64 e2, int two_s, u64& F, int& e3) {
    // 1. r^2 + eps^2 = S2 2^62 + S1 2^32 + S0 with a 31-bit split b = bh 2^31 + bl:
    //    b^2 = bh^2 2^62 + bh bl 2^32 + bl^2, each product < 2^62, no carries.
    u64 S0 = e0, S1 = e1, S2 = e2;
    {
        const u32 bl = xl & 0x7FFFFFFFu, bh = shf_l(xl, xh, 1);
        S0 = mad_wide(bl, bl, S0); S1 = mad_wide(bh, bl, S1); S2 = mad_wide(bh, bh, S2);
    }
    {
        const u32 bl = yl & 0x7FFFFFFFu, bh = shf_l(yl, yh, 1);
        S0 = mad_wide(bl, bl, S0); S1 = mad_wide(bh, bl, S1); S2 = mad_wide(bh, bh, S2);
    }
    {
        const u32 bl = zl & 0x7FFFFFFFu, bh = shf_l(zl, zh, 1);
        S0 = mad_wide(bl, bl, S0); S1 = mad_wide(bh, bl, S1); S2 = mad_wide(bh, bh, S2);
    }
    // R = S2 2^62 + S1 2^32 + S0 as limbs r3 r2 r1 (r0 = low word of S0 is not needed)
    const u64 m1 = (u64)(u32)(S0 >> 32) + (u32)S1 + ((u32)S2 << 30);  // limb 1 plus its carries (< 2^34)
    const u64 m2 = (S1 >> 32) + (S2 >> 2) + (m1 >> 32);              // limbs 2, 3
    const u32 r3 = (u32)(m2 >> 32), r2 = (u32)m2, r1 = (u32)m1;
    int lz;
    u32 Th, Tl;
#ifdef __CUDA_ARCH__
    const bool fast = UNIFORM ? __all_sync(0xffffffffu, r3 != 0u) : r3 != 0u;
#else
    const bool fast = r3 != 0u;
#endif
    // 2. T = leading 63 bits (bit 62 set): R < 2^127 leaves at least one leading zero
    if (fast) {
        lz = clz32(r3);
        Th = shf_l(r2, r3, lz - 1);
        Tl = shf_l(r1, r2, lz - 1);
    } else {
        const u64 hi = m2, lo = ((u64)r1 << 32) | (u32)S0;
        if ((hi | lo) == 0) return false;
        u64 T;
        if (hi) {
            lz = clz64(hi);
            T = lz > 1 ? (hi << (lz - 1)) | (lo >> (65 - lz)) : hi;
        } else {
            lz = clz64(lo);
            T = lz ? lo << (lz - 1) : lo >> 1;
            lz += 64;
        }
        Th = (u32)(T >> 32);
        Tl = (u32)T;
    }
    const int e = 127 - lz - two_s;                                  // r^2 = (T / 2^62) 2^e
    const int q = e & 1, k = e >> 1;                                 //     = M 2^q 2^(2k)
    // 3. FP32 seed for x = M 2^q in [1, 4); y0 = Y 2^(ey - 23)
    const u32 xb = (q ? 0x40000000u : 0x3F800000u) | ((Th >> 7) & 0x7FFFFFu);
    const u32 yb = float_bits(seed_rsqrt(bits_float(xb)));
    const int ey = (int)(yb >> 23) - 127;
    const u32 Y = (yb & 0x7FFFFFu) | 0x800000u;
    //    h = 1 - x y0^2 = 1 - T Y^2 2^(q + 2 ey - 108), as H = h 2^62 = 2^62 - (T Y^2 / 2^32) >> sh;
    //    T Y^2 / 2^32 with Y^2 = A 2^32 + B: Th A 2^32 + (Th B + Tl A + hi32(Tl B)); Th < 2^31
    // keeps the bracket below 2^64
    const u64 Y2 = wide(Y, Y);
    const u32 B = (u32)Y2, A = (u32)(Y2 >> 32);
    const u64 acc = mad_wide(Tl, A, mad_wide(Th, B, (u64)mulhi32(Tl, B)));
    const u64 C = wide(Th, A);                                       // < 2^47, weight 2^32
    const u64 mid = (acc >> 32) + (u32)C;                            // limb 1 (+ carry in bit 32)
    const u32 p0 = (u32)acc, p1 = (u32)mid, p2 = (u32)(C >> 32) + (u32)(mid >> 32);
    const int sh = 14 - q - 2 * ey;                                  // in [13, 18]
    const u32 s_lo = shf_r(p0, p1, sh), s_hi = shf_r(p1, p2, sh);
    const long long H = (long long)((1ull << 62) - (((u64)s_hi << 32) | s_lo));
    // 4. 1 + c = 1 + 3/2 h + 15/8 h^2 = 1 + (12 h + 15 h^2) / 8 in 2^-62 fixed point
    const int Hs = (int)(H >> 20);
    const u32 Q = (u32)((u64)((long long)Hs * Hs) >> 22);
    const long long C12 = (long long)mad_wide(Q, 15u, (u64)(H * 12));
    const u64 M1 = (1ull << 62) + (u64)(C12 >> 3);
    //    y0^3 (1 + c): Y^3 / 2^8 from Y8 = Y 2^8 as (Y8^2 Y8) / 2^32, times M1, high 64 bits
    //    (the low-by-low partial product lies below the last kept bit and is dropped)
    const u32 Y8 = Y << 8;
    const u64 Y2s = wide(Y8, Y8);
    const u64 Y3 = mad_wide((u32)(Y2s >> 32), Y8, (u64)mulhi32((u32)Y2s, Y8));
    const u32 Y3h = (u32)(Y3 >> 32), Y3l = (u32)Y3, Mh = (u32)(M1 >> 32), Ml = (u32)M1;
    F = mad_wide(Y3h, Mh, (u64)mulhi32(Y3h, Ml) + mulhi32(Y3l, Mh));   // F 2^(3 ey - 59) = y0^3 (1+c)
    e3 = 3 * (ey - k);                                                // (r^2)^(-3/2) = F 2^(e3 - 59)
    return true;
}

// sign-less n 2^(be1 + 1 - 1086) for a 64-bit n with bit 63 set, rounded to double.
FIX_HD double assemble(u32 nh, u32 nl, int be1) {
    const u32 bhi = ((u32)be1 << 20) + (nh >> 11);                    // the leading 1 adds the last exponent unit
    const u32 blo = shf_l(nl, nh, 21);
    const u64 bits = (((u64)bhi << 32) | blo) + ((nl >> 10) & 1u);   // round: carries into the exponent if needed
    if ((unsigned)be1 > 2045u) return be1 < 0 ? 0.0 : bits_double(0x7FF0000000000000ull);
    return bits_double(bits);
}

// 5. (r^2)^(-3/2) = F 2^(e3 - 59), rounded to double.
FIX_HD double finish_f(u64 F, int e3) {
    const u32 Fh = (u32)(F >> 32), Fl = (u32)F;
    const int lzf = clz32(Fh);                                       // F >= 2^58: Fh != 0
    return assemble(shf_l(Fl, Fh, lzf), Fl << lzf, 1026 - lzf + e3);
}

// 5'. G m (r^2)^(-3/2): the 53-bit mantissa of G m (double bits gm) multiplied in
// before the one rounding (the high 64 bits of F 2^2 x mantissa 2^11; the
// low-by-low partial product lies below the last kept bit).  A zero, subnormal
// or non-finite G m takes an FP64 product.
FIX_HD double finish_mf(u64 F, int e3, u64 gm) {
    const int em = (int)((gm >> 52) & 0x7FF);
    if ((unsigned)(em - 1) >= 2046u) return bits_double(gm) * finish_f(F, e3);
    const u64 A = F << 2, B = (((gm & 0xFFFFFFFFFFFFFull) | (1ull << 52)) << 11);
    const u32 ah = (u32)(A >> 32), al = (u32)A, bh = (u32)(B >> 32), bl = (u32)B;
    const u64 P = mad_wide(ah, bh, (u64)mulhi32(ah, bl) + mulhi32(al, bh));   // F m 2^-51, in [2^59, 2^64)
    const u32 Ph = (u32)(P >> 32), Pl = (u32)P;
    const int lzp = clz32(Ph);
    return assemble(shf_l(Pl, Ph, lzp), Pl << lzp, em + 2 - lzp + e3);
}

template <bool UNIFORM>
FIX_HD double rinv3_limbs(u32 xh, u32 xl, u32 yh, u32 yl, u32 zh, u32 zl, u64 e0, u64 e1, u64 e2, int two_s) {
    u64 F;
    int e3;
    if (!rinv3_core<UNIFORM>(xh, xl, yh, yl, zh, zl, e0, e1, e2, two_s, F, e3)) return bits_double(0x7FF0000000000000ull);
    return finish_f(F, e3);
}

// G m / (r^2 + eps^2)^(3/2) with G m given as double bits.
template <bool UNIFORM>
FIX_HD double rinv3m_limbs(u32 xh, u32 xl, u32 yh, u32 yl, u32 zh, u32 zl, u64 e0, u64 e1, u64 e2, int two_s,
                           u64 gm) {
    u64 F;
    int e3;
    if (!rinv3_core<UNIFORM>(xh, xl, yh, yl, zh, zl, e0, e1, e2, two_s, F, e3))
        return bits_double(gm) * bits_double(0x7FF0000000000000ull);          // as G m / 0
    return finish_mf(F, e3, gm);
}

}  // namespace fixpair
