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
// Relative error of the result: the final rounding (2^-53) plus a few 2^-60
// from truncated low bits and the O(h^3) tail.  The helpers compile for the host
// too, so their arithmetic can be checked against extended precision on a CPU.
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

// sign * a * 2^-s as a float, round to nearest even; fbias = 190 - s.  Results
// outside the float range flush to zero or saturate to infinity.
FIX_HD float abs_to_float(u64 a, u64 sign, int fbias) {
    const int lz = clz64(a);
    const u64 n = a << (lz & 63);
    const u64 r = n + 0x7FFFFFFFFFull + ((n >> 40) & 1ull);          // half an ulp at bit 40, ties to even
    const int carry = r < n;
    const u32 frac = carry ? 0u : (u32)((r >> 40) & 0x7FFFFFull);
    int e = fbias - lz + carry;
    u32 bits = ((u32)e << 23) | frac;
    bits = e <= 0 ? 0u : (e >= 255 ? 0x7F800000u : bits);
    bits |= (u32)sign & 0x80000000u;
    return a ? bits_float(bits) : 0.0f;
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

// (r^2 + eps^2)^(-3/2) for r^2 = (ax^2 + ay^2 + az^2) 2^-2s, eps^2 = (e2hi 2^64 +
// e2lo) 2^-2s; a* < 2^62, e2 < 2^124.  two_s = 2s.  Returns +inf for a zero
// radius (as 1/0 does), 0 or +inf where the result leaves the double range.
FIX_HD double rinv3(u64 ax, u64 ay, u64 az, u64 e2hi, u64 e2lo, int two_s) {
    // 1. exact r^2 + eps^2 on the 2^-2s grid: a^2 = ah^2 2^64 + 2 ah al 2^32 + al^2
    u128 R = ((u128)e2hi << 64) | e2lo;
    u64 p1 = 0, p2 = 0;
    {
        const u32 h = (u32)(ax >> 32), l = (u32)ax;
        R += wide(l, l); p1 += wide(h, l); p2 += wide(h, h);
    }
    {
        const u32 h = (u32)(ay >> 32), l = (u32)ay;
        R += wide(l, l); p1 += wide(h, l); p2 += wide(h, h);
    }
    {
        const u32 h = (u32)(az >> 32), l = (u32)az;
        R += wide(l, l); p1 += wide(h, l); p2 += wide(h, h);
    }
    R += (u128)p1 << 33;                                             // each ah al < 2^62: sum < 2^64
    R += (u128)p2 << 64;
    const u64 Rh = (u64)(R >> 64), Rl = (u64)R;
    if ((Rh | Rl) == 0) return bits_double(0x7FF0000000000000ull);
    const int lz = Rh ? clz64(Rh) : 64 + clz64(Rl);
    const u64 T = (u64)((R << lz) >> 64);                            // leading 64 bits, bit 63 set
    // r^2 = (T / 2^63) 2^e = M 2^q 2^(2k), M in [1, 2), q in {0, 1}
    const int e = 127 - lz - two_s;
    const int q = e & 1;
    const int k = e >> 1;                                            // floor(e / 2)

    // 2. FP32 seed for x = M 2^q in [1, 4)
    const u32 xb = ((u32)(127 + q) << 23) | ((u32)(T >> 40) & 0x7FFFFFu);
    const u32 yb = float_bits(seed_rsqrt(bits_float(xb)));
    const int ey = (int)(yb >> 23) - 127;                             // y0 = Y 2^(ey - 23)
    const u32 Y = (yb & 0x7FFFFFu) | 0x800000u;

    // 3. h = 1 - x y0^2 = 1 - T Y^2 2^(q + 2 ey - 109), as H = h 2^62
    const u64 Y2 = wide(Y, Y);                                       // < 2^48, exact
    const u32 Y2h = (u32)(Y2 >> 32), Y2l = (u32)Y2;
    const u32 Th = (u32)(T >> 32), Tl = (u32)T;
    const u128 P = ((u128)wide(Th, Y2h) << 32) + wide(Th, Y2l) + wide(Tl, Y2h) + mulhi32(Tl, Y2l);  // ~ T Y^2 / 2^32
    const int sh = 15 - q - 2 * ey;
    const long long H = (long long)((1ull << 62) - (u64)(P >> sh));

    // 4. 1 + c = 1 + 3/2 h + 15/8 h^2 in 2^-62 fixed point
    const int Hs = (int)(H >> 20);                                   // h 2^42, |Hs| < 2^22
    const long long Q = ((long long)Hs * Hs) >> 22;                  // h^2 2^62
    const u64 M1 = (1ull << 62) + (u64)(H + (H >> 1) + 2 * Q - (Q >> 3));
    //    y0^3 = Y^3 2^(3 ey - 69), Y^3 < 2^72 kept as its top 64 bits (Y^3 / 2^8)
    const u64 Y3 = (wide(Y2h, Y) << 24) + (wide(Y2l, Y) >> 8);
    const u64 F = mulhi64(Y3, M1);                                   // y0^3 (1 + c) = F 2^(3 ey - 59)

    // 5. (r^2)^(-3/2) = F 2^(3 ey - 59 - 3k), rounded to double
    const int lzf = clz64(F);
    const u64 n = F << lzf;
    const u64 r = n + 0x3FFull + ((n >> 11) & 1ull);
    const int carry = r < n;
    const u64 frac = carry ? 0ull : ((r >> 11) & 0xFFFFFFFFFFFFFull);
    const int be = 1023 + 4 - lzf + 3 * ey - 3 * k + carry;
    if (be <= 0) return 0.0;
    if (be >= 2047) return bits_double(0x7FF0000000000000ull);
    return bits_double(((u64)be << 52) | frac);
}

}  // namespace fixpair
