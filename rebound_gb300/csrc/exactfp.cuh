// Correctly rounded FP64 division and square root on the integer pipes.
//
// GB300 issues FP64 at ~1/70 of its FP32 rate; an IEEE division or square root
// there is a sequence of about ten FP64-pipe instructions.  The kernels that must
// reproduce the reference bit for bit (the exact tree walk) spend half their FP64
// issue on these two operations, so they are rebuilt here from integer arithmetic,
// giving the IEEE round-to-nearest-even result exactly:
//
//   1. an FP32 seed (MUFU rcp / rsqrt) of the leading 24 bits of the operand;
//   2. Newton–Raphson refinement in 2^-62 fixed point, folded into one binomial
//      series step (1/(1-e) = 1 + e + e^2, (1-h)^(-1/2) = 1 + h/2 + 3h^2/8), which
//      brings the quotient / root to within a few units of its 54-bit truncation;
//   3. the exact remainder (a 2^K - Q b, or N - Q^2, formed modulo 2^64 because
//      it is known to be small) corrects Q to the exact floor (Markstein's final
//      correction step, done in integers);
//   4. rounding: the 54th bit decides, since neither a quotient nor a square root
//      of FP64 operands can fall exactly halfway between two doubles.
//
// Operands or results outside the normal range take the hardware operation (a
// rare branch).  Both routines compile for the host as well; there they are
// compared bit for bit with the host's IEEE division and square root.
#pragma once
#include "fixpair.cuh"

namespace exactfp {

using fixpair::u32;
using fixpair::u64;

FIX_HD u64 dbits(double d) {
#ifdef __CUDA_ARCH__
    return (u64)__double_as_longlong(d);
#else
    u64 b;
    memcpy(&b, &d, 8);
    return b;
#endif
}

#ifndef EXACTFP_HOST_RCP
#define EXACTFP_HOST_RCP(x) (1.0f / (x))
#endif
// Approximate reciprocal (MUFU); the refinement below tolerates a seed error
// well beyond its 2^-23 bound.
FIX_HD float seed_rcp(float x) {
#ifdef __CUDA_ARCH__
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
#else
    return EXACTFP_HOST_RCP(x);
#endif
}

constexpr u64 kFrac = 0xFFFFFFFFFFFFFull;
constexpr u64 kHidden = 1ull << 52;

// a / b rounded to nearest even; `special` is set (and the value is meaningless)
// for a zero, subnormal, infinite or NaN operand or a quotient near the ends of
// the range.  No branch: every input runs the same instructions.
FIX_HD double div_try(double a, double b, u32& special) {
    const u64 ab = dbits(a), bb = dbits(b);
    const int ea = (int)((ab >> 52) & 0x7FF), eb = (int)((bb >> 52) & 0x7FF);
    const int be = ea - eb + 1023;                                  // biased exponent if ma >= mb
    special |= ((unsigned)(ea - 1) >= 2046u || (unsigned)(eb - 1) >= 2046u || (unsigned)(be - 2) >= 2043u) ? 1u : 0u;
    const u64 ma = (ab & kFrac) | kHidden, mb = (bb & kFrac) | kHidden;
    const int lt = ma < mb ? 1 : 0;
    // 1. seed y0 ~ 1/B, B = mb / 2^52 in [1, 2); y0 = Y 2^(ey - 23)
    const u32 xb = 0x3F800000u | (u32)((mb >> 29) & 0x7FFFFFu);
    const u32 yb = fixpair::float_bits(seed_rcp(fixpair::bits_float(xb)));
    const int ey = (int)(yb >> 23) - 127;
    const u32 Y = (yb & 0x7FFFFFu) | 0x800000u;
    // 2. e = 1 - B y0 as E = e 2^62:  B y0 = mb Y 2^(ey - 75)
    const u32 mbh = (u32)(mb >> 32), mbl = (u32)mb;
    const u64 pl = fixpair::wide(mbl, Y);                            // mb Y = (mbh Y) 2^32 + pl, < 2^77
    const u64 top = fixpair::wide(mbh, Y) + (pl >> 32);              // (mb Y) >> 32, < 2^46
    const int sh = 13 - ey;                                          // (mb Y) >> sh ~ 2^62
    const u64 bys = (top << (32 - sh)) | ((u32)pl >> sh);
    const long long E = (long long)((1ull << 62) - bys);             // |e| < 2^-20
    //    1/B = y0 (1 + e + e^2 + O(e^3)) = Y M1 2^(ey - 85), M1 = (1 + e + e^2) 2^62
    const int Es = (int)(E >> 20);
    const long long Q2 = ((long long)Es * Es) >> 22;                 // e^2 2^62
    const u64 M1 = (1ull << 62) + (u64)(E + Q2);
    const u64 R = fixpair::mad_wide(Y, (u32)(M1 >> 32), (u64)fixpair::mulhi32(Y, (u32)M1)) << 9;   // ~ Y M1 / 2^23
    // 3. Q = floor(ma 2^K / mb), K = 53 + lt, Q in [2^53, 2^54):
    //    ma 2^K / mb = ma 2^(K - 52) / B = ma R 2^(K + ey - 114) = (ma 2^11 R / 2^64) 2^(lt + ey - 8)
    const u64 hi = fixpair::mulhi64(ma << 11, R);
    u64 Q = hi >> (8 - lt - ey);
    //    exact remainder modulo 2^64 (its true value is small) and correction.
    //    Error of Q against floor(ma 2^K / mb) = floor(T), T < 2^54: R is low by
    //    less than 2^-53 relative (the 9 bits cleared by << 9 of a value >= 2^62),
    //    which costs less than 2.0000005 units; the series and E / Q2 roundings
    //    move Q by less than 2^-61 relative (0.007 units) either way.  So Q is in
    //    [floor(T) - 3, floor(T) + 1]: one downward step, up to three upward.
    const u64 num_lo = ma << (53 + lt);                              // low 64 bits of ma 2^K
    long long rem = (long long)(num_lo - Q * mb);
    if (rem < 0) { Q -= 1; rem += (long long)mb; }
    for (int k = 0; k < 3 && rem >= (long long)mb; k++) { Q += 1; rem -= (long long)mb; }
    // 4. round (no ties) and assemble; the hidden bit of Q >> 1 adds the last exponent unit
    const u64 mant = (Q >> 1) + (Q & 1);
    const u64 bits = ((u64)(be - lt - 1) << 52) + mant;
    return fixpair::bits_double(bits | ((ab ^ bb) & 0x8000000000000000ull));
}

// The hardware operations for the special cases, out of line on the device: a
// call is never evaluated speculatively, whereas an inline `sp ? a / b : q`
// would have the compiler issue the whole FP64 division sequence every time.
#ifdef __CUDA_ARCH__
static __device__ __noinline__ double hw_div(double a, double b) { return a / b; }
static __device__ __noinline__ double hw_sqrt(double x) { return sqrt(x); }
static __device__ __noinline__ double hw_mul(double a, double b) { return a * b; }
static __device__ __noinline__ double hw_add(double a, double b) { return a + b; }
#else
inline double hw_div(double a, double b) { return a / b; }
inline double hw_sqrt(double x) { return __builtin_sqrt(x); }
inline double hw_mul(double a, double b) { return a * b; }
inline double hw_add(double a, double b) { return a + b; }
#endif

// a / b rounded to nearest even (the hardware division for the special cases).
FIX_HD double div_rn(double a, double b) {
    u32 sp = 0;
    const double q = div_try(a, b, sp);
    return sp ? hw_div(a, b) : q;
}

// sqrt(x) rounded to nearest even; `special` is set for x not a positive normal
// number.  No branch.
FIX_HD double sqrt_try(double x, u32& special) {
    const u64 xb_ = dbits(x);
    const int ex = (int)(xb_ >> 52);                                 // sign bit included: negatives are special
    special |= (unsigned)(ex - 1) >= 2046u ? 1u : 0u;
    const u64 mx = (xb_ & kFrac) | kHidden;
    const int t = ex - 1075;                                         // x = mx 2^t
    const int odd = t & 1;
    const u64 m2 = mx << odd;                                        // x = m2 2^(t - odd), m2 in [2^52, 2^54)
    // 1. seed y0 ~ 1/sqrt(X), X = m2 / 2^52 in [1, 4); y0 = Y 2^(ey - 23)
    const u32 fb = ((u32)(127 + odd) << 23) | (u32)((mx >> 29) & 0x7FFFFFu);
    const u32 yb = fixpair::float_bits(fixpair::seed_rsqrt(fixpair::bits_float(fb)));
    const int ey = (int)(yb >> 23) - 127;
    const u32 Y = (yb & 0x7FFFFFu) | 0x800000u;
    // 2. h = 1 - X y0^2 as H = h 2^62:  X y0^2 = m2 Y^2 2^(2 ey - 98)
    const u64 Y2 = fixpair::wide(Y, Y);                              // < 2^48
    const u32 Y2h = (u32)(Y2 >> 32), Y2l = (u32)Y2;
    const u32 mh = (u32)(m2 >> 32), ml = (u32)m2;                    // mh < 2^22
    //    P = (m2 Y^2) >> 32 = mh Y2h 2^32 + mh Y2l + ml Y2h + hi32(ml Y2l)   (< 2^70)
    const u64 acc = fixpair::mad_wide(ml, Y2h, fixpair::mad_wide(mh, Y2l, (u64)fixpair::mulhi32(ml, Y2l)));   // < 2^55
    const u64 C = fixpair::wide(mh, Y2h);                            // < 2^38, weight 2^32
    const u64 mid = (acc >> 32) + (u32)C;
    const u32 p0 = (u32)acc, p1 = (u32)mid, p2 = (u32)(C >> 32) + (u32)(mid >> 32);
    const int sh = 4 - 2 * ey;                                       // H = 2^62 - (P >> sh), sh in [4, 8]
    const u32 s_lo = fixpair::shf_r(p0, p1, sh), s_hi = fixpair::shf_r(p1, p2, sh);
    const long long H = (long long)((1ull << 62) - (((u64)s_hi << 32) | s_lo));
    //    (1 - h)^(-1/2) = 1 + h/2 + 3 h^2 / 8: M1 = 2^62 + (4 H + 3 Q2) / 8
    const int Hs = (int)(H >> 20);
    const u32 Q2 = (u32)((u64)((long long)Hs * Hs) >> 22);
    const u64 M1 = (1ull << 62) + (u64)((long long)fixpair::mad_wide(Q2, 3u, (u64)(H * 4)) >> 3);
    // 3. sqrt(N), N = m2 2^54:  sqrt(N) = X y0 (1 + c) 2^53 = m2 Y M1 2^(ey - 84)
    const u64 YM = fixpair::mad_wide(Y, (u32)(M1 >> 32), (u64)fixpair::mulhi32(Y, (u32)M1)) << 9;   // ~ Y M1 / 2^23
    const u64 hi = fixpair::mulhi64(m2 << 10, YM);                   // m2 YM 2^10 / 2^64
    u64 Q = hi >> (7 - ey);                                          // sqrt(N) = m2 YM 2^(ey - 61)
    //    exact remainder N - Q^2 modulo 2^64, then floor correction: 0 <= N - Q^2 <= 2Q
    const u64 n_lo = m2 << 54;
    long long rem = (long long)(n_lo - Q * Q);
    for (int k = 0; k < 3 && rem < 0; k++) { rem += (long long)(2 * Q - 1); Q -= 1; }
    for (int k = 0; k < 3 && rem > (long long)(2 * Q); k++) { Q += 1; rem -= (long long)(2 * Q - 1); }
    // 4. round (no ties) and assemble: sqrt(x) = sqrt(N) 2^((t - odd - 54) / 2), Q in [2^53, 2^54)
    const u64 mant = (Q >> 1) + (Q & 1);
    const int be = 1049 + ((t - odd) >> 1);                          // 1023 + 53 + (t - odd - 54) / 2
    return fixpair::bits_double(((u64)(be - 1) << 52) + mant);
}

// sqrt(x) rounded to nearest even (the hardware square root for the special cases).
FIX_HD double sqrt_rn(double x) {
    u32 sp = 0;
    const double r = sqrt_try(x, sp);
    return sp ? hw_sqrt(x) : r;
}

// ---------------------------------------------------------------------------
// Squares, products and sums of non-negative numbers.  Each FP64 instruction on
// GB300 holds the FP64 pipe for 64 clocks per warp (0.5 lanes per clock per SM
// sub-partition), while the ALU and IMAD pipes issue a warp instruction every
// clock or two; the same IEEE round-to-nearest-even results built from 30-45
// 32-bit integer instructions leave the FP64 pipe free for the rest of the
// work.  (A general signed addition needs about twice as many instructions and
// stays on the FP64 pipe.)
//
// The *_try forms return the exact result when the operands and the result are
// normal numbers and otherwise set `special` (the value is then meaningless):
// the caller recomputes such rare cases with hardware FP64 in a branch of its
// own, so that no FP64 instruction is issued on the common path.
//
// Rounding: a significand s with its leading bit at bit 62 keeps bits 62..10;
// bits 9..0 decide, with every bit shifted out below bit 0 jammed into bit 0
// (sticky).  Jamming keeps floor(s / 2) and whether anything is left below,
// which is all a rounding position two or more bits up reads.

// s = sh:sl (leading bit at 62, sticky in bit 0) rounded to 53 bits, ties to
// even, added to the biased exponent minus one (be1) in the high word: a
// round-up to 2^53 carries into the exponent.  Returns the double's bits.
FIX_HD u64 round_assemble(u32 sh, u32 sl, u32 be1) {
    const u32 add = 0x1FFu + ((sl >> 10) & 1u);
    const u32 lo = sl + add;
    const u32 hi = sh + (lo < sl ? 1u : 0u);
    const u32 mlo = fixpair::shf_r(lo, hi, 10), mhi = hi >> 10;
    return ((u64)((be1 << 20) + mhi) << 32) | mlo;
}

// P = p3:p2:p1:p0 in [2^104, 2^106) (a product of two 53-bit significands) to the
// rounded double; e: the biased exponent of the product if P < 2^105.
FIX_HD double finish_product(u32 p0, u32 p1, u32 p2, u32 p3, int e, u32 sign, u32& special) {
    const u32 top = p3 >> 9;                                         // P >= 2^105
    const int sh = 10 + (int)top;                                    // s = P >> (32 + sh)
    const u32 sl = fixpair::shf_r(p1, p2, sh), shi = fixpair::shf_r(p2, p3, sh);
    const u32 sticky = (p0 | (p1 & ((1u << sh) - 1u))) != 0u ? 1u : 0u;
    e += (int)top;
    special |= (unsigned)(e - 1) >= 2045u ? 1u : 0u;                 // subnormal or overflowing result
    return fixpair::bits_double(round_assemble(shi, sl | sticky, (u32)(e - 1)) | ((u64)sign << 32));
}

// a * a.
FIX_HD double sqr_try(double a, u32& special) {
    const u64 A = dbits(a);
    const u32 ah = (u32)(A >> 32), al = (u32)A;
    const int ea = (int)((ah >> 20) & 0x7FFu);
    special |= (unsigned)(ea - 1) >= 2046u ? 1u : 0u;                // zero, subnormal, inf, NaN
    const u32 h = (ah & 0xFFFFFu) | 0x100000u;                       // significand = h 2^32 + al, h < 2^21
    // P = h^2 2^64 + 2 h al 2^32 + al^2
    const u64 ll = fixpair::wide(al, al);
    const u64 t = fixpair::mad_wide(h << 1, al, ll >> 32);           // < 2^55
    const u64 u = fixpair::mad_wide(h, h, t >> 32);                  // < 2^43
    return finish_product((u32)ll, (u32)t, (u32)u, (u32)(u >> 32), 2 * ea - 1023, 0u, special);
}

// a * b.
FIX_HD double mul_try(double a, double b, u32& special) {
    const u64 A = dbits(a), B = dbits(b);
    const u32 ah = (u32)(A >> 32), al = (u32)A, bh = (u32)(B >> 32), bl = (u32)B;
    const int ea = (int)((ah >> 20) & 0x7FFu), eb = (int)((bh >> 20) & 0x7FFu);
    special |= ((unsigned)(ea - 1) >= 2046u || (unsigned)(eb - 1) >= 2046u) ? 1u : 0u;
    const u32 ha = (ah & 0xFFFFFu) | 0x100000u, hb = (bh & 0xFFFFFu) | 0x100000u;
    // P = ha hb 2^64 + (ha bl + al hb) 2^32 + al bl
    const u64 ll = fixpair::wide(al, bl);
    const u64 t1 = fixpair::mad_wide(ha, bl, ll >> 32);              // < 2^54
    const u64 t2 = fixpair::mad_wide(al, hb, (u32)t1);               // < 2^54
    const u64 u = fixpair::mad_wide(ha, hb, t1 >> 32) + (t2 >> 32);  // < 2^43
    return finish_product((u32)ll, (u32)t2, (u32)u, (u32)(u >> 32), ea + eb - 1023, (ah ^ bh) & 0x80000000u,
                          special);
}

// a + b for a, b >= +0 (no cancellation, no sign).
FIX_HD double add_pos_try(double a, double b, u32& special) {
    const u64 A = dbits(a), B = dbits(b);
    const bool sw = B > A;
    const u64 X = sw ? B : A, Y = sw ? A : B;
    const u32 xh = (u32)(X >> 32), yh = (u32)(Y >> 32);
    const int ex = (int)(xh >> 20), ey = (int)(yh >> 20);            // sign bits included: negatives are special
    special |= (ey == 0 || ex >= 2047) ? 1u : 0u;
    const u64 mx = ((X & kFrac) | kHidden) << 10;                    // leading bit at 62
    const u64 my = ((Y & kFrac) | kHidden) << 10;
    const int d = ex - ey < 63 ? ex - ey : 63;
    const u64 t = my >> d;
    const u64 s0 = mx + (t | ((t << d) != my ? 1ull : 0ull));        // sticky; < 2^64
    const u32 c = (u32)(s0 >> 63);                                   // renormalise by one bit, keeping the sticky
    const u32 sl = fixpair::shf_r((u32)s0, (u32)(s0 >> 32), (int)c) | ((u32)s0 & c);
    const u32 shi = (u32)(s0 >> 32) >> c;
    const int e = ex + (int)c;
    special |= e >= 2046 ? 1u : 0u;
    return fixpair::bits_double(round_assemble(shi, sl, (u32)(e - 1)));
}

// The same with the hardware operation for the special cases.
FIX_HD double sqr_rn(double a) {
    u32 sp = 0;
    const double r = sqr_try(a, sp);
    return sp ? hw_mul(a, a) : r;
}
FIX_HD double mul_rn(double a, double b) {
    u32 sp = 0;
    const double r = mul_try(a, b, sp);
    return sp ? hw_mul(a, b) : r;
}
FIX_HD double add_pos_rn(double a, double b) {
    u32 sp = 0;
    const double r = add_pos_try(a, b, sp);
    return sp ? hw_add(a, b) : r;
}

// w2 > c * r2 for w2 >= +0 (not NaN) and c = 2^k: the product is r2 with k
// added to its exponent, exact while it stays normal, and non-negative doubles
// order as their bit patterns.  Returns -1 when r2 is not a positive normal
// number or the product leaves the normal range (the caller then compares in
// FP64).
FIX_HD int gt_scaled_pow2(double w2, double r2, int k) {
    const u64 R = dbits(r2);
    const int er = (int)(R >> 52);                                   // the sign bit included: negatives fail
    if ((unsigned)(er - 1) >= 2046u || (unsigned)(er + k - 1) >= 2046u) return -1;
    return dbits(w2) > R + ((u64)(long long)k << 52) ? 1 : 0;
}

}  // namespace exactfp
