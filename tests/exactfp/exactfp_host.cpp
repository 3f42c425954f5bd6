// Bit-for-bit check of the integer-pipe IEEE routines (rebound_gb300/csrc/exactfp.cuh)
// against the host's own IEEE double arithmetic (TEST INFRASTRUCTURE ONLY).
//
// Usage: exactfp_host <cases per class> <seed>
// Prints one line per routine: "<name> <cases> <mismatches>", then the first
// mismatches found (operands and both results as bit patterns).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "exactfp.cuh"

using exactfp::u64;

static u64 g_state;
static u64 next() {                                   // splitmix64
    u64 z = (g_state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double from_bits(u64 b) { double d; memcpy(&d, &b, 8); return d; }
static u64 to_bits(double d) { u64 b; memcpy(&b, &d, 8); return b; }

// A double with biased exponent e (clamped to [0, 2047]), a random or sparse
// significand and a random sign.
static double make(int e, int sparse) {
    if (e < 0) e = 0;
    if (e > 2047) e = 2047;
    u64 frac = next() & exactfp::kFrac;
    if (sparse == 1) frac &= ~((1ull << (next() % 53)) - 1);          // trailing zeros: exact / tie cases
    if (sparse == 2) frac = (next() & 1) ? frac | 0xFFFFFFF : frac & ~0xFFFFFFFull;
    return from_bits(((next() & 1) << 63) | ((u64)e << 52) | frac);
}

// Operand pairs by class: 0 wide random exponents, 1 close exponents
// (cancellation), 2 sparse significands, 3 exponent gaps around 53-64,
// 4 range ends (zeros, subnormals, huge, inf/nan), 5 the tree walk's ranges.
static void pair(int cls, double& a, double& b) {
    const int ea = 1 + (int)(next() % 2046);
    switch (cls) {
        case 0: a = make(ea, 0); b = make(1 + (int)(next() % 2046), 0); break;
        case 1: a = make(ea, (int)(next() % 3)); b = make(ea - (int)(next() % 3), (int)(next() % 3)); break;
        case 2: a = make(ea, 1); b = make(ea - (int)(next() % 80), 1); break;
        case 3: a = make(ea, (int)(next() % 3)); b = make(ea - 50 - (int)(next() % 20), (int)(next() % 3)); break;
        case 4: {
            const int pick[8] = {0, 1, 2, 2045, 2046, 2047, 1023, 3};
            a = make(pick[next() % 8] + (int)(next() % 3) - 1, (int)(next() % 3));
            b = make(pick[next() % 8] + (int)(next() % 3) - 1, (int)(next() % 3));
            if (next() % 8 == 0) b = (next() & 1) ? -a : a;
            if (next() % 8 == 0) b = 0.0 * ((next() & 1) ? -1 : 1);
            break;
        }
        default: a = make(1023 + (int)(next() % 24) - 12, 0); b = make(1023 + (int)(next() % 24) - 12, 0); break;
    }
    if (next() % 64 == 0) b = a;
}

static int report(const char* name, long n, long bad) {
    printf("%s %ld %ld\n", name, n, bad);
    return bad != 0;
}

static bool same(double x, double y) { return (std::isnan(x) && std::isnan(y)) || to_bits(x) == to_bits(y); }

int main(int argc, char** argv) {
    const long n = argc > 1 ? atol(argv[1]) : 1000000;
    g_state = argc > 2 ? strtoull(argv[2], nullptr, 10) : 1;
    long bad_pos = 0, bad_mul = 0, bad_sqr = 0, bad_div = 0, bad_sqrt = 0, bad_cmp = 0;
    int shown = 0;
    for (int cls = 0; cls < 6; cls++) {
        for (long k = 0; k < n; k++) {
            double a, b;
            pair(cls, a, b);
            const double rm = exactfp::mul_rn(a, b);
            const double rq = exactfp::sqr_rn(a);
            const double pa = fabs(a), pb = fabs(b);
            const double rp = exactfp::add_pos_rn(pa, pb);
            if (!same(rm, a * b)) bad_mul++;
            if (!same(rq, a * a)) bad_sqr++;
            if (!same(rp, pa + pb)) bad_pos++;
            if (!same(exactfp::div_rn(a, b), a / b)) bad_div++;
            if (!same(exactfp::sqrt_rn(pa), sqrt(pa))) bad_sqrt++;
            const int kpow = -(int)(next() % 6);
            const int c = exactfp::gt_scaled_pow2(pa, pb, kpow);
            if (c >= 0 && !std::isnan(pa) && (c == 1) != (pa > ldexp(1.0, kpow) * pb)) bad_cmp++;   // w2 is never NaN
            if (shown < 8 && (!same(rm, a * b) || !same(rq, a * a) || !same(rp, pa + pb))) {
                printf("MISMATCH class %d a %016llx b %016llx "
                       "mul %016llx/%016llx sqr %016llx/%016llx pos %016llx/%016llx\n",
                       cls, (unsigned long long)to_bits(a), (unsigned long long)to_bits(b),
                       (unsigned long long)to_bits(rm), (unsigned long long)to_bits(a * b),
                       (unsigned long long)to_bits(rq), (unsigned long long)to_bits(a * a),
                       (unsigned long long)to_bits(rp), (unsigned long long)to_bits(pa + pb));
                shown++;
            }
        }
    }
    const long tot = 6 * n;
    int fail = 0;
    fail |= report("add_pos_rn", tot, bad_pos);
    fail |= report("mul_rn", tot, bad_mul);
    fail |= report("sqr_rn", tot, bad_sqr);
    fail |= report("div_rn", tot, bad_div);
    fail |= report("sqrt_rn", tot, bad_sqrt);
    fail |= report("gt_scaled_pow2", tot, bad_cmp);
    return fail;
}
