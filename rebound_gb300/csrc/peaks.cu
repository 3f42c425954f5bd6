// Instruction-class throughput probes on the current GPU: the FP64 and FP32
// pipe peaks that bound the direct-sum kernels (the measured peaks file
// holds only HBM and BF16-tensor figures).  Each thread runs independent
// dependency chains so the pipe, not latency, limits the rate.
#include "rgpu_internal.cuh"
#include "exactfp.cuh"

namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;

__global__ void probe_dfma(double* out, double a, double b) {
    double acc[kChains];
    for (int c = 0; c < kChains; c++) acc[c] = threadIdx.x * 1e-3 + c;
    for (int it = 0; it < kIters; it++)
#pragma unroll
        for (int c = 0; c < kChains; c++) acc[c] = fma(acc[c], a, b);
    double s = 0.;
    for (int c = 0; c < kChains; c++) s += acc[c];
    if (s == 1234.5678) out[0] = s;
}

__global__ void probe_ffma(float* out, float a, float b) {
    float acc[kChains];
    for (int c = 0; c < kChains; c++) acc[c] = threadIdx.x * 1e-3f + c;
    for (int it = 0; it < kIters; it++)
#pragma unroll
        for (int c = 0; c < kChains; c++) acc[c] = fmaf(acc[c], a, b);
    float s = 0.f;
    for (int c = 0; c < kChains; c++) s += acc[c];
    if (s == 1234.5678f) out[0] = s;
}

// Round trips double -> float -> double: two conversions per chain step.
__global__ void probe_cvt(double* out, double a) {
    double acc[kChains];
    for (int c = 0; c < kChains; c++) acc[c] = threadIdx.x * 1e-3 + c + a;
    for (int it = 0; it < kIters / 2; it++)
#pragma unroll
        for (int c = 0; c < kChains; c++) {
            float f = (float)acc[c];
            f = __int_as_float(__float_as_int(f) ^ 1);   // keep the chain live without FP work
            acc[c] = (double)f;
        }
    double s = 0.;
    for (int c = 0; c < kChains; c++) s += acc[c];
    if (s == 1234.5678) out[0] = s;
}

__global__ void probe_rsqrt(float* out, float a) {
    float acc[kChains];
    for (int c = 0; c < kChains; c++) acc[c] = 1.0f + threadIdx.x * 1e-3f + c + a;
    for (int it = 0; it < kIters; it++)
#pragma unroll
        for (int c = 0; c < kChains; c++) acc[c] = rsqrtf(acc[c]);
    float s = 0.f;
    for (int c = 0; c < kChains; c++) s += acc[c];
    if (s == 1234.5678f) out[0] = s;
}

// Integer ALU pipe: dependent 3-input logic ops (one LOP3 each, written as
// inline PTX so the compiler can neither fold nor move them to another pipe).
__device__ __forceinline__ unsigned lop3_xor(unsigned a, unsigned b, unsigned c) {
    unsigned d;
    asm volatile("lop3.b32 %0, %1, %2, %3, 0x96;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}

__global__ void probe_alu(unsigned* out, unsigned m) {
    unsigned u[kChains], v[kChains];
    for (int c = 0; c < kChains; c++) { u[c] = threadIdx.x * 7u + c; v[c] = c * 31u + m; }
    for (int it = 0; it < kIters / 2; it++)
#pragma unroll
        for (int c = 0; c < kChains; c++) {
            u[c] = lop3_xor(u[c], v[c], m);
            v[c] = lop3_xor(v[c], u[c], it);
        }
    unsigned t = 0;
    for (int c = 0; c < kChains; c++) t += u[c] + v[c];
    if (t == 12345u) out[0] = t;
}

// Throughput of one FP64 routine: each thread applies it to a stream of
// independent operands (consecutive bit patterns near 1.0), so the pipes that
// carry the routine, not latency, set the rate.  OP: 5 integer-pipe division,
// 6 integer-pipe square root, 7 integer-pipe square, 8 integer-pipe product,
// 9 integer-pipe non-negative sum, 10 hardware division, 11 hardware square
// root, 12 hardware addition.
template <int OP>
__global__ void probe_routine(unsigned long long* out, unsigned long long base, double c) {
    unsigned long long acc = 0;
    exactfp::u32 special = 0;
    const unsigned long long b0 = base + threadIdx.x * 977ull + blockIdx.x * 131ull;
#pragma unroll 4
    for (int it = 0; it < kIters; it++) {
        const double x = __longlong_as_double((long long)(b0 + (unsigned long long)it * 0x10001ull));
        double r;
        if (OP == 5) r = exactfp::div_rn(c, x);
        if (OP == 6) r = exactfp::sqrt_rn(x);
        if (OP == 7) r = exactfp::sqr_try(x, special);
        if (OP == 8) r = exactfp::mul_try(x, c, special);
        if (OP == 9) r = exactfp::add_pos_try(x, c, special);
        if (OP == 10) r = c / x;
        if (OP == 11) r = sqrt(x);
        if (OP == 12) r = x + c;
        acc ^= (unsigned long long)__double_as_longlong(r);
    }
    if (acc == 0x123456789ull || special == 77u) out[0] = acc + special;
}

// Self-check of the integer-pipe IEEE division and square root against the
// hardware operations on pseudo-random normal operands (splitmix64 stream).
__device__ __forceinline__ unsigned long long splitmix(unsigned long long& s) {
    unsigned long long z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ double random_double(unsigned long long& s, int emin, int span) {
    const unsigned long long r = splitmix(s), f = splitmix(s);
    const int e = emin + (int)(r % (unsigned)span);
    unsigned long long frac = f & 0xFFFFFFFFFFFFFull;
    const int pat = (int)((r >> 32) & 7);
    if (pat == 0) frac = 0;
    if (pat == 1) frac = 0xFFFFFFFFFFFFFull;
    if (pat == 2) frac &= 0xFFFFull;
    if (pat == 3) frac = 0xFFFFFFFFFFFFFull - (frac & 0xFFFFull);
    const unsigned long long sign = (r >> 40) & 1ull;
    return __longlong_as_double((long long)((sign << 63) | ((unsigned long long)(e + 1023) << 52) | frac));
}

__global__ void exactfp_check(long long n, unsigned long long seed, unsigned long long* bad) {
    unsigned long long local = 0;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        unsigned long long s = seed ^ (0x632BE59BD9B4E019ull * (unsigned long long)(k + 1));
        const double a = random_double(s, -300, 601), b = random_double(s, -300, 601);
        const double x = fabs(random_double(s, -1000, 2001));
        if (__double_as_longlong(exactfp::div_rn(a, b)) != __double_as_longlong(a / b)) local++;
        if (__double_as_longlong(exactfp::sqrt_rn(x)) != __double_as_longlong(sqrt(x))) local++;
        // non-negative sums (wide and close exponents), products and squares
        const double c = __longlong_as_double(__double_as_longlong(a) ^ (long long)(splitmix(s) & 0x3FFFFFull));
        const double ya = fabs(a), yb = fabs(b), yc = fabs(c);
        if (__double_as_longlong(exactfp::add_pos_rn(ya, yb)) != __double_as_longlong(ya + yb)) local++;
        if (__double_as_longlong(exactfp::add_pos_rn(ya, yc)) != __double_as_longlong(ya + yc)) local++;
        if (__double_as_longlong(exactfp::mul_rn(a, b)) != __double_as_longlong(a * b)) local++;
        if (__double_as_longlong(exactfp::sqr_rn(c)) != __double_as_longlong(c * c)) local++;
    }
    if (local) atomicAdd(bad, local);
}

}  // namespace

extern "C" int rgpu_selftest_exactfp(long long n, unsigned long long seed, long long* mismatches) {
    if (!mismatches || n < 0) return RGPU_ERR_ARG;
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, sizeof(unsigned long long)) != cudaSuccess) return RGPU_ERR_NOMEM;
    cudaMemset(d, 0, sizeof(unsigned long long));
    int dev = 0, nsm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    exactfp_check<<<nsm * 8, 256>>>(n, seed, d);
    g_launches++;
    unsigned long long h = 0;
    cudaError_t err = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (err != cudaSuccess) return RGPU_ERR_CUDA;
    *mismatches = (long long)h;
    return RGPU_OK;
}

extern "C" int rgpu_probe_rate(int which, double* ops_per_s) {
    if (!ops_per_s || which < 0 || which > 12) return RGPU_ERR_ARG;
    int dev = 0, nsm = 1;
    if (cudaGetDevice(&dev) != cudaSuccess) return RGPU_ERR_CUDA;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    void* buf = nullptr;
    if (cudaMalloc(&buf, 64) != cudaSuccess) return RGPU_ERR_NOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int threads = 256, blocks = nsm * 8;
    double ops = (double)threads * blocks * (which >= 5 ? 1 : kChains) * kIters;
    const unsigned long long one = 0x3FF0000000000000ull;
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        cudaEventRecord(e0);
        switch (which) {
            case 0: probe_dfma<<<blocks, threads>>>((double*)buf, 0.999999, 1e-7); break;
            case 1: probe_ffma<<<blocks, threads>>>((float*)buf, 0.999999f, 1e-7f); break;
            case 2: probe_cvt<<<blocks, threads>>>((double*)buf, 0.5); break;
            case 4: probe_alu<<<blocks, threads>>>((unsigned*)buf, 3u); break;
            case 5: probe_routine<5><<<blocks, threads>>>((unsigned long long*)buf, one, 1.0000001); break;
            case 6: probe_routine<6><<<blocks, threads>>>((unsigned long long*)buf, one, 1.0000001); break;
            case 7: probe_routine<7><<<blocks, threads>>>((unsigned long long*)buf, one, 1.0000001); break;
            case 8: probe_routine<8><<<blocks, threads>>>((unsigned long long*)buf, one, 1.0000001); break;
            case 9: probe_routine<9><<<blocks, threads>>>((unsigned long long*)buf, one, 1.0000001); break;
            case 10: probe_routine<10><<<blocks, threads>>>((unsigned long long*)buf, one, 1.0000001); break;
            case 11: probe_routine<11><<<blocks, threads>>>((unsigned long long*)buf, one, 1.0000001); break;
            case 12: probe_routine<12><<<blocks, threads>>>((unsigned long long*)buf, one, 1.0000001); break;
            default: probe_rsqrt<<<blocks, threads>>>((float*)buf, 0.5f); break;
        }
        g_launches++;
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    if (err != cudaSuccess) return RGPU_ERR_CUDA;
    *ops_per_s = ops / (best * 1e-3);
    return RGPU_OK;
}
