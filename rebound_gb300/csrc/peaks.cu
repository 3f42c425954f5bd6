// Instruction-class throughput probes on the current GPU: the FP64 and FP32
// pipe peaks that bound the direct-sum kernels (the measured peaks file
// holds only HBM and BF16-tensor figures).  Each thread runs independent
// dependency chains so the pipe, not latency, limits the rate.
#include "rgpu_internal.cuh"

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

}  // namespace

extern "C" int rgpu_probe_rate(int which, double* ops_per_s) {
    if (!ops_per_s || which < 0 || which > 4) return RGPU_ERR_ARG;
    int dev = 0, nsm = 1;
    if (cudaGetDevice(&dev) != cudaSuccess) return RGPU_ERR_CUDA;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    void* buf = nullptr;
    if (cudaMalloc(&buf, 64) != cudaSuccess) return RGPU_ERR_NOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int threads = 256, blocks = nsm * 8;
    double ops = (double)threads * blocks * kChains * kIters;
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        cudaEventRecord(e0);
        switch (which) {
            case 0: probe_dfma<<<blocks, threads>>>((double*)buf, 0.999999, 1e-7); break;
            case 1: probe_ffma<<<blocks, threads>>>((float*)buf, 0.999999f, 1e-7f); break;
            case 2: probe_cvt<<<blocks, threads>>>((double*)buf, 0.5); break;
            case 4: probe_alu<<<blocks, threads>>>((unsigned*)buf, 3u); break;
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
