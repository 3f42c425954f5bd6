// Batched WHFast kernels: one thread per planetary system, systems grouped by
// body count so every thread of a warp runs the same unrolled code.  State is
// structure-of-arrays [field][body][system] so a warp's loads and stores are
// coalesced across systems; each thread keeps its system in registers (spilling
// to L1-cached local memory for the largest systems) for a whole chunk of
// steps.  Included twice: ensemble.cu (FMA contraction, fast) and
// ensemble_exact.cu (--fmad=false, bit-identical to the reference).
#pragma once
#include "whfast_core.cuh"

#ifndef ENSEMBLE_NS
#error "define ENSEMBLE_NS before including ensemble_kernels.cuh"
#endif

namespace ENSEMBLE_NS {

template <int NB>
__global__ void __launch_bounds__(256) steps_kernel(double* __restrict__ st, const double* __restrict__ dt,
                                                    double* __restrict__ t, int count, int n_steps, double G,
                                                    uint32_t* status) {
    const int sid = blockIdx.x * blockDim.x + threadIdx.x;
    if (sid >= count) return;
    const size_t f = (size_t)NB * count;           // stride between fields
    wh::System<NB> s;
#pragma unroll
    for (int i = 0; i < NB; i++) {
        const size_t o = (size_t)i * count + sid;
        s.x[i] = st[0 * f + o]; s.y[i] = st[1 * f + o]; s.z[i] = st[2 * f + o];
        s.vx[i] = st[3 * f + o]; s.vy[i] = st[4 * f + o]; s.vz[i] = st[5 * f + o];
        s.m[i] = st[6 * f + o];
    }
    const double h = dt[sid];
    for (int k = 0; k < n_steps; k++) wh::step_safe<NB>(s, G, 0.0, h, NB, NB, 0, status);
    t[sid] += h * n_steps;
#pragma unroll
    for (int i = 0; i < NB; i++) {
        const size_t o = (size_t)i * count + sid;
        st[0 * f + o] = s.x[i]; st[1 * f + o] = s.y[i]; st[2 * f + o] = s.z[i];
        st[3 * f + o] = s.vx[i]; st[4 * f + o] = s.vy[i]; st[5 * f + o] = s.vz[i];
    }
}

template <int NB>
__global__ void energy_kernel(const double* __restrict__ st, int count, double G, double* __restrict__ out) {
    const int sid = blockIdx.x * blockDim.x + threadIdx.x;
    if (sid >= count) return;
    const size_t f = (size_t)NB * count;
    wh::System<NB> s;
#pragma unroll
    for (int i = 0; i < NB; i++) {
        const size_t o = (size_t)i * count + sid;
        s.x[i] = st[0 * f + o]; s.y[i] = st[1 * f + o]; s.z[i] = st[2 * f + o];
        s.vx[i] = st[3 * f + o]; s.vy[i] = st[4 * f + o]; s.vz[i] = st[5 * f + o];
        s.m[i] = st[6 * f + o];
    }
    out[sid] = wh::energy<NB>(s, G, NB, NB, 0);
}

typedef void (*StepsFn)(double*, const double*, double*, int, int, double, uint32_t*);
typedef void (*EnergyFn)(const double*, int, double, double*);

inline StepsFn steps_for(int nb) {
    switch (nb) {
        case 2: return steps_kernel<2>; case 3: return steps_kernel<3>; case 4: return steps_kernel<4>;
        case 5: return steps_kernel<5>; case 6: return steps_kernel<6>; case 7: return steps_kernel<7>;
        case 8: return steps_kernel<8>; case 9: return steps_kernel<9>; case 10: return steps_kernel<10>;
        case 11: return steps_kernel<11>; case 12: return steps_kernel<12>; case 13: return steps_kernel<13>;
        case 14: return steps_kernel<14>; case 15: return steps_kernel<15>; case 16: return steps_kernel<16>;
        default: return nullptr;
    }
}

inline EnergyFn energy_for(int nb) {
    switch (nb) {
        case 2: return energy_kernel<2>; case 3: return energy_kernel<3>; case 4: return energy_kernel<4>;
        case 5: return energy_kernel<5>; case 6: return energy_kernel<6>; case 7: return energy_kernel<7>;
        case 8: return energy_kernel<8>; case 9: return energy_kernel<9>; case 10: return energy_kernel<10>;
        case 11: return energy_kernel<11>; case 12: return energy_kernel<12>; case 13: return energy_kernel<13>;
        case 14: return energy_kernel<14>; case 15: return energy_kernel<15>; case 16: return energy_kernel<16>;
        default: return nullptr;
    }
}

}  // namespace ENSEMBLE_NS
