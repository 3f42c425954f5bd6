// Batched WHFast kernels: one thread per planetary system, systems grouped by
// body count so every thread of a warp runs the same unrolled code.  State is
// structure-of-arrays [field][body][system] so a warp's loads and stores are
// coalesced across systems; each thread keeps its system in registers (spilling
// to L1-cached local memory for the largest systems) for a whole chunk of
// steps.  Included three times: ensemble.cu (FMA contraction, fast),
// ensemble_exact.cu (--fmad=false, bit-identical to the reference) and
// ensemble_dh.cu (democratic heliocentric coordinates, --fmad=false).
#pragma once
#include "whfast_core.cuh"

#ifndef ENSEMBLE_NS
#error "define ENSEMBLE_NS before including ensemble_kernels.cuh"
#endif
#ifndef ENSEMBLE_STEP
#define ENSEMBLE_STEP wh::step_safe     // Jacobi coordinates; ensemble_dh.cu: democratic heliocentric
#endif

namespace ENSEMBLE_NS {

// Advance system `sid` of one bucket by n_steps (state in, state out).
template <int NB>
__device__ __noinline__ void advance_system(double* __restrict__ st, const double* __restrict__ dt,
                                            double* __restrict__ t, int count, int sid, int n_steps, double G,
                                            uint32_t* status) {
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
    for (int k = 0; k < n_steps; k++) ENSEMBLE_STEP<NB>(s, G, 0.0, h, NB, NB, 0, status);
    t[sid] += h * n_steps;
#pragma unroll
    for (int i = 0; i < NB; i++) {
        const size_t o = (size_t)i * count + sid;
        st[0 * f + o] = s.x[i]; st[1 * f + o] = s.y[i]; st[2 * f + o] = s.z[i];
        st[3 * f + o] = s.vx[i]; st[4 * f + o] = s.vy[i]; st[5 * f + o] = s.vz[i];
    }
}

// One work unit: 32 consecutive systems of one bucket.
struct Unit {
    double* st;
    const double* dt;
    double* t;
    int count, nb, first, pad;
};

// Persistent scheduler: each warp takes the next unit from a global counter.
// Units are ordered by decreasing body count (longest first), so the last
// units handed out are the cheapest and the SMs finish together.
__global__ void __launch_bounds__(128) persistent_kernel(const Unit* __restrict__ units, int n_units, int n_steps,
                                                         double G, unsigned int* counter, uint32_t* status) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned int u = 0;
        if (lane == 0) u = atomicAdd(counter, 1u);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= (unsigned)n_units) return;
        const Unit U = units[u];
        const int sid = U.first + lane;
        if (sid >= U.count) continue;
        switch (U.nb) {
            case 2: advance_system<2>(U.st, U.dt, U.t, U.count, sid, n_steps, G, status); break;
            case 3: advance_system<3>(U.st, U.dt, U.t, U.count, sid, n_steps, G, status); break;
            case 4: advance_system<4>(U.st, U.dt, U.t, U.count, sid, n_steps, G, status); break;
            case 5: advance_system<5>(U.st, U.dt, U.t, U.count, sid, n_steps, G, status); break;
            case 6: advance_system<6>(U.st, U.dt, U.t, U.count, sid, n_steps, G, status); break;
            case 7: advance_system<7>(U.st, U.dt, U.t, U.count, sid, n_steps, G, status); break;
            case 8: advance_system<8>(U.st, U.dt, U.t, U.count, sid, n_steps, G, status); break;
            case 9: advance_system<9>(U.st, U.dt, U.t, U.count, sid, n_steps, G, status); break;
            case 10: advance_system<10>(U.st, U.dt, U.t, U.count, sid, n_steps, G, status); break;
            case 11: advance_system<11>(U.st, U.dt, U.t, U.count, sid, n_steps, G, status); break;
            case 12: advance_system<12>(U.st, U.dt, U.t, U.count, sid, n_steps, G, status); break;
            case 13: advance_system<13>(U.st, U.dt, U.t, U.count, sid, n_steps, G, status); break;
            case 14: advance_system<14>(U.st, U.dt, U.t, U.count, sid, n_steps, G, status); break;
            case 15: advance_system<15>(U.st, U.dt, U.t, U.count, sid, n_steps, G, status); break;
            default: advance_system<16>(U.st, U.dt, U.t, U.count, sid, n_steps, G, status); break;
        }
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

typedef void (*EnergyFn)(const double*, int, double, double*);

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
