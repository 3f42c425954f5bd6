// Pieces shared by the plain (one simulation per call) WHFast path: the
// handle's coordinate buffer, the operator program that whfast.cu builds and
// whfast_prog.cu runs, and the load / store helpers.
#pragma once
#include "whfast_core.cuh"

struct WhfastBuffers {
    double* jac = nullptr;   // 7 * cap: x, y, z, vx, vy, vz, m (Jacobi, p_jh)
    double* keep = nullptr;  // 7 * cap: p_jh saved across a keep_unsynchronized synchronize
    size_t cap = 0, keep_cap = 0;
};

namespace wh_plain {

// Operators of a WHFast program: one step or synchronize, laid out by the host
// in the reference's order.
enum : uint8_t {
    kOpFromInertial = 0,  // inertial -> Jacobi coordinates (positions and velocities)
    kOpDrift,             // Kepler drift of every Jacobi body by d
    kOpCom,               // centre-of-mass drift by d
    kOpToInertial,        // Jacobi -> inertial
    kOpGravity,           // BASIC gravity, the 0-1 pair skipped, into the accelerations
    kOpGravityJacobi,     // gravity = JACOBI (src/gravity.c:108-162)
    kOpKick,              // interaction step by d with the Jacobi term
    kOpKickNoJacobiTerm,  // interaction step by d, Jacobi term already in the gravity
    kOpJerk,              // accelerations += d * jerk (kernel MODIFIEDKICK)
    kOpLazyShift,         // positions of bodies 1.. += d * accelerations (kernel LAZY)
    kOpJump,              // jump step by d (democratic heliocentric and WHDS coordinates)
    kOpGravityCompensated,  // gravity = COMPENSATED (src/gravity.c:284-531), same terms skipped
    kOpGravityNone,       // gravity = NONE: zero accelerations
};

// Up to 400 operators per launch keeps the kernel's parameters under 4 KB;
// longer calls run as several launches (the whole state goes through memory
// between them, so a split anywhere is exact).
constexpr int kMaxOps = 400;
struct Program {
    double d[kMaxOps];
    uint8_t op[kMaxOps];
    int32_t n;
};

template <int NB>
__device__ void load_sys(wh::System<NB>& s, const ParticlesSoA& p, int N) {
#pragma unroll
    for (int i = 0; i < NB; i++) {
        const bool on = i < N;
        s.x[i] = on ? p.x[i] : 0.; s.y[i] = on ? p.y[i] : 0.; s.z[i] = on ? p.z[i] : 0.;
        s.vx[i] = on ? p.vx[i] : 0.; s.vy[i] = on ? p.vy[i] : 0.; s.vz[i] = on ? p.vz[i] : 0.;
        s.m[i] = on ? p.m[i] : 0.;
    }
}

template <int NB>
__device__ void store_pos_vel(const wh::System<NB>& s, ParticlesSoA& p, int N) {
#pragma unroll
    for (int i = 0; i < NB; i++) {
        if (i >= N) break;
        p.x[i] = s.x[i]; p.y[i] = s.y[i]; p.z[i] = s.z[i];
        p.vx[i] = s.vx[i]; p.vy[i] = s.vy[i]; p.vz[i] = s.vz[i];
    }
}

template <int NB>
__device__ void load_jac(wh::Jacobi<NB>& j, const double* jac, size_t cap, int N) {
#pragma unroll
    for (int i = 0; i < NB; i++) {
        const bool on = i < N;
        j.x[i] = on ? jac[0 * cap + i] : 0.; j.y[i] = on ? jac[1 * cap + i] : 0.; j.z[i] = on ? jac[2 * cap + i] : 0.;
        j.vx[i] = on ? jac[3 * cap + i] : 0.; j.vy[i] = on ? jac[4 * cap + i] : 0.; j.vz[i] = on ? jac[5 * cap + i] : 0.;
        j.m[i] = on ? jac[6 * cap + i] : 0.;
    }
}

template <int NB>
__device__ void store_jac(const wh::Jacobi<NB>& j, double* jac, size_t cap, int N) {
#pragma unroll
    for (int i = 0; i < NB; i++) {
        if (i >= N) break;
        jac[0 * cap + i] = j.x[i]; jac[1 * cap + i] = j.y[i]; jac[2 * cap + i] = j.z[i];
        jac[3 * cap + i] = j.vx[i]; jac[4 * cap + i] = j.vy[i]; jac[5 * cap + i] = j.vz[i];
        jac[6 * cap + i] = j.m[i];
    }
}

// N_active as WHFast reads it (src/integrator_whfast.c:1119): with
// testparticle_type = 1 every body takes part in the coordinate transforms; the
// gravity keeps the plain N_active (n_active) for its test-particle loop.
inline int wh_active(const rgpu_sim* s) {
    return (s->cfg.testparticle_type == 1 || s->cfg.N_active < 0) ? (int)s->N : (int)s->cfg.N_active;
}

// Runs one program on the handle's system (whfast_prog.cu).
int launch_program(rgpu_sim* s, const Program& prog);

}  // namespace wh_plain
