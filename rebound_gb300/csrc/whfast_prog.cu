// WHFast programs on an rgpu_sim: the plain one-simulation-per-call path in Jacobi
// coordinates with a first symplectic corrector of order 3, 5, 7, 11 or 17, the
// second corrector, or the kernels MODIFIEDKICK, COMPOSITION and LAZY
// (src/integrator_whfast.c:653-785, 1113-1259; Wisdom, Holman & Touma 1996;
// Wisdom 2006; Rein, Tamayo & Brown 2019).  The host lays each call out as a list
// of operators in the reference's order; one thread runs the list.  Every
// operator has a single call site in the interpreter loop, so the Kepler solver
// is inlined once per body count however long the corrector is.  Compiled with
// --fmad=false: bit-identical to the reference's serial build.
#include "whfast_plain.cuh"

namespace {

using namespace wh_plain;

// reb_gravity_jacobi_calculate_acceleration (src/gravity.c:108-162): direct terms
// plus the Jacobi terms of the Jacobi Hamiltonian's interaction part; no
// softening, every body treated as active.  Rolled loops: the operator is off
// the hot path and keeps the program kernel small.
template <int NB>
__device__ void gravity_jacobi(const wh::System<NB>& s, double ax[NB], double ay[NB], double az[NB], double G,
                               int N) {
    double Rx = 0., Ry = 0., Rz = 0., M = 0.;
#pragma unroll 1
    for (int j = 0; j < N; j++) {
        ax[j] = 0.; ay[j] = 0.; az[j] = 0.;
        const double xj = s.x[j], yj = s.y[j], zj = s.z[j], mj = s.m[j];
        // the Jacobi vector of body j and its length do not depend on i
        double Qx = 0., Qy = 0., Qz = 0., dr3 = 1.;
        if (j > 1) {
            Qx = xj - Rx / M; Qy = yj - Ry / M; Qz = zj - Rz / M;
            const double dr = sqrt(Qx * Qx + Qy * Qy + Qz * Qz);
            dr3 = dr * dr * dr;
        }
#pragma unroll 1
        for (int i = 0; i <= j; i++) {
            if (j > 1) {
                const double dQ = i < j ? -mj : M;          // arranged so that m_j = 0 does not divide
                const double pf = G * dQ / dr3;
                ax[i] += pf * Qx; ay[i] += pf * Qy; az[i] += pf * Qz;
            }
            if (i != j && (i != 0 || j != 1)) {
                const double dx = s.x[i] - xj, dy = s.y[i] - yj, dz = s.z[i] - zj;
                const double dr = sqrt(dx * dx + dy * dy + dz * dz);
                const double pf = G / (dr * dr * dr);
                const double pfi = pf * s.m[i], pfj = pf * mj;
                ax[i] -= pfj * dx; ay[i] -= pfj * dy; az[i] -= pfj * dz;
                ax[j] += pfi * dx; ay[j] += pfi * dy; az[j] += pfi * dz;
            }
        }
        Rx += mj * xj; Ry += mj * yj; Rz += mj * zj;
        M += mj;
    }
}

// reb_integrator_whfast_calculate_jerk (src/integrator_whfast.c:786-870): the time
// derivative of the JACOBI accelerations, then a += d * jerk (:1196-1203).
template <int NB>
__device__ void add_jerk(const wh::System<NB>& s, double ax[NB], double ay[NB], double az[NB], double G, double d,
                         int N) {
    double jx[NB], jy[NB], jz[NB];
    double Rx = 0., Ry = 0., Rz = 0., M = 0., Ax = 0., Ay = 0., Az = 0.;
#pragma unroll 1
    for (int j = 0; j < N; j++) {
        jx[j] = 0.; jy[j] = 0.; jz[j] = 0.;
        const double xj = s.x[j], yj = s.y[j], zj = s.z[j], mj = s.m[j];
        const double axj = ax[j], ayj = ay[j], azj = az[j];
        double Qx = 0., Qy = 0., Qz = 0., dax = 0., day = 0., daz = 0., dr = 1.;
        if (j > 1) {
            Qx = xj - Rx / M; Qy = yj - Ry / M; Qz = zj - Rz / M;
            dax = axj - Ax / M; day = ayj - Ay / M; daz = azj - Az / M;
            dr = sqrt(Qx * Qx + Qy * Qy + Qz * Qz);
        }
#pragma unroll 1
        for (int i = 0; i <= j; i++) {
            if (j > 1) {
                const double dQ = i < j ? -mj : M;
                const double pf2 = G * dQ / (dr * dr * dr);
                jx[i] += pf2 * dax; jy[i] += pf2 * day; jz[i] += pf2 * daz;
                const double alpha = dax * Qx + day * Qy + daz * Qz;
                const double pf1 = 3. * alpha * pf2 / (dr * dr);
                jx[i] -= pf1 * Qx; jy[i] -= pf1 * Qy; jz[i] -= pf1 * Qz;
            }
            if (j != i && (i != 0 || j != 1)) {
                const double dx = xj - s.x[i], dy = yj - s.y[i], dz = zj - s.z[i];
                const double ddx = axj - ax[i], ddy = ayj - ay[i], ddz = azj - az[i];
                const double r = sqrt(dx * dx + dy * dy + dz * dz);
                const double alpha = ddx * dx + ddy * dy + ddz * dz;
                const double pf2 = G / (r * r * r);
                const double pf2i = pf2 * s.m[i], pf2j = pf2 * mj;
                jx[j] -= ddx * pf2i; jy[j] -= ddy * pf2i; jz[j] -= ddz * pf2i;
                jx[i] += ddx * pf2j; jy[i] += ddy * pf2j; jz[i] += ddz * pf2j;
                const double pf1 = 3. * alpha * pf2 / (r * r);
                const double pf1i = pf1 * s.m[i], pf1j = pf1 * mj;
                jx[j] += dx * pf1i; jy[j] += dy * pf1i; jz[j] += dz * pf1i;
                jx[i] -= dx * pf1j; jy[i] -= dy * pf1j; jz[i] -= dz * pf1j;
            }
        }
        Ax += axj * mj; Ay += ayj * mj; Az += azj * mj;
        Rx += xj * mj; Ry += yj * mj; Rz += zj * mj;
        M += mj;
    }
#pragma unroll 1
    for (int i = 0; i < N; i++) {
        ax[i] += d * jx[i]; ay[i] += d * jy[i]; az[i] += d * jz[i];
    }
}

template <int NB>
__global__ void __launch_bounds__(32) whfast_program(ParticlesSoA p, double* jac, size_t cap, int N, int Na, int tp,
                                                     double G, double eps2, const __grid_constant__ Program prog,
                                                     uint32_t* status) {
    if (threadIdx.x != 0) return;
    wh::System<NB> s;
    wh::Jacobi<NB> j;
    double ax[NB], ay[NB], az[NB];
    load_sys(s, p, N);
    load_jac(j, jac, cap, N);
#pragma unroll
    for (int i = 0; i < NB; i++) {
        const bool on = i < N;
        ax[i] = on ? p.ax[i] : 0.; ay[i] = on ? p.ay[i] : 0.; az[i] = on ? p.az[i] : 0.;
    }
#pragma unroll 1
    for (int k = 0; k < prog.n; k++) {
        const double d = prog.d[k];
        const int op = prog.op[k];
        switch (op) {
            case kOpFromInertial: wh::to_jacobi(s, j, N, Na); break;
            case kOpDrift: wh::kepler_step(j, s.m[0], G, d, N, Na, status); break;
            case kOpCom: wh::com_step(j, d); break;
            case kOpToInertial: wh::to_inertial(s, j, N, Na); break;
            case kOpGravity: wh::gravity_01(s, ax, ay, az, G, eps2, N, Na, tp); break;
            case kOpGravityJacobi: gravity_jacobi(s, ax, ay, az, G, N); break;
            case kOpKick:
            case kOpKickNoJacobiTerm:
                wh::interaction_step(j, s, ax, ay, az, G, d, N, Na, op == kOpKick);
                break;
            case kOpJerk: add_jerk(s, ax, ay, az, G, d, N); break;
            case kOpLazyShift:
#pragma unroll 1
                for (int i = 1; i < N; i++) {
                    s.x[i] += d * ax[i]; s.y[i] += d * ay[i]; s.z[i] += d * az[i];
                }
                break;
            default: atomicOr(status, DEV_ERR_PROGRAM); return;
        }
    }
    store_pos_vel(s, p, N);
    store_jac(j, jac, cap, N);
#pragma unroll
    for (int i = 0; i < NB; i++) {
        if (i >= N) break;
        p.ax[i] = ax[i]; p.ay[i] = ay[i]; p.az[i] = az[i];
    }
}

typedef void (*ProgKernel)(ParticlesSoA, double*, size_t, int, int, int, double, double, const Program,
                           uint32_t*);

ProgKernel kernel_for(int n) {
    switch (n) {
        case 1: case 2: return whfast_program<2>;
        case 3: return whfast_program<3>;
        case 4: return whfast_program<4>;
        case 5: return whfast_program<5>;
        case 6: return whfast_program<6>;
        case 7: return whfast_program<7>;
        case 8: return whfast_program<8>;
        case 9: return whfast_program<9>;
        case 10: return whfast_program<10>;
        case 11: return whfast_program<11>;
        case 12: return whfast_program<12>;
        case 13: case 14: return whfast_program<14>;
        case 15: case 16: return whfast_program<16>;
        default: return nullptr;
    }
}

}  // namespace

int wh_plain::launch_program(rgpu_sim* s, const Program& prog) {
    if (prog.n <= 0) return RGPU_OK;
    const int N = (int)s->N;
    ProgKernel k = kernel_for(N);
    if (!k) return set_error(s, RGPU_ERR_UNSUPPORTED, "WHFast on the GPU supports 2..16 particles per simulation");
    const rgpu_config& c = s->cfg;
    ktimer_begin(s);
    k<<<1, 32, 0, s->stream>>>(s->p, s->wh->jac, s->cap, N, (int)n_active(s), c.testparticle_type, c.G,
                               c.softening * c.softening, prog, s->d_status);
    ktimer_end(s);
    g_launches++;
    RGPU_CUDA(s, cudaGetLastError());
    return RGPU_OK;
}
