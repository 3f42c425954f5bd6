// WHFast in democratic heliocentric coordinates (Duncan, Levison & Lee 1998) on an
// rgpu_sim: the plain one-simulation-per-call path with
// coordinates = REB_INTEGRATOR_WHFAST_COORDINATES_DEMOCRATICHELIOCENTRIC and the
// DEFAULT kernel (src/integrator_whfast.c:1113-1259).  Per step: Kepler drift of
// every body about the star (mu = G m_0) and centre-of-mass drift, half jump, the
// planets' mutual accelerations (every term involving the star skipped), kick,
// half jump, and with safe_mode the closing half drift.  Compiled with
// --fmad=false like the Jacobi unit: bit-identical to the reference's serial build.
#include "whfast_plain.cuh"

namespace {

using namespace wh_plain;

template <int NB>
__global__ void __launch_bounds__(32) whfast_plain_dh(ParticlesSoA p, double* buf, size_t cap, int N, int Na, int Ng, int tp,
                                                      double G, double eps2, double dt, int flags, uint32_t* status) {
    if (threadIdx.x != 0) return;
    wh::System<NB> s;
    wh::Jacobi<NB> h;                                   // democratic heliocentric coordinates (p_h)
    load_sys(s, p, N);
    const bool sync_only = (flags & kSyncOnly) != 0;
    if (!sync_only && (flags & kFromInertial)) wh::to_dh(s, h, N, Na);
    else load_jac(h, buf, cap, N);
    // One drift call site (rolled passes) keeps one inlined copy of the Kepler solver:
    // pass 0 = the opening drift (dt/2 when synchronized, dt when not) and the kick, or
    // the synchronize drift; pass 1 = the closing drift of safe_mode.
#pragma unroll 1
    for (int pass = 0; pass < 2; pass++) {
        if (pass == 1 && (sync_only || !(flags & kSyncAtEnd))) break;
        const double d = (pass == 0 && !sync_only && !(flags & kFirstHalf)) ? dt : dt / 2.;
        wh::kepler_step_dh(h, s.m[0], G, d, N, status);
        wh::com_step(h, d);
        if (pass == 0 && !sync_only) wh::jump_step_dh(h, s, dt / 2., N, Na);   // opening half jump
        wh::dh_to_inertial(s, h, N, Na);
        if (pass == 0 && !sync_only) {
            double ax[NB], ay[NB], az[NB];
            wh::gravity_01<NB, 1>(s, ax, ay, az, G, eps2, N, Ng, tp);
            wh::interaction_step_dh(h, ax, ay, az, dt, N);
            wh::jump_step_dh(h, s, dt / 2., N, Na);
#pragma unroll
            for (int i = 0; i < NB; i++) {
                if (i >= N) break;
                p.ax[i] = ax[i]; p.ay[i] = ay[i]; p.az[i] = az[i];
            }
        }
    }
    store_pos_vel(s, p, N);
    store_jac(h, buf, cap, N);               // synchronize keeps the drifted coordinates, as the reference
}

typedef void (*PlainKernel)(ParticlesSoA, double*, size_t, int, int, int, int, double, double, double, int, uint32_t*);

PlainKernel kernel_for(int n) {
    switch (n) {
        case 1: case 2: return whfast_plain_dh<2>;
        case 3: return whfast_plain_dh<3>;
        case 4: return whfast_plain_dh<4>;
        case 5: return whfast_plain_dh<5>;
        case 6: return whfast_plain_dh<6>;
        case 7: return whfast_plain_dh<7>;
        case 8: return whfast_plain_dh<8>;
        case 9: return whfast_plain_dh<9>;
        case 10: return whfast_plain_dh<10>;
        case 11: return whfast_plain_dh<11>;
        case 12: return whfast_plain_dh<12>;
        case 13: case 14: return whfast_plain_dh<14>;
        case 15: case 16: return whfast_plain_dh<16>;
        default: return nullptr;
    }
}

}  // namespace

int wh_plain::launch_dh(rgpu_sim* s, int flags) {
    const int N = (int)s->N;
    PlainKernel k = kernel_for(N);
    if (!k) return set_error(s, RGPU_ERR_UNSUPPORTED, "WHFast on the GPU supports 2..16 particles per simulation");
    const rgpu_config& c = s->cfg;
    ktimer_begin(s);
    k<<<1, 32, 0, s->stream>>>(s->p, s->wh->jac, s->cap, N, wh_active(s), (int)n_active(s), c.testparticle_type, c.G,
                               c.softening * c.softening, c.dt, flags, s->d_status);
    ktimer_end(s);
    g_launches++;
    RGPU_CUDA(s, cudaGetLastError());
    return RGPU_OK;
}
