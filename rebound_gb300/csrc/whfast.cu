// WHFast on an rgpu_sim: the plain, one-simulation-per-call GPU path that a
// REBOUND integrator plugin drives one step at a time
// (src/integrator_whfast.c:1113-1259).  One kernel launch per step; the
// system's state lives in the handle's SoA arrays (inertial) plus a Jacobi
// buffer for safe_mode = 0.  Compiled with --fmad=false: bit-identical to the
// reference's serial build.
#include "whfast_plain.cuh"

namespace {

using namespace wh_plain;

// One step (or a synchronize) of src/integrator_whfast.c for the handle's system.
template <int NB>
__global__ void __launch_bounds__(32) whfast_plain(ParticlesSoA p, double* jac, size_t cap, int N, int Na, int tp,
                                                   double G, double eps2, double dt, int flags, uint32_t* status) {
    if (threadIdx.x != 0) return;
    wh::System<NB> s;
    wh::Jacobi<NB> j;
    load_sys(s, p, N);
    const bool sync_only = (flags & kSyncOnly) != 0;
    if (!sync_only && (flags & kFromInertial)) wh::to_jacobi(s, j, N, Na);
    else load_jac(j, jac, cap, N);
    // One drift call site (rolled passes) keeps one inlined copy of the Kepler solver:
    // pass 0 = the opening drift (dt/2 when synchronized, dt when not) and the kick, or
    // the synchronize drift; pass 1 = the closing drift of safe_mode.
#pragma unroll 1
    for (int pass = 0; pass < 2; pass++) {
        if (pass == 1 && (sync_only || !(flags & kSyncAtEnd))) break;
        const double d = (pass == 0 && !sync_only && !(flags & kFirstHalf)) ? dt : dt / 2.;
        wh::kepler_step(j, s.m[0], G, d, N, Na, status);
        wh::com_step(j, d);
        wh::to_inertial(s, j, N, Na);
        if (pass == 0 && !sync_only) {
            double ax[NB], ay[NB], az[NB];
            wh::gravity_01(s, ax, ay, az, G, eps2, N, Na, tp);
            wh::interaction_step(j, s, ax, ay, az, G, dt, N, Na);
#pragma unroll
            for (int i = 0; i < NB; i++) {
                if (i >= N) break;
                p.ax[i] = ax[i]; p.ay[i] = ay[i]; p.az[i] = az[i];
            }
        }
    }
    store_pos_vel(s, p, N);
    store_jac(j, jac, cap, N);               // synchronize keeps the drifted coordinates, as the reference
}

typedef void (*PlainKernel)(ParticlesSoA, double*, size_t, int, int, int, double, double, double, int, uint32_t*);

template <int NB>
PlainKernel pick() { return whfast_plain<NB>; }

PlainKernel kernel_for(int n) {
    switch (n) {
        case 1: case 2: return pick<2>();
        case 3: return pick<3>();
        case 4: return pick<4>();
        case 5: return pick<5>();
        case 6: return pick<6>();
        case 7: return pick<7>();
        case 8: return pick<8>();
        case 9: return pick<9>();
        case 10: return pick<10>();
        case 11: return pick<11>();
        case 12: return pick<12>();
        case 13: case 14: return pick<14>();
        case 15: case 16: return pick<16>();
        default: return nullptr;
    }
}

int ensure_jac(rgpu_sim* s) {
    if (!s->wh) s->wh = new WhfastBuffers();
    if (s->wh->cap >= s->cap && s->wh->jac) return RGPU_OK;
    cudaFree(s->wh->jac);
    s->wh->jac = nullptr;
    RGPU_CUDA(s, cudaMalloc(&s->wh->jac, sizeof(double) * 7 * s->cap));
    s->wh->cap = s->cap;
    return RGPU_OK;
}

int launch(rgpu_sim* s, int flags) {
    const int N = (int)s->N;
    RGPU_TRY(ensure_jac(s));
    if (s->cfg.whfast_coordinates == 1) return launch_dh(s, flags);
    PlainKernel k = kernel_for(N);
    if (!k) return set_error(s, RGPU_ERR_UNSUPPORTED, "WHFast on the GPU supports 2..16 particles per simulation");
    const rgpu_config& c = s->cfg;
    ktimer_begin(s);
    k<<<1, 32, 0, s->stream>>>(s->p, s->wh->jac, s->cap, N, (int)n_active(s), c.testparticle_type, c.G,
                               c.softening * c.softening, c.dt, flags, s->d_status);
    ktimer_end(s);
    g_launches++;
    RGPU_CUDA(s, cudaGetLastError());
    return RGPU_OK;
}

}  // namespace

int whfast_step(rgpu_sim* s) {
    if (s->N == 0) return RGPU_OK;
    rgpu_config& c = s->cfg;
    if (c.whfast_coordinates != 0 && c.whfast_coordinates != 1)
        return set_error(s, RGPU_ERR_UNSUPPORTED, "WHFast coordinates: 0 (Jacobi) or 1 (democratic heliocentric)");
    c.gravity_ignore_terms = c.whfast_coordinates == 1 ? 2 : 1;  // :929-938
    int flags = 0;
    if (c.whfast_safe_mode || s->did_modify) {
        if (!s->whfast_synchronized) RGPU_TRY(whfast_synchronize(s));
        flags |= kFromInertial;
    }
    if (s->whfast_synchronized) flags |= kFirstHalf;
    if (c.whfast_safe_mode) flags |= kSyncAtEnd;
    RGPU_TRY(launch(s, flags));
    s->whfast_synchronized = c.whfast_safe_mode != 0;
    c.t += c.dt / 2.;                                            // two half steps, as :1186 and :1244
    c.t += c.dt / 2.;
    return RGPU_OK;
}

int whfast_synchronize(rgpu_sim* s) {
    if (s->whfast_synchronized || s->N == 0) { s->whfast_synchronized = true; return RGPU_OK; }
    RGPU_TRY(launch(s, kSyncOnly));
    s->whfast_synchronized = true;
    return RGPU_OK;
}

void whfast_free(rgpu_sim* s) {
    if (!s->wh) return;
    cudaFree(s->wh->jac);
    delete s->wh;
    s->wh = nullptr;
}

namespace {
__global__ void kepler_batch(const double* __restrict__ in, const double* __restrict__ mu,
                             const double* __restrict__ dt, double* __restrict__ out, size_t n, size_t stride_d,
                             uint32_t* status) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* r = in + i * stride_d;
    double x = r[0], y = r[1], z = r[2], vx = r[3], vy = r[4], vz = r[5];
    wh::kepler_solver(x, y, z, vx, vy, vz, mu[i], dt[i], status);
    double* o = out + i * 6;
    o[0] = x; o[1] = y; o[2] = z; o[3] = vx; o[4] = vy; o[5] = vz;
}
}  // namespace

// Device Kepler drift of n independent bodies; the GPU counterpart of the
// reference's public reb_integrator_whfast_kepler_solver
// (src/integrator_whfast.c:241-427).  Inputs are records of `stride` bytes whose
// first six doubles are x, y, z, vx, vy, vz; outputs are 6 doubles per body.
extern "C" int rgpu_kepler_solve(const void* bodies, size_t stride, const double* mu, const double* dt,
                                 double* out, size_t n) {
    if (!bodies || !mu || !dt || !out || stride < 48 || stride % 8) return RGPU_ERR_ARG;
    if (n == 0) return RGPU_OK;
    double *d_in = nullptr, *d_mu = nullptr, *d_dt = nullptr, *d_out = nullptr;
    uint32_t* d_st = nullptr;
    int rc = RGPU_OK;
    if (cudaMalloc(&d_in, n * stride) != cudaSuccess || cudaMalloc(&d_mu, n * 8) != cudaSuccess ||
        cudaMalloc(&d_dt, n * 8) != cudaSuccess || cudaMalloc(&d_out, n * 48) != cudaSuccess ||
        cudaMalloc(&d_st, 4) != cudaSuccess) {
        rc = RGPU_ERR_CUDA;
    } else {
        cudaMemcpy(d_in, bodies, n * stride, cudaMemcpyHostToDevice);
        cudaMemcpy(d_mu, mu, n * 8, cudaMemcpyHostToDevice);
        cudaMemcpy(d_dt, dt, n * 8, cudaMemcpyHostToDevice);
        cudaMemset(d_st, 0, 4);
        kepler_batch<<<(unsigned)((n + 127) / 128), 128>>>(d_in, d_mu, d_dt, d_out, n, stride / 8, d_st);
        g_launches++;
        uint32_t st = 0;
        if (cudaMemcpy(out, d_out, n * 48, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(&st, d_st, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = RGPU_ERR_CUDA;
        else if (st)
            rc = RGPU_ERR_ARG;
    }
    cudaFree(d_in); cudaFree(d_mu); cudaFree(d_dt); cudaFree(d_out); cudaFree(d_st);
    return rc;
}
