// WHFast on an rgpu_sim: the plain, one-simulation-per-call GPU path that a
// REBOUND integrator plugin drives one step at a time
// (src/integrator_whfast.c:1113-1259).  Each step or synchronize is laid out as
// a program of operators in the reference's order (ProgramBuilder) and run by
// whfast_program (whfast_prog.cu) in one launch: one lane interprets it, the
// Kepler drifts use one lane per body.  The system's state lives in the
// handle's SoA arrays (inertial) plus a coordinate buffer for safe_mode = 0.
// Compiled with --fmad=false: bit-identical to the reference's serial build.
#include "whfast_plain.cuh"

namespace {

using namespace wh_plain;

int ensure_jac(rgpu_sim* s) {
    if (!s->wh) s->wh = new WhfastBuffers();
    if (s->wh->cap >= s->cap && s->wh->jac) return RGPU_OK;
    cudaFree(s->wh->jac);
    s->wh->jac = nullptr;
    RGPU_CUDA(s, cudaMalloc(&s->wh->jac, sizeof(double) * 7 * s->cap));
    s->wh->cap = s->cap;
    return RGPU_OK;
}

// --- programs: every step and synchronize ---------------------------------------
// The corrector coefficients of src/integrator_whfast.c:124-158 (Wisdom, Holman &
// Touma 1996; Wisdom 2006), kept digit for digit: the products with dt must round
// as the reference's do.
constexpr double kCorrA[9] = {0.,
    0.41833001326703777398908601289259374469640768464934,
    0.83666002653407554797817202578518748939281536929867,
    1.2549900398011133219672580386777812340892230539480,
    1.6733200530681510959563440515703749787856307385973,
    2.0916500663351888699454300644629687234820384232467,
    2.5099800796022266439345160773555624681784461078960,
    2.9283100928692644179236020902481562128748537925454,
    3.3466401061363021919126881031407499575712614771947};
constexpr double kCorrB3[1] = {-0.024900596027799867499350357910273437184309981229127};
constexpr double kCorrB5[2] = {-0.0083001986759332891664501193034244790614366604097090,
                               0.041500993379666445832250596517122395307183302048545};
constexpr double kCorrB7[3] = {0.0024926811426922105779030593952776964450539008582219,
                               -0.018270923246702131478062356884535264841652263842597,
                               0.053964399093127498721765893493510877532452806339655};
constexpr double kCorrB11[5] = {0.00020361579647854651301632818774633716473696537436847,
                                -0.0023487215292295354188307328851055489876255097419754,
                                0.012309078592019946317544564763237909911330686448336,
                                -0.038121613681288650508647613260247372125243616270670,
                                0.072593394748842738674253180742744961827622366521517};
constexpr double kCorrB17[8] = {-0.0000043347415473373580190650223498124944896789841432241,
                                0.000076436355227935738363241846979413475106795392377415,
                                -0.00063599983075817658983166881625078545864140848560259,
                                0.0033132577069380655655490196833451994080066801611459,
                                -0.012071760822342291062449751726959664253913904872527,
                                0.032422198864713580293681523029577130832258806467604,
                                -0.065192863576377893658290760803725762027864651086787,
                                0.093056103771425958591541059067553547100903397724386};
constexpr double kCorr2B = 0.03486083443891981449909050107438281205803;

enum { kKernelDefault = 0, kKernelModifiedKick = 1, kKernelComposition = 2, kKernelLazy = 3 };

// Appends operators to a program and launches it whenever it fills up.
struct ProgramBuilder {
    rgpu_sim* s;
    Program prog;
    int rc = RGPU_OK;
    uint8_t grav, kick;          // the gravity and kick operators of the configured kernel

    explicit ProgramBuilder(rgpu_sim* sim) : s(sim) {
        prog.n = 0;
        const bool jac = s->cfg.whfast_kernel == kKernelModifiedKick || s->cfg.whfast_kernel == kKernelLazy;
        // :929-931 switch gravity to JACOBI; otherwise the simulation's own gravity
        const int g = s->cfg.gravity;
        grav = jac ? kOpGravityJacobi
                   : g == RGPU_GRAVITY_COMPENSATED ? kOpGravityCompensated
                   : g == RGPU_GRAVITY_NONE ? kOpGravityNone : kOpGravity;
        kick = jac ? kOpKickNoJacobiTerm : kOpKick;
    }
    void push(uint8_t op, double d = 0.) {
        if (prog.n == kMaxOps) flush();
        prog.op[prog.n] = op;
        prog.d[prog.n] = d;
        prog.n++;
    }
    int flush() {
        if (prog.n && rc == RGPU_OK) rc = launch_program(s, prog);
        prog.n = 0;
        return rc;
    }
    void drift(double d) { push(kOpDrift, d); }
    void drift_com(double d) { push(kOpDrift, d); push(kOpCom, d); }
    void evaluate_kick(double d) { push(kOpToInertial); push(grav); push(kick, d); }

    // reb_whfast_corrector_Z (:653-694, Jacobi coordinates)
    void corrector_z(double a, double b) {
        drift(a);
        evaluate_kick(-b);
        drift(-2. * a);
        evaluate_kick(b);
        drift(a);
    }
    // reb_whfast_apply_corrector (:696-751): a_k = +-A_k dt, b_k = +-inv B_k dt
    void apply_corrector(double inv, int order) {
        const double dt = s->cfg.dt;
        if (order == 3) {
            corrector_z(kCorrA[1] * dt, -inv * kCorrB3[0] * dt);
            corrector_z(-kCorrA[1] * dt, inv * kCorrB3[0] * dt);
            return;
        }
        const double* B = order == 5 ? kCorrB5 : order == 7 ? kCorrB7 : order == 11 ? kCorrB11 : kCorrB17;
        const int h = order == 5 ? 2 : order == 7 ? 3 : order == 11 ? 5 : 8;
        for (int k = 0; k < h; k++) corrector_z(-kCorrA[h - k] * dt, -inv * B[k] * dt);
        for (int k = h - 1; k >= 0; k--) corrector_z(kCorrA[h - k] * dt, inv * B[k] * dt);
    }
    // reb_whfast_operator_C / _Y / _U and reb_whfast_apply_corrector2 (:753-785)
    void operator_c(double a, double b) { drift(a); evaluate_kick(b); drift(-a); }
    void operator_y(double a, double b) { operator_c(a, b); operator_c(-a, -b); }
    void operator_u(double a, double b) { drift(a); operator_y(a, b); operator_y(a, -b); drift(-a); }
    void apply_corrector2(double inv) {
        const double a = 0.5 * inv * s->cfg.dt;
        const double b = kCorr2B * inv * s->cfg.dt;
        operator_u(a, b);
        operator_u(-a, b);
    }
    // the synchronize sequence (:1051-1111): closing drift, correctors undone, inertial
    void synchronize() {
        const rgpu_config& c = s->cfg;
        const double d = c.whfast_kernel == kKernelComposition ? 3. * c.dt / 8. : c.dt / 2.;
        drift_com(d);
        if (c.whfast_corrector2) apply_corrector2(-1.);
        if (c.whfast_corrector) apply_corrector(-1., c.whfast_corrector);
        push(kOpToInertial);
    }
};

int ensure_keep(rgpu_sim* s) {
    if (s->wh->keep && s->wh->keep_cap == s->wh->cap) return RGPU_OK;
    cudaFree(s->wh->keep);
    s->wh->keep = nullptr;
    RGPU_CUDA(s, cudaMalloc(&s->wh->keep, sizeof(double) * 7 * s->wh->cap));
    s->wh->keep_cap = s->wh->cap;
    return RGPU_OK;
}

// reb_integrator_whfast_init's checks (src/integrator_whfast.c:909-928).
int check_config(rgpu_sim* s) {
    const rgpu_config& c = s->cfg;
    if (c.whfast_coordinates < 0 || c.whfast_coordinates > 3)
        return set_error(s, RGPU_ERR_ARG, "WHFast coordinates: 0 Jacobi, 1 democratic heliocentric, 2 WHDS, 3 barycentric");
    if (c.whfast_kernel < 0 || c.whfast_kernel > 3)
        return set_error(s, RGPU_ERR_ARG, "Kernel method must be 0 (default), 1 (exact modified kick), 2 (composition kernel), or 3 (lazy implementer's modified kick). ");
    if (c.whfast_kernel != kKernelDefault && c.whfast_coordinates != 0)
        return set_error(s, RGPU_ERR_ARG, "Non-standard kernel requires Jacobi coordinates.");
    if (c.whfast_corrector != 0 && c.whfast_coordinates != 0 && c.whfast_coordinates != 3)
        return set_error(s, RGPU_ERR_ARG, "Symplectic correctors are only compatible with Jacobi and Barycentric coordinates.");
    const int k = c.whfast_corrector;
    if (k != 0 && k != 3 && k != 5 && k != 7 && k != 11 && k != 17)
        return set_error(s, RGPU_ERR_ARG, "First symplectic correctors are only available in the following orders: 0, 3, 5, 7, 11, 17.");
    if (c.whfast_corrector2 != 0 && c.whfast_coordinates != 0)
        return set_error(s, RGPU_ERR_UNSUPPORTED, "The second symplectic corrector runs in Jacobi coordinates on the GPU.");
    if (c.gravity != RGPU_GRAVITY_BASIC && c.gravity != RGPU_GRAVITY_COMPENSATED && c.gravity != RGPU_GRAVITY_NONE)
        return set_error(s, RGPU_ERR_UNSUPPORTED, "WHFast on the GPU evaluates BASIC, COMPENSATED or NONE gravity");
    if (c.whfast_keep_unsynchronized && c.whfast_safe_mode)
        return set_error(s, RGPU_ERR_ARG, "whfast->keep_unsynchronized == 1 is not compatible with safe_mode. Must set whfast->safe_mode = 0.");
    return RGPU_OK;
}

// One step as a program (src/integrator_whfast.c:1113-1259).
int program_step(rgpu_sim* s, bool from_inertial) {
    const rgpu_config& c = s->cfg;
    const double dt = c.dt;
    ProgramBuilder b(s);
    if (from_inertial) b.push(kOpFromInertial);
    if (s->whfast_synchronized) {
        if (c.whfast_corrector) b.apply_corrector(1., c.whfast_corrector);
        if (c.whfast_corrector2) b.apply_corrector2(1.);
        b.drift_com(c.whfast_kernel == kKernelComposition ? 5. * dt / 8. : dt / 2.);
    } else {
        b.drift_com(dt);
    }
    const bool jumps = c.whfast_coordinates == 1 || c.whfast_coordinates == 2;
    if (jumps) b.push(kOpJump, dt / 2.);
    b.push(kOpToInertial);
    b.push(b.grav);
    switch (c.whfast_kernel) {
        case kKernelDefault:
            b.push(b.kick, dt);
            if (jumps) b.push(kOpJump, dt / 2.);
            break;
        case kKernelModifiedKick: b.push(kOpJerk, dt * dt / 12.); b.push(b.kick, dt); break;
        case kKernelComposition:
            b.push(b.kick, -dt / 6.);
            b.drift_com(-dt / 4.);
            b.evaluate_kick(dt / 6.);
            b.drift_com(dt / 8.);
            b.evaluate_kick(dt);
            b.drift_com(-dt / 8.);
            b.evaluate_kick(-dt / 6.);
            b.drift_com(dt / 4.);
            b.evaluate_kick(dt / 6.);
            break;
        case kKernelLazy: b.push(kOpLazyShift, dt * dt / 12.); b.push(b.grav); b.push(b.kick, dt); break;
    }
    if (c.whfast_safe_mode) b.synchronize();
    return b.flush();
}

}  // namespace

int whfast_step(rgpu_sim* s) {
    if (s->N == 0) return RGPU_OK;
    rgpu_config& c = s->cfg;
    RGPU_TRY(check_config(s));
    const int k = c.whfast_coordinates;                          // :929-938
    c.gravity_ignore_terms = k == 0 ? 1 : k == 3 ? 0 : 2;
    bool from_inertial = false;
    if (c.whfast_safe_mode || s->did_modify) {
        if (!s->whfast_synchronized) RGPU_TRY(whfast_synchronize(s));
        from_inertial = true;
    }
    RGPU_TRY(ensure_jac(s));
    RGPU_TRY(program_step(s, from_inertial));
    s->whfast_synchronized = c.whfast_safe_mode != 0;
    c.t += c.dt / 2.;                                            // two half steps, as :1186 and :1244
    c.t += c.dt / 2.;
    return RGPU_OK;
}

int whfast_synchronize(rgpu_sim* s) {
    if (s->whfast_synchronized || s->N == 0) { s->whfast_synchronized = true; return RGPU_OK; }
    RGPU_TRY(check_config(s));
    RGPU_TRY(ensure_jac(s));
    const bool keep = s->cfg.whfast_keep_unsynchronized != 0;
    const size_t bytes = sizeof(double) * 7 * s->wh->cap;
    if (keep) {                                                  // :1060-1064
        RGPU_TRY(ensure_keep(s));
        RGPU_CUDA(s, cudaMemcpyAsync(s->wh->keep, s->wh->jac, bytes, cudaMemcpyDeviceToDevice, s->stream));
    }
    {
        ProgramBuilder b(s);
        b.synchronize();
        RGPU_TRY(b.flush());
    }
    if (keep) {                                                  // :1102-1104
        RGPU_CUDA(s, cudaMemcpyAsync(s->wh->jac, s->wh->keep, bytes, cudaMemcpyDeviceToDevice, s->stream));
        return RGPU_OK;
    }
    s->whfast_synchronized = true;
    return RGPU_OK;
}

int whfast_load_coordinates(rgpu_sim* s, const double* host7N) {
    RGPU_TRY(ensure_jac(s));
    for (int f = 0; f < 7; f++)
        RGPU_CUDA(s, cudaMemcpyAsync(s->wh->jac + f * s->wh->cap, host7N + f * s->N, sizeof(double) * s->N,
                                     cudaMemcpyHostToDevice, s->stream));
    return RGPU_OK;
}

void whfast_free(rgpu_sim* s) {
    if (!s->wh) return;
    cudaFree(s->wh->jac);
    cudaFree(s->wh->keep);
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
