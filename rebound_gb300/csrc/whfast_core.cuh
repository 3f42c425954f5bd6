// WHFast building blocks for one small system: the Kepler solver, the Jacobi
// and democratic heliocentric transforms, kicks, jumps and the full safe_mode
// steps the ensembles run (src/integrator_whfast.c and src/transformations.c of
// REBOUND 5.0.0).  The plain path's program kernel (whfast_prog.cu) composes
// them with the other coordinate systems, kernels and correctors.
//
// Each function restates the reference routine it names with the same
// sequence of floating-point operations, so a translation unit compiled with
// --fmad=false reproduces the reference bit for bit (IEEE division and square
// root are correctly rounded on both).  The batched ensemble includes this
// header from a unit compiled with FMA contraction, trading bit-identity for
// fewer FP64 instructions.
//
// Every data-dependent loop carries an iteration cap; on hitting it the
// solver records DEV_ERR_KEPLER in the device status word and continues with
// its current estimate instead of spinning.
#pragma once
#include "exactfp.cuh"
#include "rgpu_internal.cuh"

namespace wh {

constexpr int kMaxBodies = 16;

// Division and square root.  By default the IEEE operations, as the reference
// computes them.  A unit that defines WH_FAST_MATH before including this header
// (the FMA-contracted ensemble and serving kernels, which already trade
// bit-identity for speed) gets them from the hardware's approximate reciprocal
// and reciprocal square root refined by Newton steps in FP64 (within an ulp or
// two of IEEE, checked by rgpu_selftest_fastmath): fewer instructions on GB300's
// narrow FP64 pipe.  A unit that defines WH_INT_DIVSQRT takes the IEEE-exact
// division and square root built on the integer pipes (exactfp), out of line so
// the many call sites share one copy: they leave the FP64 pipe to the rest of
// the step (the thread-per-system ensemble: +12 % system-steps/s) and, being
// exact, keep a bit-exact unit bit-exact.
#ifdef WH_FAST_MATH
__device__ __forceinline__ double fast_rcp(double b) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(b));
    double e = fma(-b, y, 1.0);
    y = fma(y, e, y);
    e = fma(-b, y, 1.0);
    return fma(y, e, y);
}
__device__ __forceinline__ double fast_div(double a, double b) {
    const double y = fast_rcp(b);
    const double q = a * y;
    return fma(fma(-b, q, a), y, q);
}
__device__ __forceinline__ double fast_sqrt(double x) {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    y = y * fma(-0.5 * x * y, y, 1.5);
    const double s = x * y;
    const double r = fma(fma(-s, s, x), 0.5 * y, s);
    // positive finite: r; 0 and +inf give themselves, negative and NaN give NaN (as IEEE)
    const bool pos = x > 0. && x < __longlong_as_double(0x7ff0000000000000LL);
    return pos ? r : (x == 0. || x > 0. ? x : __longlong_as_double(0x7ff8000000000000LL));
}
#endif
#if defined(WH_INT_DIVSQRT)
static __device__ __noinline__ double int_div(double a, double b) { return ::exactfp::div_rn(a, b); }
static __device__ __noinline__ double int_sqrt(double x) { return ::exactfp::sqrt_rn(x); }
#define WH_DIV(a, b) (::wh::int_div((a), (b)))
#define WH_RCP(b) (::wh::int_div(1.0, (b)))
#define WH_SQRT(x) (::wh::int_sqrt(x))
#elif defined(WH_FAST_MATH)
#define WH_DIV(a, b) (::wh::fast_div((a), (b)))
#define WH_RCP(b) (::wh::fast_rcp(b))
#define WH_SQRT(x) (::wh::fast_sqrt(x))
#else
#define WH_DIV(a, b) ((a) / (b))
#define WH_RCP(b) (1. / (b))
#define WH_SQRT(x) (sqrt(x))
#endif

template <int NB>
struct System {
    double x[NB], y[NB], z[NB], vx[NB], vy[NB], vz[NB], m[NB];
};

template <int NB>
struct Jacobi {
    double x[NB], y[NB], z[NB], vx[NB], vy[NB], vz[NB], m[NB];
};

__device__ static const double kInvFact[14] = {
    1., 1., 1. / 2., 1. / 6., 1. / 24., 1. / 120., 1. / 720., 1. / 5040., 1. / 40320., 1. / 362880.,
    1. / 3628800., 1. / 39916800., 1. / 479001600., 1. / 6227020800.};

// stumpff_cs3 (src/integrator_whfast.c:189-212).
__device__ __forceinline__ void stumpff_c3(double cs[4], double z, uint32_t* status) {
    unsigned n = 0;
    while (fabs(z) > 0.1) {
        z = z / 4.;
        n++;
        if (n > 1200) { atomicOr(status, DEV_ERR_KEPLER); break; }   // z = inf would never shrink
    }
    const int nmax = 13;
    double co = kInvFact[nmax], ce = kInvFact[nmax - 1];
#pragma unroll
    for (int np = nmax - 2; np >= 3; np -= 2) {
        co = kInvFact[np] - z * co;
        ce = kInvFact[np - 1] - z * ce;
    }
    cs[3] = co;
    cs[2] = ce;
    cs[1] = kInvFact[1] - z * co;
    cs[0] = kInvFact[0] - z * ce;
    for (; n > 0; n--) {
        cs[3] = (cs[2] + cs[0] * cs[3]) * 0.25;
        cs[2] = cs[1] * cs[1] * 0.5;
        cs[1] = cs[0] * cs[1];
        cs[0] = 2. * cs[0] * cs[0] - 1.;
    }
}

// stiefel_Gs3 (src/integrator_whfast.c:226-232).
__device__ __forceinline__ void stiefel_g3(double Gs[4], double beta, double X, uint32_t* status) {
    const double X2 = X * X;
    stumpff_c3(Gs, beta * X2, status);
    Gs[1] *= X;
    Gs[2] *= X2;
    Gs[3] *= X2 * X;
}

// The solver depends on no template parameter: under WH_INT_DIVSQRT it is
// compiled once, out of line, instead of once per body-count instantiation
// (half the build time of the ensemble unit, and +7 % system-steps/s from the
// smaller kernel).
#ifdef WH_INT_DIVSQRT
#define WH_SOLVER static __device__ __noinline__
#else
#define WH_SOLVER __device__ inline
#endif

// reb_integrator_whfast_kepler_solver (src/integrator_whfast.c:241-427) for one body.
WH_SOLVER void kepler_solver(double& px, double& py, double& pz, double& pvx, double& pvy, double& pvz,
                                     double mu, double dt, uint32_t* status) {
    const double x = px, y = py, z = pz, vx = pvx, vy = pvy, vz = pvz;
    const double r0 = WH_SQRT(x * x + y * y + z * z);
    const double r0i = WH_RCP(r0);
    const double v2 = vx * vx + vy * vy + vz * vz;
    const double beta = 2. * mu * r0i - v2;
    const double eta0 = x * vx + y * vy + z * vz;
    const double zeta0 = mu - beta * r0;
    double X, Gs[4], X_per_period = __longlong_as_double(0x7ff8000000000000LL);
#ifndef WH_INT_DIVSQRT
    double invperiod = 0.;
#endif
    if (beta > 0.) {
        const double sb = WH_SQRT(beta);
#ifndef WH_INT_DIVSQRT
        invperiod = WH_DIV(sb * beta, 2. * M_PI * mu);
#endif
        X_per_period = WH_DIV(2. * M_PI, sb);
        const double dtr0i = dt * r0i;
        X = dtr0i * (1. - dtr0i * eta0 * 0.5 * r0i);
    } else {
        X = 0.;
    }
    int converged = 0;
    double oldX = X;
    stiefel_g3(Gs, beta, X, status);
    const double e1 = eta0 * Gs[1] + zeta0 * Gs[2];
    double ri = WH_RCP(r0 + e1);
    X = ri * (X * e1 - eta0 * Gs[2] - zeta0 * Gs[3] + dt);
    if (fabs(X - oldX) > 0.01 * X_per_period) {
        // Quartic (Laguerre-type) solver, up to 64 iterations, converged when X repeats.
        X = WH_DIV(beta * dt, mu);
        // Converged when X repeats an earlier iterate (a cycle).  The bit-exact
        // flavours compare with every earlier iterate, as the reference; the
        // fast flavour keeps the last 8 in a ring (less local memory per thread).
#ifdef WH_FAST_MATH
        constexpr int kHist = 8;
#else
        constexpr int kHist = 64;
#endif
        double prevX[kHist];
        for (int nl = 1; nl < 64; nl++) {
            stiefel_g3(Gs, beta, X, status);
            const double f = r0 * X + eta0 * Gs[2] + zeta0 * Gs[3] - dt;
            const double fp = r0 + eta0 * Gs[1] + zeta0 * Gs[2];
            const double fpp = eta0 * Gs[0] + zeta0 * Gs[1];
            const double den = fp + WH_SQRT(fabs(16. * fp * fp - 20. * f * fpp));
            X = WH_DIV(X * den - 5. * f, den);
            const int stored = nl - 1 < kHist ? nl - 1 : kHist;
            for (int i = 0; i < stored; i++) {
                if (X == prevX[i]) { nl = 64; converged = 1; break; }
            }
            if (nl < 64) prevX[(nl - 1) % kHist] = X;
        }
        const double e2 = eta0 * Gs[1] + zeta0 * Gs[2];
        ri = WH_RCP(r0 + e2);
    } else {
        double oldX2;
        for (int nh = 1; nh < 32; nh++) {
            oldX2 = oldX;
            oldX = X;
            stiefel_g3(Gs, beta, X, status);
            const double e2 = eta0 * Gs[1] + zeta0 * Gs[2];
            ri = WH_RCP(r0 + e2);
            X = ri * (X * e2 - eta0 * Gs[2] - zeta0 * Gs[3] + dt);
            if (X == oldX || X == oldX2) { converged = 1; break; }
        }
    }
    if (!converged) {
        // Bisection fallback (src/integrator_whfast.c:333-370), capped.
        double Xmin, Xmax;
        if (beta > 0.) {
#ifdef WH_INT_DIVSQRT
            // the ensemble forms the orbital frequency only here, where it is
            // used (the reference forms it up front for a warning, :258)
            const double sb = WH_SQRT(beta);
            const double invperiod = WH_DIV(sb * beta, 2. * M_PI * mu);
#endif
            Xmin = X_per_period * floor(dt * invperiod);
            Xmax = Xmin + X_per_period;
        } else {
            const double h2 = r0 * r0 * v2 - eta0 * eta0;
            const double q = h2 / mu / (1. + sqrt(1. - h2 * beta / (mu * mu)));
            const double vq = copysign(sqrt(h2) / q, dt);
            Xmin = dt / (fabs(vq * dt) + r0);
            Xmax = dt / q;
            if (dt < 0.) { const double t = Xmin; Xmin = Xmax; Xmax = t; }
        }
        X = (Xmax + Xmin) / 2.;
        int it = 0;
        do {
            stiefel_g3(Gs, beta, X, status);
            const double s = r0 * X + eta0 * Gs[2] + zeta0 * Gs[3] - dt;
            if (s >= 0.) Xmax = X; else Xmin = X;
            X = (Xmax + Xmin) / 2.;
            if (++it > 4096) { atomicOr(status, DEV_ERR_KEPLER); break; }
        } while (fabs(Xmax - Xmin) > fabs((Xmax + Xmin) * 1e-15));
        const double e2 = eta0 * Gs[1] + zeta0 * Gs[2];
        ri = WH_RCP(r0 + e2);
    }
    if (isnan(ri)) { ri = 0.; Gs[1] = 0.; Gs[2] = 0.; Gs[3] = 0.; }
    const double f = -mu * Gs[2] * r0i;
    const double g = dt - mu * Gs[3];
    const double fd = -mu * Gs[1] * r0i * ri;
    const double gd = -mu * Gs[2] * ri;
    px += f * x + g * vx;
    py += f * y + g * vy;
    pz += f * z + g * vz;
    pvx += fd * x + gd * vx;
    pvy += fd * y + gd * vy;
    pvz += fd * z + gd * vz;
}

// reb_transformations_inertial_to_jacobi_posvel (src/transformations.c:34-81).
template <int NB>
__device__ __forceinline__ void to_jacobi(const System<NB>& s, Jacobi<NB>& j, int N, int Na) {
    double eta = s.m[0];
    double sx = eta * s.x[0], sy = eta * s.y[0], sz = eta * s.z[0];
    double svx = eta * s.vx[0], svy = eta * s.vy[0], svz = eta * s.vz[0];
#pragma unroll
    for (int i = 1; i < NB; i++) {
        if (i >= Na) break;
        const double ei = 1. / eta;
        eta += s.m[i];
        const double pme = eta * ei;
        j.m[i] = s.m[i];
        j.x[i] = s.x[i] - sx * ei; j.y[i] = s.y[i] - sy * ei; j.z[i] = s.z[i] - sz * ei;
        j.vx[i] = s.vx[i] - svx * ei; j.vy[i] = s.vy[i] - svy * ei; j.vz[i] = s.vz[i] - svz * ei;
        sx = sx * pme + s.m[i] * j.x[i]; sy = sy * pme + s.m[i] * j.y[i]; sz = sz * pme + s.m[i] * j.z[i];
        svx = svx * pme + s.m[i] * j.vx[i]; svy = svy * pme + s.m[i] * j.vy[i]; svz = svz * pme + s.m[i] * j.vz[i];
    }
    const double ei = 1. / eta;
#pragma unroll
    for (int i = 1; i < NB; i++) {
        if (i < Na || i >= N) continue;
        j.m[i] = s.m[i];
        j.x[i] = s.x[i] - sx * ei; j.y[i] = s.y[i] - sy * ei; j.z[i] = s.z[i] - sz * ei;
        j.vx[i] = s.vx[i] - svx * ei; j.vy[i] = s.vy[i] - svy * ei; j.vz[i] = s.vz[i] - svz * ei;
    }
    const double mti = 1. / eta;
    j.m[0] = eta;
    j.x[0] = sx * mti; j.y[0] = sy * mti; j.z[0] = sz * mti;
    j.vx[0] = svx * mti; j.vy[0] = svy * mti; j.vz[0] = svz * mti;
}

// reb_transformations_jacobi_to_inertial_posvel (src/transformations.c:178-226).
template <int NB>
__device__ __forceinline__ void to_inertial(System<NB>& s, const Jacobi<NB>& j, int N, int Na) {
    double eta = j.m[0];
    double sx = j.x[0] * eta, sy = j.y[0] * eta, sz = j.z[0] * eta;
    double svx = j.vx[0] * eta, svy = j.vy[0] * eta, svz = j.vz[0] * eta;
#pragma unroll
    for (int i = NB - 1; i >= 1; i--) {
        if (i >= N || i < Na) continue;
        const double ei = 1. / eta;
        s.x[i] = j.x[i] + sx * ei; s.y[i] = j.y[i] + sy * ei; s.z[i] = j.z[i] + sz * ei;
        s.vx[i] = j.vx[i] + svx * ei; s.vy[i] = j.vy[i] + svy * ei; s.vz[i] = j.vz[i] + svz * ei;
    }
#pragma unroll
    for (int i = NB - 1; i >= 1; i--) {
        if (i >= Na) continue;
        const double ei = 1. / eta;
        const double mi = s.m[i];
        sx = (sx - mi * j.x[i]) * ei; sy = (sy - mi * j.y[i]) * ei; sz = (sz - mi * j.z[i]) * ei;
        svx = (svx - mi * j.vx[i]) * ei; svy = (svy - mi * j.vy[i]) * ei; svz = (svz - mi * j.vz[i]) * ei;
        s.x[i] = j.x[i] + sx; s.y[i] = j.y[i] + sy; s.z[i] = j.z[i] + sz;
        s.vx[i] = j.vx[i] + svx; s.vy[i] = j.vy[i] + svy; s.vz[i] = j.vz[i] + svz;
        eta -= mi;
        sx *= eta; sy *= eta; sz *= eta; svx *= eta; svy *= eta; svz *= eta;
    }
    const double mi = 1. / eta;
    s.x[0] = sx * mi; s.y[0] = sy * mi; s.z[0] = sz * mi;
    s.vx[0] = svx * mi; s.vy[0] = svy * mi; s.vz[0] = svz * mi;
}

// Kepler drift of every Jacobi body, serial-eta branch (src/integrator_whfast.c:589-636).
template <int NB>
__device__ __forceinline__ void kepler_step(Jacobi<NB>& j, double m0, double G, double dt, int N, int Na,
                                            uint32_t* status) {
    double eta = m0;
    // Rolled on purpose: one copy of the solver per instantiation keeps code
    // size and compile time bounded (the Jacobi arrays then live in L1-cached
    // local memory, cheap next to the solver's FP64 work).
#pragma unroll 1
    for (int i = 1; i < NB; i++) {
        if (i >= N) break;
        if (i < Na) eta += j.m[i];
        kepler_solver(j.x[i], j.y[i], j.z[i], j.vx[i], j.vy[i], j.vz[i], eta * G, dt, status);
    }
}

// reb_integrator_whfast_com_step (src/integrator_whfast.c:638-651).
template <int NB>
__device__ __forceinline__ void com_step(Jacobi<NB>& j, double dt) {
    j.x[0] += dt * j.vx[0];
    j.y[0] += dt * j.vy[0];
    j.z[0] += dt * j.vz[0];
}

// BASIC gravity with gravity_ignore_terms = 1 (skip the 0-1 pair), serial
// pairwise order (src/gravity.c:195-257, starti = 2, startj = 0).
// STARTJ = 1: gravity_ignore_terms = 2, every term involving particle 0 skipped
// (democratic heliocentric coordinates; src/gravity.c:180-181, startj = 1).
template <int NB, int STARTJ = 0>
__device__ __forceinline__ void gravity_01(const System<NB>& s, double ax[NB], double ay[NB], double az[NB],
                                           double G, double eps2, int N, int Na, int tp) {
#pragma unroll
    for (int i = 0; i < NB; i++) { ax[i] = 0.; ay[i] = 0.; az[i] = 0.; }
#pragma unroll
    for (int i = 2; i < NB; i++) {
        if (i >= Na) break;
#pragma unroll
        for (int jj = STARTJ; jj < i; jj++) {
            const double dx = (0. + s.x[i]) - s.x[jj];
            const double dy = (0. + s.y[i]) - s.y[jj];
            const double dz = (0. + s.z[i]) - s.z[jj];
            const double r = WH_SQRT(dx * dx + dy * dy + dz * dz + eps2);
            const double pf = WH_DIV(G, r * r * r);
            const double pfj = -pf * s.m[jj];
            const double pfi = pf * s.m[i];
            ax[i] += pfj * dx; ay[i] += pfj * dy; az[i] += pfj * dz;
            ax[jj] += pfi * dx; ay[jj] += pfi * dy; az[jj] += pfi * dz;
        }
    }
    const int st = Na > 2 ? Na : 2;
#pragma unroll
    for (int i = 2; i < NB; i++) {
        if (i < st || i >= N) continue;
#pragma unroll
        for (int jj = STARTJ; jj < NB; jj++) {
            if (jj >= Na) break;
            const double dx = (0. + s.x[i]) - s.x[jj];
            const double dy = (0. + s.y[i]) - s.y[jj];
            const double dz = (0. + s.z[i]) - s.z[jj];
            const double r = WH_SQRT(dx * dx + dy * dy + dz * dz + eps2);
            const double pf = WH_DIV(G, r * r * r);
            const double pfj = -pf * s.m[jj];
            ax[i] += pfj * dx; ay[i] += pfj * dy; az[i] += pfj * dz;
            if (tp) {
                const double pfi = pf * s.m[i];
                ax[jj] += pfi * dx; ay[jj] += pfi * dy; az[jj] += pfi * dz;
            }
        }
    }
}

// Interaction (kick) step in Jacobi coordinates: inertial_to_jacobi_acc
// (src/transformations.c:147-176) then src/integrator_whfast.c:447-472.
template <int NB>
__device__ __forceinline__ void interaction_step(Jacobi<NB>& j, const System<NB>& s, const double ax[NB],
                                                 const double ay[NB], const double az[NB], double G, double dt,
                                                 int N, int Na, bool jacobi_term = true) {
    double jax[NB], jay[NB], jaz[NB];
    double eta = s.m[0];
    double sx = eta * ax[0], sy = eta * ay[0], sz = eta * az[0];
#pragma unroll
    for (int i = 1; i < NB; i++) {
        if (i >= Na) break;
        const double ei = 1. / eta;
        eta += s.m[i];
        const double pme = eta * ei;
        jax[i] = ax[i] - sx * ei; jay[i] = ay[i] - sy * ei; jaz[i] = az[i] - sz * ei;
        sx = sx * pme + s.m[i] * jax[i]; sy = sy * pme + s.m[i] * jay[i]; sz = sz * pme + s.m[i] * jaz[i];
    }
    {
        const double ei = 1. / eta;
#pragma unroll
        for (int i = 1; i < NB; i++) {
            if (i < Na || i >= N) continue;
            jax[i] = ax[i] - sx * ei; jay[i] = ay[i] - sy * ei; jaz[i] = az[i] - sz * ei;
        }
    }
    eta = s.m[0];
#pragma unroll
    for (int i = 1; i < NB; i++) {
        if (i >= N) break;
        const double qx = j.x[i], qy = j.y[i], qz = j.z[i];
        if (i < Na) eta += j.m[i];
        j.vx[i] += dt * jax[i];
        j.vy[i] += dt * jay[i];
        j.vz[i] += dt * jaz[i];
        if (i > 1 && jacobi_term) {   // with gravity = JACOBI the term is in the accelerations
            const double rj2i = WH_RCP(qx * qx + qy * qy + qz * qz);
            const double rji = WH_SQRT(rj2i);
            const double rj3iM = rji * rj2i * G * eta;
            const double pf = dt * rj3iM;
            j.vx[i] += pf * qx;
            j.vy[i] += pf * qy;
            j.vz[i] += pf * qz;
        }
    }
}

// --- democratic heliocentric coordinates (Duncan, Levison & Lee 1998) -----------
// h[0]: centre of mass (position and velocity) and total mass; h[i], i >= 1:
// heliocentric position, barycentric velocity.

// reb_transformations_inertial_to_democraticheliocentric_posvel (src/transformations.c:388-425).
template <int NB>
__device__ __forceinline__ void to_dh(const System<NB>& s, Jacobi<NB>& h, int N, int Na) {
    double x0 = 0., y0 = 0., z0 = 0., vx0 = 0., vy0 = 0., vz0 = 0., m0 = 0.;
#pragma unroll
    for (int i = 0; i < NB; i++) {
        if (i >= Na) break;
        const double m = s.m[i];
        x0 += s.x[i] * m; y0 += s.y[i] * m; z0 += s.z[i] * m;
        vx0 += s.vx[i] * m; vy0 += s.vy[i] * m; vz0 += s.vz[i] * m;
        m0 += m;
    }
    h.x[0] = x0 / m0; h.y[0] = y0 / m0; h.z[0] = z0 / m0;
    h.vx[0] = vx0 / m0; h.vy[0] = vy0 / m0; h.vz[0] = vz0 / m0;
    h.m[0] = m0;
#pragma unroll
    for (int i = 1; i < NB; i++) {
        if (i >= N) break;
        h.x[i] = s.x[i] - s.x[0]; h.y[i] = s.y[i] - s.y[0]; h.z[i] = s.z[i] - s.z[0];
        h.vx[i] = s.vx[i] - h.vx[0]; h.vy[i] = s.vy[i] - h.vy[0]; h.vz[i] = s.vz[i] - h.vz[0];
        h.m[i] = s.m[i];
    }
}

// reb_transformations_democraticheliocentric_to_inertial_posvel (src/transformations.c:427-473).
template <int NB>
__device__ __forceinline__ void dh_to_inertial(System<NB>& s, const Jacobi<NB>& h, int N, int Na) {
    const double mtot = h.m[0];
    double x0 = 0., y0 = 0., z0 = 0.;
#pragma unroll
    for (int i = 1; i < NB; i++) {
        if (i >= Na) break;
        const double m = h.m[i];
        x0 += h.x[i] * m / mtot; y0 += h.y[i] * m / mtot; z0 += h.z[i] * m / mtot;
        s.m[i] = m;
    }
    s.x[0] = h.x[0] - x0; s.y[0] = h.y[0] - y0; s.z[0] = h.z[0] - z0;
#pragma unroll
    for (int i = 1; i < NB; i++) {
        if (i >= N) break;
        s.x[i] = h.x[i] + s.x[0]; s.y[i] = h.y[i] + s.y[0]; s.z[i] = h.z[i] + s.z[0];
    }
    const double m0 = s.m[0];
#pragma unroll
    for (int i = 1; i < NB; i++) {
        if (i >= N) break;
        s.vx[i] = h.vx[i] + h.vx[0]; s.vy[i] = h.vy[i] + h.vy[0]; s.vz[i] = h.vz[i] + h.vz[0];
    }
    double vx0 = 0., vy0 = 0., vz0 = 0.;
#pragma unroll
    for (int i = 1; i < NB; i++) {
        if (i >= Na) break;
        const double m = s.m[i];
        vx0 += h.vx[i] * m / m0; vy0 += h.vy[i] * m / m0; vz0 += h.vz[i] * m / m0;
    }
    s.vx[0] = h.vx[0] - vx0; s.vy[0] = h.vy[0] - vy0; s.vz[0] = h.vz[0] - vz0;
}

// Kepler drift about the star alone, mu = G m_0 (src/integrator_whfast.c:611-616).
template <int NB>
__device__ __forceinline__ void kepler_step_dh(Jacobi<NB>& h, double m0, double G, double dt, int N,
                                               uint32_t* status) {
#pragma unroll 1
    for (int i = 1; i < NB; i++) {
        if (i >= N) break;
        kepler_solver(h.x[i], h.y[i], h.z[i], h.vx[i], h.vy[i], h.vz[i], m0 * G, dt, status);
    }
}

// Jump step: drift by the star's momentum share (src/integrator_whfast.c:536-553).
template <int NB>
__device__ __forceinline__ void jump_step_dh(Jacobi<NB>& h, const System<NB>& s, double dt, int N, int Na) {
    const double m0 = s.m[0];
    double px = 0., py = 0., pz = 0.;
#pragma unroll
    for (int i = 1; i < NB; i++) {
        if (i >= Na) break;
        const double m = s.m[i];
        px += m * h.vx[i]; py += m * h.vy[i]; pz += m * h.vz[i];
    }
#pragma unroll
    for (int i = 1; i < NB; i++) {
        if (i >= N) break;
        h.x[i] += dt * (px / m0); h.y[i] += dt * (py / m0); h.z[i] += dt * (pz / m0);
    }
}

// Interaction kick with the planets' mutual accelerations (src/integrator_whfast.c:494-500).
template <int NB>
__device__ __forceinline__ void interaction_step_dh(Jacobi<NB>& h, const double ax[NB], const double ay[NB],
                                                    const double az[NB], double dt, int N) {
#pragma unroll
    for (int i = 1; i < NB; i++) {
        if (i >= N) break;
        h.vx[i] += dt * ax[i]; h.vy[i] += dt * ay[i]; h.vz[i] += dt * az[i];
    }
}

// One WHFast step with safe_mode = 1 (src/integrator_whfast.c:1113-1259 with
// the synchronize of :1051-1111): the state enters and leaves synchronized.
template <int NB>
__device__ __forceinline__ void step_safe(System<NB>& s, double G, double eps2, double dt, int N, int Na, int tp,
                                          uint32_t* status) {
    Jacobi<NB> j;
    to_jacobi(s, j, N, Na);
    kepler_step(j, s.m[0], G, dt / 2., N, Na, status);
    com_step(j, dt / 2.);
    to_inertial(s, j, N, Na);
    double ax[NB], ay[NB], az[NB];
    gravity_01(s, ax, ay, az, G, eps2, N, Na, tp);
    interaction_step(j, s, ax, ay, az, G, dt, N, Na);
    kepler_step(j, s.m[0], G, dt / 2., N, Na, status);
    com_step(j, dt / 2.);
    to_inertial(s, j, N, Na);
}

// One WHFast step in democratic heliocentric coordinates with safe_mode = 1 (the
// splitting WHFast512 vectorises, src/integrator_whfast512.c; the step of
// src/integrator_whfast.c:1113-1259 with coordinates = DEMOCRATICHELIOCENTRIC):
// drift, half jump, kick by the planets' mutual forces, half jump, drift.
template <int NB>
__device__ __forceinline__ void step_safe_dh(System<NB>& s, double G, double eps2, double dt, int N, int Na, int tp,
                                             uint32_t* status) {
    Jacobi<NB> h;
    to_dh(s, h, N, Na);
    kepler_step_dh(h, s.m[0], G, dt / 2., N, status);
    com_step(h, dt / 2.);
    jump_step_dh(h, s, dt / 2., N, Na);
    dh_to_inertial(s, h, N, Na);
    double ax[NB], ay[NB], az[NB];
    gravity_01<NB, 1>(s, ax, ay, az, G, eps2, N, Na, tp);
    interaction_step_dh(h, ax, ay, az, dt, N);
    jump_step_dh(h, s, dt / 2., N, Na);
    kepler_step_dh(h, s.m[0], G, dt / 2., N, status);
    com_step(h, dt / 2.);
    dh_to_inertial(s, h, N, Na);
}

// Total energy (src/tools.c:108-162) of one system.
template <int NB>
__device__ __forceinline__ double energy(const System<NB>& s, double G, int N, int Na, int tp) {
    const int Ni = tp == 0 ? Na : N;
    double ek = 0., ep = 0.;
#pragma unroll
    for (int i = 0; i < NB; i++) {
        if (i >= Ni) break;
        ek += 0.5 * s.m[i] * (s.vx[i] * s.vx[i] + s.vy[i] * s.vy[i] + s.vz[i] * s.vz[i]);
    }
#pragma unroll
    for (int i = 0; i < NB; i++) {
        if (i >= Na) break;
#pragma unroll
        for (int jj = i + 1; jj < NB; jj++) {
            if (jj >= Ni) break;
            const double dx = s.x[i] - s.x[jj], dy = s.y[i] - s.y[jj], dz = s.z[i] - s.z[jj];
            ep -= G * s.m[jj] * s.m[i] / sqrt(dx * dx + dy * dy + dz * dz);
        }
    }
    return ek + ep;
}

}  // namespace wh
