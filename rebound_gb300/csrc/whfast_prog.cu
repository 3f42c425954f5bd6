// WHFast programs on an rgpu_sim: the plain one-simulation-per-call path in any
// coordinate system (Jacobi, democratic heliocentric, WHDS, barycentric), with a
// first symplectic corrector of order 3, 5, 7, 11 or 17, the second corrector and
// the kernels DEFAULT, MODIFIEDKICK, COMPOSITION and LAZY
// (src/integrator_whfast.c:653-785, 1113-1259; Wisdom, Holman & Touma 1996;
// Wisdom 2006; Rein, Tamayo & Brown 2019).  The host lays each call out as a list
// of operators in the reference's order; one warp runs the list.  The Kepler
// drifts take one body per lane, the forces one pair and then one body per lane,
// and the coordinate transforms, jumps and kicks one quantity or one body per
// lane; the rest runs on lane 0.  Every operator has a single call
// site in the interpreter loop, so the Kepler solver is inlined once per body
// count however long the corrector is.  Every plain WHFast step and synchronize
// runs here, the default configuration included.  Compiled with
// --fmad=false: bit-identical to the reference's serial build.
#include "whfast_plain.cuh"

namespace {

using namespace wh_plain;

// --- forces over the lanes -------------------------------------------------------
// The reference's serial force loops visit the pairs (i, j) in a fixed order and
// add each pair's terms to both bodies.  In every loop below, a body's sum takes its
// terms in ascending partner order, so the same sums can be formed one body per lane:
// first each pair's displacement and factors are formed once, one pair per lane
// (pair p = hi (hi - 1) / 2 + lo for lo < hi), and each lane then adds its body's
// terms in the reference's order.  Per-body quantities that the serial loop builds
// from running sums (the Jacobi vectors) are formed one body per lane, each lane
// repeating the running sums' additions in the same order.  Every result is
// bit-identical to the serial loop.  One warp runs one simulation, and each FP64 warp
// instruction holds the FP64 pipe for about 64 clocks however few lanes are active, so
// the split divides the step's FP64 instruction count.  All lanes call these
// functions; the caller brackets each call with __syncwarp().  The JACOBI force, the
// jerk and the COMPENSATED force (kernels MODIFIEDKICK and LAZY, gravity
// COMPENSATED) are compiled out of line, apart from the default step's code.

template <int NB>
struct PairTerms {
    static constexpr int kPairs = NB * (NB - 1) / 2;
    double dx[kPairs], dy[kPairs], dz[kPairs], pf[kPairs];   // displacement, G / r^3
    double ex[kPairs], ey[kPairs], ez[kPairs], pf1[kPairs];  // jerk: acceleration difference, 3 alpha G / r^5
};

template <int NB>
struct BodyTerms {
    double qx[NB], qy[NB], qz[NB];            // Jacobi vector of body j
    double ex[NB], ey[NB], ez[NB];            // its acceleration relative to the interior centre of mass
    double fm[NB], fM[NB], f1m[NB], f1M[NB];  // factors with dQ = -m_j and dQ = M
};

// Pair p's indices (lo < hi).
__device__ __forceinline__ void pair_of(int p, int& hi, int& lo) {
    hi = 1;
    while ((hi + 1) * hi / 2 <= p) hi++;
    lo = p - hi * (hi - 1) / 2;
}

// reb_gravity_jacobi_calculate_acceleration (src/gravity.c:108-162): direct terms
// plus the Jacobi terms of the Jacobi Hamiltonian's interaction part; no
// softening, every body treated as active.  Body k takes, in the serial loop's
// order: the pair terms of the partners below it and its own Jacobi term (outer
// index j = k), then for each j > k the Jacobi term of j and the pair term.
template <int NB>
__device__ __noinline__ void gravity_jacobi_lanes(const wh::System<NB>& s, double* ax, double* ay, double* az,
                                     PairTerms<NB>& t, BodyTerms<NB>& b, int lane, double G, int N) {
    if (lane < N && lane > 1) {
        const int j = lane;
        double Rx = 0., Ry = 0., Rz = 0., M = 0.;
#pragma unroll 1
        for (int k = 0; k < j; k++) {
            const double mk = s.m[k];
            Rx += mk * s.x[k]; Ry += mk * s.y[k]; Rz += mk * s.z[k];
            M += mk;
        }
        const double Qx = s.x[j] - Rx / M, Qy = s.y[j] - Ry / M, Qz = s.z[j] - Rz / M;
        const double dr = sqrt(Qx * Qx + Qy * Qy + Qz * Qz);
        const double dr3 = dr * dr * dr;
        b.qx[j] = Qx; b.qy[j] = Qy; b.qz[j] = Qz;
        b.fm[j] = G * (-s.m[j]) / dr3;
        b.fM[j] = G * M / dr3;
    }
    const int npair = N * (N - 1) / 2;
#pragma unroll 1
    for (int p0 = 0; p0 < npair; p0 += 32) {
        const int p = p0 + lane;
        if (p < npair && p > 0) {                   // pair 0 is (0, 1), skipped
            int hi, lo;
            pair_of(p, hi, lo);
            const double dx = s.x[lo] - s.x[hi], dy = s.y[lo] - s.y[hi], dz = s.z[lo] - s.z[hi];
            const double dr = sqrt(dx * dx + dy * dy + dz * dz);
            t.dx[p] = dx; t.dy[p] = dy; t.dz[p] = dz;
            t.pf[p] = G / (dr * dr * dr);
        }
    }
    __syncwarp();
    if (lane >= N) return;
    const int k = lane;
    double sx = 0., sy = 0., sz = 0.;
#pragma unroll 1
    for (int i = 0; i < k; i++) {                   // outer index k: partners below
        if (i == 0 && k == 1) continue;
        const int p = k * (k - 1) / 2 + i;
        const double pfi = t.pf[p] * s.m[i];
        sx += pfi * t.dx[p]; sy += pfi * t.dy[p]; sz += pfi * t.dz[p];
    }
    if (k > 1) {
        const double pf = b.fM[k];
        sx += pf * b.qx[k]; sy += pf * b.qy[k]; sz += pf * b.qz[k];
    }
#pragma unroll 1
    for (int j = k + 1; j < N; j++) {               // outer index j > k
        if (j > 1) {
            const double pf = b.fm[j];
            sx += pf * b.qx[j]; sy += pf * b.qy[j]; sz += pf * b.qz[j];
        }
        if (k == 0 && j == 1) continue;
        const int p = j * (j - 1) / 2 + k;
        const double pfj = t.pf[p] * s.m[j];
        sx -= pfj * t.dx[p]; sy -= pfj * t.dy[p]; sz -= pfj * t.dz[p];
    }
    ax[k] = sx; ay[k] = sy; az[k] = sz;
}

// reb_integrator_whfast_calculate_jerk (src/integrator_whfast.c:786-870): the time
// derivative of the JACOBI accelerations, then a += d * jerk (:1196-1203).  The
// same order as gravity_jacobi_lanes, two updates per term.
template <int NB>
__device__ __noinline__ void add_jerk_lanes(const wh::System<NB>& s, double* ax, double* ay, double* az, PairTerms<NB>& t,
                               BodyTerms<NB>& b, int lane, double G, double d, int N) {
    if (lane < N && lane > 1) {
        const int j = lane;
        double Rx = 0., Ry = 0., Rz = 0., M = 0., Ax = 0., Ay = 0., Az = 0.;
#pragma unroll 1
        for (int k = 0; k < j; k++) {
            const double mk = s.m[k];
            Ax += ax[k] * mk; Ay += ay[k] * mk; Az += az[k] * mk;
            Rx += s.x[k] * mk; Ry += s.y[k] * mk; Rz += s.z[k] * mk;
            M += mk;
        }
        const double Qx = s.x[j] - Rx / M, Qy = s.y[j] - Ry / M, Qz = s.z[j] - Rz / M;
        const double dax = ax[j] - Ax / M, day = ay[j] - Ay / M, daz = az[j] - Az / M;
        const double dr = sqrt(Qx * Qx + Qy * Qy + Qz * Qz);
        const double alpha = dax * Qx + day * Qy + daz * Qz;
        b.qx[j] = Qx; b.qy[j] = Qy; b.qz[j] = Qz;
        b.ex[j] = dax; b.ey[j] = day; b.ez[j] = daz;
        const double fm = G * (-s.m[j]) / (dr * dr * dr);
        const double fM = G * M / (dr * dr * dr);
        b.fm[j] = fm;
        b.fM[j] = fM;
        b.f1m[j] = 3. * alpha * fm / (dr * dr);
        b.f1M[j] = 3. * alpha * fM / (dr * dr);
    }
    const int npair = N * (N - 1) / 2;
#pragma unroll 1
    for (int p0 = 0; p0 < npair; p0 += 32) {
        const int p = p0 + lane;
        if (p < npair && p > 0) {                   // pair 0 is (0, 1), skipped
            int hi, lo;
            pair_of(p, hi, lo);
            const double dx = s.x[hi] - s.x[lo], dy = s.y[hi] - s.y[lo], dz = s.z[hi] - s.z[lo];
            const double ddx = ax[hi] - ax[lo], ddy = ay[hi] - ay[lo], ddz = az[hi] - az[lo];
            const double r = sqrt(dx * dx + dy * dy + dz * dz);
            const double alpha = ddx * dx + ddy * dy + ddz * dz;
            const double pf2 = G / (r * r * r);
            t.dx[p] = dx; t.dy[p] = dy; t.dz[p] = dz;
            t.ex[p] = ddx; t.ey[p] = ddy; t.ez[p] = ddz;
            t.pf[p] = pf2;
            t.pf1[p] = 3. * alpha * pf2 / (r * r);
        }
    }
    __syncwarp();
    const int k = lane < N ? lane : 0;             // lanes beyond N repeat body 0 and write nothing
    double jx = 0., jy = 0., jz = 0.;
#pragma unroll 1
    for (int i = 0; i < k; i++) {                   // outer index k: partners below
        if (i == 0 && k == 1) continue;
        const int p = k * (k - 1) / 2 + i;
        const double pf2i = t.pf[p] * s.m[i];
        jx -= t.ex[p] * pf2i; jy -= t.ey[p] * pf2i; jz -= t.ez[p] * pf2i;
        const double pf1i = t.pf1[p] * s.m[i];
        jx += t.dx[p] * pf1i; jy += t.dy[p] * pf1i; jz += t.dz[p] * pf1i;
    }
    if (k > 1) {
        const double pf2 = b.fM[k], pf1 = b.f1M[k];
        jx += pf2 * b.ex[k]; jy += pf2 * b.ey[k]; jz += pf2 * b.ez[k];
        jx -= pf1 * b.qx[k]; jy -= pf1 * b.qy[k]; jz -= pf1 * b.qz[k];
    }
#pragma unroll 1
    for (int j = k + 1; j < N; j++) {               // outer index j > k
        if (j > 1) {
            const double pf2 = b.fm[j], pf1 = b.f1m[j];
            jx += pf2 * b.ex[j]; jy += pf2 * b.ey[j]; jz += pf2 * b.ez[j];
            jx -= pf1 * b.qx[j]; jy -= pf1 * b.qy[j]; jz -= pf1 * b.qz[j];
        }
        if (k == 0 && j == 1) continue;
        const int p = j * (j - 1) / 2 + k;
        const double pf2j = t.pf[p] * s.m[j];
        jx += t.ex[p] * pf2j; jy += t.ey[p] * pf2j; jz += t.ez[p] * pf2j;
        const double pf1j = t.pf1[p] * s.m[j];
        jx -= t.dx[p] * pf1j; jy -= t.dy[p] * pf1j; jz -= t.dz[p] * pf1j;
    }
    __syncwarp();                                   // every lane has read the accelerations
    if (lane < N) { ax[k] += d * jx; ay[k] += d * jy; az[k] += d * jz; }
}

// --- coordinate systems other than Jacobi (src/transformations.c:295-644) ---------
// coords: 0 Jacobi, 1 democratic heliocentric, 2 WHDS (Hernandez & Dehnen 2017),
// 3 barycentric; the values of REB_INTEGRATOR_WHFAST_COORDINATES.
// Each transform, jump and kick below is the reference's serial loop split over the
// lanes, by quantity (x, y, z, vx, vy, vz: independent running sums) or by body
// (independent per-body updates), every sum kept in the reference's order, so the
// results are bit-identical.  One warp runs one simulation and each FP64 warp
// instruction holds the FP64 pipe for about 64 clocks however many lanes are active,
// so the split divides the instruction count.  All lanes call these functions (some
// hold a __syncwarp()); the caller brackets each call with __syncwarp().

template <class T>
__device__ __forceinline__ auto qrow(T& a, int q) -> decltype(&a.x[0]) {
    return q == 0 ? a.x : q == 1 ? a.y : q == 2 ? a.z : q == 3 ? a.vx : q == 4 ? a.vy : a.vz;
}

// reb_transformations_inertial_to_democraticheliocentric_posvel (:388-425), as
// wh::to_dh: lanes 0-5 one quantity each (every lane forms the same mass sum), lane 0
// also the masses.
template <int NB>
__device__ void to_dh_lanes(const wh::System<NB>& s, wh::Jacobi<NB>& h, int N, int Na, int lane) {
    if (lane >= 6) return;
    const double* sq = qrow(s, lane);
    double* hq = qrow(h, lane);
    double sum = 0., m0 = 0.;
#pragma unroll
    for (int i = 0; i < NB; i++) {
        if (i >= Na) break;
        const double m = s.m[i];
        sum += sq[i] * m;
        m0 += m;
    }
    const double c = sum / m0;
    hq[0] = c;
    // positions relative to the star, velocities relative to the centre of mass
    const double base = lane < 3 ? sq[0] : c;
#pragma unroll
    for (int i = 1; i < NB; i++) {
        if (i >= N) break;
        hq[i] = sq[i] - base;
        if (lane == 0) h.m[i] = s.m[i];
    }
    if (lane == 0) h.m[0] = m0;
}

// reb_transformations_democraticheliocentric_to_inertial_posvel (:427-473), as
// wh::dh_to_inertial: lanes 0-2 the positions (lane 0 also copies the masses), lanes
// 3-5 the velocities, which read the masses from h (the values lane 0 copies).
template <int NB>
__device__ void dh_to_inertial_lanes(wh::System<NB>& s, const wh::Jacobi<NB>& h, int N, int Na, int lane) {
    if (lane >= 6) return;
    const double* hq = qrow(h, lane);
    double* sq = qrow(s, lane);
    if (lane < 3) {
        const double mtot = h.m[0];
        double c = 0.;
#pragma unroll
        for (int i = 1; i < NB; i++) {
            if (i >= Na) break;
            const double m = h.m[i];
            c += hq[i] * m / mtot;
            if (lane == 0) s.m[i] = m;
        }
        const double s0 = hq[0] - c;
        sq[0] = s0;
#pragma unroll
        for (int i = 1; i < NB; i++) {
            if (i >= N) break;
            sq[i] = hq[i] + s0;
        }
    } else {
        const double m0 = s.m[0];
#pragma unroll
        for (int i = 1; i < NB; i++) {
            if (i >= N) break;
            sq[i] = hq[i] + hq[0];
        }
        double c = 0.;
#pragma unroll
        for (int i = 1; i < NB; i++) {
            if (i >= Na) break;
            const double m = h.m[i];
            c += hq[i] * m / m0;
        }
        sq[0] = hq[0] - c;
    }
}

// reb_transformations_inertial_to_whds_posvel (:295-345): democratic heliocentric
// positions and centre of mass, then lane i scales active body i's velocity by
// (m_0 + m_i) / m_0.
template <int NB>
__device__ void to_whds_lanes(const wh::System<NB>& s, wh::Jacobi<NB>& h, int N, int Na, int lane) {
    to_dh_lanes(s, h, N, Na, lane);
    __syncwarp();
    const int i = lane;
    if (i < 1 || i >= Na) return;
    const double m0 = s.m[0];
    const double mf = (m0 + s.m[i]) / m0;
    h.vx[i] = mf * (s.vx[i] - h.vx[0]); h.vy[i] = mf * (s.vy[i] - h.vy[0]); h.vz[i] = mf * (s.vz[i] - h.vz[0]);
}

// reb_transformations_whds_to_inertial_posvel (:347-381): positions and masses as
// democratic heliocentric, then lane i rescales active body i's velocity and lanes 0-2
// form the star's velocity, one component each.
template <int NB>
__device__ void whds_to_inertial_lanes(wh::System<NB>& s, const wh::Jacobi<NB>& h, int N, int Na, int lane) {
    dh_to_inertial_lanes(s, h, N, Na, lane);
    __syncwarp();
    const double m0 = s.m[0];
    if (lane >= 1 && lane < Na) {
        const int i = lane;
        const double mf = (m0 + s.m[i]) / m0;
        s.vx[i] = h.vx[i] / mf + h.vx[0]; s.vy[i] = h.vy[i] / mf + h.vy[0]; s.vz[i] = h.vz[i] / mf + h.vz[0];
    }
    if (lane < 3) {
        const double* hv = qrow(h, 3 + lane);
        double v0 = 0.;
#pragma unroll
        for (int i = 1; i < NB; i++) {
            if (i >= Na) break;
            const double m = s.m[i];
            v0 += hv[i] * m / (m0 + m);
        }
        qrow(s, 3 + lane)[0] = hv[0] - v0;
    }
}

// reb_transformations_inertial_to_barycentric_posvel (:595-644): lanes 0-5 one
// quantity each (every lane forms the same mass sum), lane 0 also the masses.
template <int NB>
__device__ void to_bary_lanes(const wh::System<NB>& s, wh::Jacobi<NB>& b, int N, int Na, int lane) {
    if (lane >= 6) return;
    const double* sq = qrow(s, lane);
    double* bq = qrow(b, lane);
    const double m0 = s.m[0];
    double t = m0 * sq[0], M = m0, sum = 0., sm = 0.;
#pragma unroll
    for (int i = 1; i < NB; i++) {
        if (i >= Na) break;
        const double m = s.m[i];
        sum += sq[i] * m;
        sm += m;
    }
    t += sum;
    M += sm;
    const double mi = 1.0 / M;
    const double c = t * mi;
    bq[0] = c;
    if (lane == 0) b.m[0] = M;
#pragma unroll
    for (int i = 1; i < NB; i++) {
        if (i >= N) break;
        if (lane == 0) b.m[i] = s.m[i];
        bq[i] = sq[i] - c;
    }
}

// reb_transformations_barycentric_to_inertial_posvel (:544-593); it also rebuilds
// the star's mass as the total minus the active bodies'.  Lanes 0-5 one quantity
// each (every lane forms the same mass sum), lane 0 also the masses.
template <int NB>
__device__ void bary_to_inertial_lanes(wh::System<NB>& s, const wh::Jacobi<NB>& b, int N, int Na, int lane) {
    if (lane >= 6) return;
    const double* bq = qrow(b, lane);
    double* sq = qrow(s, lane);
    const double M = b.m[0];
    double t0 = M * bq[0], m0 = M, sum = 0., sm = 0.;
#pragma unroll
    for (int i = 1; i < NB; i++) {
        if (i >= N) break;
        const double v = bq[i] + bq[0];
        sq[i] = v;
        if (i < Na) {
            const double m = b.m[i];
            if (lane == 0) s.m[i] = m;
            sum += v * m;
            sm += m;
        }
    }
    t0 -= sum;
    m0 -= sm;
    const double m0i = 1. / m0;
    if (lane == 0) s.m[0] = m0;
    sq[0] = t0 * m0i;
}

// reb_integrator_whfast_kepler_step (src/integrator_whfast.c:589-636), one body
// per lane: lane i (1 <= i < N) drifts body i.  The bodies' Kepler solves are
// independent; the gravitational parameter of body i is G times the interior
// Jacobi mass (rebuilt by lane i with the serial loop's additions in the same
// order, so it rounds identically), m_0, m_0 + m_i (WHDS, active) or the total
// mass (barycentric).  The caller brackets the call with __syncwarp().
template <int NB>
__device__ void drift_lane(wh::Jacobi<NB>& j, double m0, double G, double dt, int N, int Na, int coords,
                           uint32_t* status) {
    const int i = threadIdx.x;
    if (i < 1 || i >= N) return;
    double e;
    if (coords == 0) {
        e = m0;
#pragma unroll 1
        for (int k = 1; k <= i; k++)
            if (k < Na) e += j.m[k];
    } else if (coords == 2) {
        e = i < Na ? m0 + j.m[i] : m0;
    } else if (coords == 3) {
        e = j.m[0];
    } else {
        e = m0;
    }
    double x = j.x[i], y = j.y[i], z = j.z[i], vx = j.vx[i], vy = j.vy[i], vz = j.vz[i];
    wh::kepler_solver(x, y, z, vx, vy, vz, e * G, dt, status);
    j.x[i] = x; j.y[i] = y; j.z[i] = z; j.vx[i] = vx; j.vy[i] = vy; j.vz[i] = vz;
}

// reb_integrator_whfast_jump_step (:526-584); nothing in Jacobi or barycentric.
// Lanes 0-2, one component each.
template <int NB>
__device__ void jump_lanes(wh::Jacobi<NB>& h, const wh::System<NB>& s, double dt, int N, int Na, int coords,
                           int lane) {
    if ((coords != 1 && coords != 2) || lane >= 3) return;
    const double* v = qrow(h, 3 + lane);
    double* x = qrow(h, lane);
    const double m0 = s.m[0];
    double p = 0.;
    if (coords == 1) {
#pragma unroll 1
        for (int i = 1; i < Na; i++) p += s.m[i] * v[i];
#pragma unroll 1
        for (int i = 1; i < N; i++) x[i] += dt * (p / m0);
        return;
    }
#pragma unroll 1
    for (int i = 1; i < Na; i++) {
        const double m = s.m[i];
        p += m * v[i] / (m0 + m);
    }
#pragma unroll 1
    for (int i = 1; i < N; i++) {
        if (i < Na) {
            const double m = s.m[i];
            x[i] += dt * (p - (m * v[i] / (m0 + m)));
        } else {
            x[i] += dt * p;
        }
    }
}

// reb_integrator_whfast_interaction_step (:431-524) outside Jacobi coordinates: lane i
// kicks body i.
template <int NB>
__device__ void kick_helio_lanes(wh::Jacobi<NB>& h, const wh::System<NB>& s, const double* ax, const double* ay,
                                 const double* az, double G, double dt, int N, int Na, int coords, int lane) {
    const int i = lane;
    if (i < 1 || i >= N) return;
    const double m0 = s.m[0];
    if (coords == 2 && i < Na) {
        const double mi = s.m[i];
        h.vx[i] += dt * (m0 + mi) * ax[i] / m0;
        h.vy[i] += dt * (m0 + mi) * ay[i] / m0;
        h.vz[i] += dt * (m0 + mi) * az[i] / m0;
    } else if (coords == 3) {
        const double dr = sqrt(h.x[i] * h.x[i] + h.y[i] * h.y[i] + h.z[i] * h.z[i]);
        const double pf = G * h.m[0] / (dr * dr * dr);
        h.vx[i] += dt * (pf * h.x[i] + ax[i]);
        h.vy[i] += dt * (pf * h.y[i] + ay[i]);
        h.vz[i] += dt * (pf * h.z[i] + az[i]);
    } else {
        h.vx[i] += dt * ax[i]; h.vy[i] += dt * ay[i]; h.vz[i] += dt * az[i];
    }
}

// BASIC gravity for any gravity_ignore_terms (src/gravity.c:180-257): pairs (i, jj)
// with i from starti (1, or 2 to skip the 0-1 pair) and jj from startj (0, or 1
// to skip body 0) below min(i, Ng); a_i always takes the pair's term, a_jj when i
// is active or testparticle_type is 1.  Bit for bit, over the lanes: the reference
// forms each pair's displacement (from the higher index to the lower) and factor
// G / r^3 once and adds -G m_jj / r^3 d to a_i and G m_i / r^3 d to a_jj, so in its
// serial loop a body's acceleration takes its terms in ascending partner order
// (the partners below it while it is the outer index, then those above it).  Here
// lane l of round r forms pair p = 32 r + l (p = i (i - 1) / 2 + jj) into shared
// memory, and then lane k adds body k's terms in ascending partner order.  One warp
// runs one simulation, so every FP64 warp instruction holds the FP64 pipe for 64
// clocks however many lanes work: N (N - 1) / 2 pairs take one round of square roots
// and divisions up to N = 8.  The state and the accelerations are in shared memory;
// the caller brackets the call with __syncwarp().
template <int NB>
__device__ void gravity_basic_lanes(const wh::System<NB>& s, double* ax, double* ay, double* az, PairTerms<NB>& t,
                                    int lane, double G, double eps2, int N, int Ng, int tp, int starti, int startj) {
    const int npair = N * (N - 1) / 2;
#pragma unroll 1
    for (int p0 = 0; p0 < npair; p0 += 32) {
        const int p = p0 + lane;
        if (p < npair) {
            int i, jj;
            pair_of(p, i, jj);
            const double dx = (0. + s.x[i]) - s.x[jj];
            const double dy = (0. + s.y[i]) - s.y[jj];
            const double dz = (0. + s.z[i]) - s.z[jj];
            const double r = sqrt(dx * dx + dy * dy + dz * dz + eps2);
            t.dx[p] = dx; t.dy[p] = dy; t.dz[p] = dz;
            t.pf[p] = G / (r * r * r);
        }
    }
    __syncwarp();
    if (lane >= N) return;
    const int k = lane;
    const int st = Ng > starti ? Ng : starti;
    double axk = 0., ayk = 0., azk = 0.;
#pragma unroll 1
    for (int q = 0; q < N; q++) {
        if (q == k) continue;
        const bool low = q < k;                  // pair (i = k, jj = q), else (i = q, jj = k)
        const int i = low ? k : q, jj = low ? q : k;
        const int jend = i < Ng ? i : Ng;
        if (i < starti || jj < startj || jj >= jend) continue;
        if (!low && !(i < st ? true : tp != 0)) continue;
        const int p = i * (i - 1) / 2 + jj;
        const double pf = t.pf[p];
        const double c = low ? -pf * s.m[jj] : pf * s.m[i];
        axk += c * t.dx[p]; ayk += c * t.dy[p]; azk += c * t.dz[p];
    }
    ax[k] = axk; ay[k] = ayk; az[k] = azk;
}

// --- Jacobi transforms and kick, one quantity per lane ------------------------------
// The serial transforms carry six independent running sums (x, y, z, vx, vy, vz)
// that share only mass scalars: the running interior mass eta, 1 / eta and the ratio of
// successive etas.  Those form a chain of additions with a division at every link.  Here
// lane i first forms link i's scalars (its eta by the serial chain's additions in the
// same order, then one division that all links share as one warp instruction), and then
// lane q forms quantity q's sum with the reference's operations in the reference's
// order.  The results are bit-identical to the serial loops; one warp runs one
// simulation, so each FP64 warp instruction costs the same however many lanes work, and
// the six sums and the per-body divisions now share instructions.

// Mass scalars of one transform, written by the lanes that form them.
template <int NB>
struct ChainScalars {
    double rcp[NB];      // forward: 1 / eta_(i-1); backward: 1 / eta before removing m_i
    double next[NB];     // forward: eta_i / eta_(i-1); backward: eta after removing m_i
    double total;        // forward: eta over the active bodies
    double total_rcp;    // forward: 1 / total; backward: 1 / eta after removing them all
    double top_rcp;      // backward: 1 / j.m[0] (test particles)
};

// Forward chain of src/transformations.c:34-81 and :147-176: eta_0 = m_0,
// eta_i = eta_(i-1) + m_i for the active bodies 1 <= i < Na.  Lane i (1 <= i < Na)
// forms 1 / eta_(i-1) and eta_i * (1 / eta_(i-1)); lane T = max(Na, 1) forms the total
// and its reciprocal.  Every lane takes part in the division.  All lanes call it.
template <int NB>
__device__ void forward_scalars(const double* m, int Na, ChainScalars<NB>& c, int lane) {
    const int T = Na > 1 ? Na : 1;
    const int l = lane < 1 ? 1 : lane > T ? T : lane;
    double e = m[0];
#pragma unroll 1
    for (int k = 1; k < l; k++) e += m[k];
    const double r = 1. / e;
    if (lane >= 1 && lane < Na) {
        const double e2 = e + m[lane];
        c.rcp[lane] = r;
        c.next[lane] = e2 * r;
    } else if (lane == T) {
        c.total = e;
        c.total_rcp = r;
    }
    __syncwarp();
}

// Backward chain of src/transformations.c:178-226: eta starts at j.m[0] and loses
// m_i for i = Na - 1 down to 1.  Lane i (1 <= i < Na) forms 1 / eta before removing
// m_i and eta after; lane 0 removes them all and forms the final reciprocal.  All
// lanes call it.
template <int NB>
__device__ void backward_scalars(double top, const double* m, int Na, ChainScalars<NB>& c, int lane) {
    const int l = lane < Na ? lane : 0;
    double e = top;
#pragma unroll 1
    for (int k = Na - 1; k > l; k--) e -= m[k];
    const double r = 1. / e;
    if (lane >= 1 && lane < Na) {
        c.rcp[lane] = r;
        c.next[lane] = e - m[lane];
    } else if (lane == 0) {
        c.total_rcp = r;
    }
    __syncwarp();
    // 1 / j.m[0]: lane Na - 1 divided it (nothing removed yet), or lane 0 when Na <= 1
    if (lane == 0) c.top_rcp = Na >= 2 ? c.rcp[Na - 1] : c.total_rcp;
    __syncwarp();
}

// reb_transformations_inertial_to_jacobi_posvel (src/transformations.c:34-81), as
// wh::to_jacobi; lanes 0-5 form the sums, lane 0 also copies the masses.
template <int NB>
__device__ void to_jacobi_lanes(const wh::System<NB>& s, wh::Jacobi<NB>& j, ChainScalars<NB>& c, int N, int Na,
                                int lane) {
    forward_scalars(s.m, Na, c, lane);
    if (lane >= 6) return;
    const double* sq = qrow(s, lane);
    double* jq = qrow(j, lane);
    double acc = s.m[0] * sq[0];
#pragma unroll
    for (int i = 1; i < NB; i++) {
        if (i >= Na) break;
        const double v = sq[i] - acc * c.rcp[i];
        jq[i] = v;
        acc = acc * c.next[i] + s.m[i] * v;
        if (lane == 0) j.m[i] = s.m[i];
    }
    const double ei = c.total_rcp;
#pragma unroll
    for (int i = 1; i < NB; i++) {
        if (i < Na || i >= N) continue;
        jq[i] = sq[i] - acc * ei;
        if (lane == 0) j.m[i] = s.m[i];
    }
    jq[0] = acc * ei;
    if (lane == 0) j.m[0] = c.total;
}

// reb_transformations_jacobi_to_inertial_posvel (src/transformations.c:178-226), as
// wh::to_inertial; lanes 0-5 form the sums (the masses are not written).
template <int NB>
__device__ void to_inertial_lanes(wh::System<NB>& s, const wh::Jacobi<NB>& j, ChainScalars<NB>& c, int N, int Na,
                                  int lane) {
    backward_scalars(j.m[0], s.m, Na, c, lane);
    if (lane >= 6) return;
    const double* jq = qrow(j, lane);
    double* sq = qrow(s, lane);
    double acc = jq[0] * j.m[0];
    const double tpi = c.top_rcp;
#pragma unroll
    for (int i = NB - 1; i >= 1; i--) {
        if (i >= N || i < Na) continue;
        sq[i] = jq[i] + acc * tpi;
    }
#pragma unroll
    for (int i = NB - 1; i >= 1; i--) {
        if (i >= Na) continue;
        acc = (acc - s.m[i] * jq[i]) * c.rcp[i];
        sq[i] = jq[i] + acc;
        acc *= c.next[i];
    }
    sq[0] = acc * c.total_rcp;
}

// Interaction (kick) step in Jacobi coordinates, as wh::interaction_step:
// inertial_to_jacobi_acc (src/transformations.c:147-176) and the velocity kick on
// lanes 0-2 (one component each), then the Jacobi term (src/integrator_whfast.c:
// 447-472) on lane i for body i >= 2, after the kick as in the serial loop.  Lane i
// rebuilds its interior mass with the serial loop's additions in the same order.
// All lanes call it; the caller brackets the call with __syncwarp().
template <int NB>
__device__ void kick_jacobi_lanes(wh::Jacobi<NB>& j, const wh::System<NB>& s, const double* const acc[3],
                                  ChainScalars<NB>& c, double G, double dt, int N, int Na, bool jacobi_term,
                                  int lane) {
    forward_scalars(s.m, Na, c, lane);
    if (lane < 3) {
        const double* a = acc[lane];
        double* v = lane == 0 ? j.vx : lane == 1 ? j.vy : j.vz;
        double ja[NB];
        double sc = s.m[0] * a[0];
#pragma unroll
        for (int i = 1; i < NB; i++) {
            if (i >= Na) break;
            ja[i] = a[i] - sc * c.rcp[i];
            sc = sc * c.next[i] + s.m[i] * ja[i];
        }
#pragma unroll
        for (int i = 1; i < NB; i++) {
            if (i < Na || i >= N) continue;
            ja[i] = a[i] - sc * c.total_rcp;
        }
#pragma unroll
        for (int i = 1; i < NB; i++) {
            if (i >= N) break;
            v[i] += dt * ja[i];
        }
    }
    __syncwarp();
    if (!jacobi_term || lane < 2 || lane >= N) return;
    const int i = lane;
    double eta = s.m[0];
#pragma unroll 1
    for (int k = 1; k <= i; k++)
        if (k < Na) eta += j.m[k];
    const double qx = j.x[i], qy = j.y[i], qz = j.z[i];
    const double rj2i = WH_RCP(qx * qx + qy * qy + qz * qz);
    const double rji = WH_SQRT(rj2i);
    const double rj3iM = rji * rj2i * G * eta;
    const double pf = dt * rj3iM;
    j.vx[i] += pf * qx;
    j.vy[i] += pf * qy;
    j.vz[i] += pf * qz;
}

// Compensated (Kahan) accumulation of one force term (src/gravity.c:431-446).
__device__ __forceinline__ void kahan_add(double& a, double& c, double inc) {
    const double y = inc - c;
    const double t = a + y;
    c = (t - a) - y;
    a = t;
}

// reb_gravity_compensated_calculate_acceleration, serial branch (src/gravity.c:
// 284-297, 415-531): pairs i < j among the active bodies, then test particles,
// each term added with a Kahan correction; ign = gravity_ignore_terms.  Over the
// lanes: an active body takes its active partners' terms in ascending order and then,
// with testparticle_type 1, the test particles' in ascending order; a test particle
// takes the active bodies' in ascending order.  Each pair's displacement (outer index
// minus inner: lower minus higher between active bodies, test particle minus active
// body) and G / (r^2 r) are formed once, one pair per lane.
template <int NB>
__device__ __noinline__ void gravity_compensated_lanes(const wh::System<NB>& s, double* ax, double* ay, double* az,
                                          PairTerms<NB>& t, int lane, double G, double eps2, int N, int Ng,
                                          int tp, int ign) {
    const int npair = N * (N - 1) / 2;
#pragma unroll 1
    for (int p0 = 0; p0 < npair; p0 += 32) {
        const int p = p0 + lane;
        if (p < npair) {
            int hi, lo;
            pair_of(p, hi, lo);
            if (lo < Ng) {                          // pairs of two test particles do not interact
                const int i = hi < Ng ? lo : hi, j = hi < Ng ? hi : lo;
                const double dx = s.x[i] - s.x[j], dy = s.y[i] - s.y[j], dz = s.z[i] - s.z[j];
                const double r2 = dx * dx + dy * dy + dz * dz + eps2;
                const double r = sqrt(r2);
                t.dx[p] = dx; t.dy[p] = dy; t.dz[p] = dz;
                t.pf[p] = G / (r2 * r);
            }
        }
    }
    __syncwarp();
    if (lane >= N) return;
    const int k = lane;
    const bool active = k < Ng;
    double sx = 0., sy = 0., sz = 0., cx = 0., cy = 0., cz = 0.;
#pragma unroll 1
    for (int q = 0; q < N; q++) {
        if (q == k) continue;
        if (ign == 1 && ((k == 0 && q == 1) || (k == 1 && q == 0))) continue;
        if (ign == 2 && (k == 0 || q == 0)) continue;
        const int hi = q > k ? q : k, lo = q > k ? k : q;
        const int p = hi * (hi - 1) / 2 + lo;
        double c;                                   // the term's factor (pfj or pfi of the serial loop)
        if (active && q < Ng) {
            c = q > k ? -t.pf[p] * s.m[q] : t.pf[p] * s.m[q];   // k is the outer index when q > k
        } else if (active) {
            if (!tp) continue;                      // test particle q kicks k only with testparticle_type 1
            c = t.pf[p] * s.m[q];
        } else {
            if (q >= Ng) continue;
            c = -t.pf[p] * s.m[q];
        }
        kahan_add(sx, cx, c * t.dx[p]); kahan_add(sy, cy, c * t.dy[p]); kahan_add(sz, cz, c * t.dz[p]);
    }
    ax[k] = sx; ay[k] = sy; az[k] = sz;
}

template <int NB>
__global__ void __launch_bounds__(32) whfast_program(ParticlesSoA p, double* jac, size_t cap, int N, int Na, int Ng,
                                                     int tp, int coords, double G, double eps2,
                                                     const __grid_constant__ Program prog, uint32_t* status) {
    // Every lane walks the program; the drifts (one body each), the forces (one
    // pair, then one body each), the coordinate transforms, jumps and kicks (one
    // quantity or one body each) run on the lanes, the centre-of-mass drift, the
    // zero force and the lazy shift on lane 0.  The state lives in shared memory so
    // that all lanes see it.
    __shared__ wh::Jacobi<NB> j;
    __shared__ wh::System<NB> s;
    __shared__ double acc[3][NB];
    __shared__ ChainScalars<NB> chain;
    __shared__ PairTerms<NB> pairs;
    __shared__ BodyTerms<NB> bodies;
    __shared__ int stop;
    const int lane = threadIdx.x;
    double* const ax = acc[0];
    double* const ay = acc[1];
    double* const az = acc[2];
    if (lane == 0) {
        stop = 0;
        load_sys(s, p, N);
        load_jac(j, jac, cap, N);
#pragma unroll
        for (int i = 0; i < NB; i++) {
            const bool on = i < N;
            ax[i] = on ? p.ax[i] : 0.; ay[i] = on ? p.ay[i] : 0.; az[i] = on ? p.az[i] : 0.;
        }
    }
    __syncwarp();
    const double m0 = p.m[0];                       // the star's mass as the drift reads it
    // gravity_ignore_terms of each coordinate system (:929-938)
    const int starti = coords == 3 ? 1 : 2;
    const int startj = (coords == 1 || coords == 2) ? 1 : 0;
#pragma unroll 1
    for (int k = 0; k < prog.n; k++) {
        const double d = prog.d[k];
        const int op = prog.op[k];
        if (op == kOpDrift) {
            drift_lane(j, m0, G, d, N, Na, coords, status);
            __syncwarp();
            continue;
        }
        if (op == kOpGravity || op == kOpGravityJacobi || op == kOpGravityCompensated || op == kOpJerk) {
            if (op == kOpGravity) {
                gravity_basic_lanes(s, ax, ay, az, pairs, lane, G, eps2, N, Ng, tp, starti, startj);
            } else if (op == kOpGravityJacobi) {
                gravity_jacobi_lanes(s, ax, ay, az, pairs, bodies, lane, G, N);
            } else if (op == kOpGravityCompensated) {
                gravity_compensated_lanes(s, ax, ay, az, pairs, lane, G, eps2, N, Ng, tp,
                                          coords == 0 ? 1 : coords == 3 ? 0 : 2);
            } else {
                add_jerk_lanes(s, ax, ay, az, pairs, bodies, lane, G, d, N);
            }
            __syncwarp();
            continue;
        }
        if (op == kOpFromInertial || op == kOpToInertial || op == kOpKick || op == kOpKickNoJacobiTerm ||
            op == kOpJump) {
            if (op == kOpFromInertial) {
                if (coords == 0) to_jacobi_lanes(s, j, chain, N, Na, lane);
                else if (coords == 1) to_dh_lanes(s, j, N, Na, lane);
                else if (coords == 2) to_whds_lanes(s, j, N, Na, lane);
                else to_bary_lanes(s, j, N, Na, lane);
            } else if (op == kOpToInertial) {
                if (coords == 0) to_inertial_lanes(s, j, chain, N, Na, lane);
                else if (coords == 1) dh_to_inertial_lanes(s, j, N, Na, lane);
                else if (coords == 2) whds_to_inertial_lanes(s, j, N, Na, lane);
                else bary_to_inertial_lanes(s, j, N, Na, lane);
            } else if (op == kOpJump) {
                jump_lanes(j, s, d, N, Na, coords, lane);
            } else if (coords == 0) {
                const double* const a3[3] = {ax, ay, az};
                kick_jacobi_lanes(j, s, a3, chain, G, d, N, Na, op == kOpKick, lane);
            } else {
                kick_helio_lanes(j, s, ax, ay, az, G, d, N, Na, coords, lane);
            }
            __syncwarp();
            continue;
        }
        if (lane == 0) {
            switch (op) {
                case kOpCom: wh::com_step(j, d); break;
                case kOpGravityNone:
#pragma unroll 1
                    for (int i = 0; i < N; i++) { ax[i] = 0.; ay[i] = 0.; az[i] = 0.; }
                    break;
                case kOpLazyShift:
#pragma unroll 1
                    for (int i = 1; i < N; i++) {
                        s.x[i] += d * ax[i]; s.y[i] += d * ay[i]; s.z[i] += d * az[i];
                    }
                    break;
                default: atomicOr(status, DEV_ERR_PROGRAM); stop = 1; break;
            }
        }
        __syncwarp();
        if (stop) return;
    }
    if (lane != 0) return;
    store_pos_vel(s, p, N);
    store_jac(j, jac, cap, N);
#pragma unroll
    for (int i = 0; i < NB; i++) {
        if (i >= N) break;
        p.ax[i] = ax[i]; p.ay[i] = ay[i]; p.az[i] = az[i];
        p.m[i] = s.m[i];                      // the barycentric transform rebuilds the star's mass
    }
}

typedef void (*ProgKernel)(ParticlesSoA, double*, size_t, int, int, int, int, int, double, double,
                           const Program, uint32_t*);

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
    k<<<1, 32, 0, s->stream>>>(s->p, s->wh->jac, s->cap, N, wh_active(s), (int)n_active(s), c.testparticle_type,
                               c.whfast_coordinates, c.G, c.softening * c.softening, prog, s->d_status);
    ktimer_end(s);
    g_launches++;
    RGPU_CUDA(s, cudaGetLastError());
    return RGPU_OK;
}
