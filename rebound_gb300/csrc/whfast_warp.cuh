// Warp-per-system WHFast (safe_mode 1, Jacobi coordinates, DEFAULT kernel):
// lane i of a warp holds body i, so the Kepler drifts of all bodies and each
// body's row of pair forces run side by side, and the Jacobi transforms become
// mass-weighted prefix / suffix sums across lanes.  With C_i the centre of mass
// of bodies 0..i-1, eta_i their mass and X the centre of mass of all bodies:
//     q_i = x_i - C_i,    x_i = q_i + X - sum_{k >= i} (m_k / eta_{k+1}) q_k,
// the closed forms of the recurrences of src/transformations.c:34-81 and :178-226
// (summed in tree order here, so results agree with the serial form to rounding).
// Used by the serving loop's WHFast slots and by the ensemble's warp mapping, with
// the division and square root of the including unit (WH_DIV / WH_SQRT).
#pragma once
#include "whfast_core.cuh"

namespace whw {

constexpr unsigned kFull = 0xffffffffu;

template <int NB>
__device__ __forceinline__ double lane_prefix(double v, int lane) {     // inclusive, lanes >= NB hold 0
#pragma unroll
    for (int d = 1; d < NB; d <<= 1) {
        const double t = __shfl_up_sync(kFull, v, d);
        if (lane >= d) v += t;
    }
    return v;
}

template <int NB>
__device__ __forceinline__ double lane_suffix(double v, int lane) {     // inclusive, lanes >= NB hold 0
#pragma unroll
    for (int d = 1; d < NB; d <<= 1) {
        const double t = __shfl_down_sync(kFull, v, d);
        if (lane + d < 32) v += t;
    }
    return v;
}

template <int NB>
__device__ __forceinline__ double lane_exclusive(double v, int lane) {  // sum over lanes < lane
    const double e = __shfl_up_sync(kFull, lane_prefix<NB>(v, lane), 1);
    return lane == 0 ? 0. : e;
}

// Q inclusive prefix (SUFFIX: suffix) sums over the NB bodies at once.  Lanes are
// regrouped so that lane L holds quantity L / NB of body L % NB, 32 / NB quantities
// per pass, and each pass scans its groups of NB lanes together: every FP64
// addition of the scan then serves several quantities (one warp instruction holds
// the FP64 pipe for 64 clocks whatever the active lanes).  On return, lane b < NB
// holds body b's sums; other lanes hold values nothing reads.
template <int NB, int Q, bool SUFFIX>
__device__ __forceinline__ void lane_scan_multi(double (&v)[Q], int lane) {
    constexpr int PER = 32 / NB;
    const int qi = lane / NB, b = lane % NB;
#pragma unroll
    for (int q0 = 0; q0 < Q; q0 += PER) {
        double t = 0.;
#pragma unroll
        for (int q = 0; q < PER; q++) {
            if (q0 + q >= Q) break;
            const double u = __shfl_sync(kFull, v[q0 + q], b);
            if (qi == q) t = u;
        }
#pragma unroll
        for (int d = 1; d < NB; d <<= 1) {
            const double w = SUFFIX ? __shfl_down_sync(kFull, t, d) : __shfl_up_sync(kFull, t, d);
            if (SUFFIX ? (b + d < NB) : (b >= d)) t += w;
        }
#pragma unroll
        for (int q = 0; q < PER; q++) {
            if (q0 + q >= Q) break;
            v[q0 + q] = __shfl_sync(kFull, t, q * NB + b);
        }
    }
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Advance one system of a [field][body][system] table (`cap` systems per field
// row) by up to `nsteps` steps of length h; called by a whole warp.
// The steps run in blocks of `block` steps, the first one `first` steps long
// when first > 0, and the call's last step always closes a block.  Within a block
// the system stays in Jacobi coordinates and the closing half drift of one step
// and the opening half drift of the next are one Kepler drift over h, as the
// reference's WHFast does with safe_mode = 0 (src/integrator_whfast.c:1113-1259);
// each block ends synchronised (inertial positions and velocities), as every
// safe_mode = 1 step does.  The two splittings are the same map and differ by
// rounding; block = 1 is the reference's default.  With budget_ns > 0 the warp
// also stops after the first block that ends budget_ns or more after it started
// (lane 0's clock decides for the whole warp), so the blocks do not depend on the
// budget.  Returns the steps taken.
template <int NB>
__device__ __forceinline__ int warp_steps(double* __restrict__ st, int cap, int sid, int nsteps, double h, double G,
                                          uint32_t* status, long long budget_ns = 0, int block = 1,
                                          int first = 0) {
    const int lane = (int)(threadIdx.x & 31);
    const size_t f = (size_t)NB * cap;
    const bool on = lane < NB;
    const size_t o = (size_t)(on ? lane : 0) * cap + sid;
    double x = 0., y = 0., z = 0., vx = 0., vy = 0., vz = 0., m = 0.;
    if (on) {
        x = st[o]; y = st[f + o]; z = st[2 * f + o];
        vx = st[3 * f + o]; vy = st[4 * f + o]; vz = st[5 * f + o]; m = st[6 * f + o];
    }
    const double h2 = h / 2.;
    // masses are constant over a request: the prefix masses once
    const double eta_in = lane_prefix<NB>(m, lane);                  // sum_{k <= i} m_k
    const double up = __shfl_up_sync(kFull, eta_in, 1);                // every lane takes part in the shuffle
    const double eta_ex = lane == 0 ? 0. : up;
    const double Mi = 1. / __shfl_sync(kFull, eta_in, NB - 1);
    const bool jac = on && lane > 0;                                 // lanes holding a Jacobi body
    const double ei = jac ? 1. / eta_ex : 0.;
    const double wf = jac ? m / eta_in : 0.;
    const double mu = G * eta_in;
    double mj[NB];
#pragma unroll
    for (int j = 0; j < NB; j++) mj[j] = __shfl_sync(kFull, m, j);
    // Pair forces are spread over the lanes: lane l of round r holds the pair
    // p = 32 r + l (bodies pi < pj, in row order).  A lone warp is bound by FP64
    // warp instructions (each holds the pipe for 64 clocks whatever the active
    // lanes), so one square root and division per pair across 32 lanes beats one
    // row per lane.
    constexpr int kPairs = NB * (NB - 1) / 2;
    constexpr int kRounds = (kPairs + 31) / 32;
    int pi[kRounds], pj[kRounds];
#pragma unroll
    for (int r = 0; r < kRounds; r++) {
        int q = 32 * r + lane, a = 0;
        while (a < NB - 1 && q >= NB - 1 - a) { q -= NB - 1 - a; a++; }
        pi[r] = a;
        pj[r] = a + 1 + q;                        // >= NB for lanes past the last pair
    }
    const unsigned long long t_start = budget_ns > 0 ? global_ns() : 0ull;
    int done = 0;
    double qx = 0., qy = 0., qz = 0., ux = 0., uy = 0., uz = 0.;
    int left = first > 0 ? first : block;          // steps left in the current block
    bool opens = true;                             // this step opens a block
    for (int k = 0; k < nsteps; k++) {
        left--;
        const bool closes = left <= 0 || k + 1 == nsteps;
        if (opens) {
        // inertial -> Jacobi (lane 0: centre of mass)
        {
            double P[6] = {m * x, m * y, m * z, m * vx, m * vy, m * vz};
            lane_scan_multi<NB, 6, false>(P, lane);
            const double Px = P[0], Py = P[1], Pz = P[2], Pvx = P[3], Pvy = P[4], Pvz = P[5];
            const double Ex = __shfl_up_sync(kFull, Px, 1), Ey = __shfl_up_sync(kFull, Py, 1),
                         Ez = __shfl_up_sync(kFull, Pz, 1);
            const double Evx = __shfl_up_sync(kFull, Pvx, 1), Evy = __shfl_up_sync(kFull, Pvy, 1),
                         Evz = __shfl_up_sync(kFull, Pvz, 1);
            const double Tx = __shfl_sync(kFull, Px, NB - 1), Ty = __shfl_sync(kFull, Py, NB - 1),
                         Tz = __shfl_sync(kFull, Pz, NB - 1);
            const double Tvx = __shfl_sync(kFull, Pvx, NB - 1), Tvy = __shfl_sync(kFull, Pvy, NB - 1),
                         Tvz = __shfl_sync(kFull, Pvz, NB - 1);
            if (lane == 0) {
                qx = Tx * Mi; qy = Ty * Mi; qz = Tz * Mi; ux = Tvx * Mi; uy = Tvy * Mi; uz = Tvz * Mi;
            } else {
                qx = x - Ex * ei; qy = y - Ey * ei; qz = z - Ez * ei;
                ux = vx - Evx * ei; uy = vy - Evy * ei; uz = vz - Evz * ei;
            }
        }
        // drift dt/2: Kepler per Jacobi body, free drift of the centre of mass
        if (jac) wh::kepler_solver(qx, qy, qz, ux, uy, uz, mu, h2, status);
        else if (lane == 0) { qx += h2 * ux; qy += h2 * uy; qz += h2 * uz; }
        }
        // Jacobi -> inertial positions
        {
            const double Xc = __shfl_sync(kFull, qx, 0), Yc = __shfl_sync(kFull, qy, 0), Zc = __shfl_sync(kFull, qz, 0);
            double W[3] = {wf * qx, wf * qy, wf * qz};
            lane_scan_multi<NB, 3, true>(W, lane);
            const double Wx = W[0], Wy = W[1], Wz = W[2];
            x = (jac ? qx : 0.) + Xc - Wx; y = (jac ? qy : 0.) + Yc - Wy; z = (jac ? qz : 0.) + Zc - Wz;
        }
        // inertial accelerations, all pairs except (0, 1), no softening (src/gravity.c:195-257):
        // G (x_i - x_j) / r^3 once per pair, then each body sums its partners' terms in order
        double gx[kRounds], gy[kRounds], gz[kRounds];
#pragma unroll
        for (int r = 0; r < kRounds; r++) {
            const int a = pi[r], b = pj[r] < NB ? pj[r] : a;
            const double dx = __shfl_sync(kFull, x, a) - __shfl_sync(kFull, x, b);
            const double dy = __shfl_sync(kFull, y, a) - __shfl_sync(kFull, y, b);
            const double dz = __shfl_sync(kFull, z, a) - __shfl_sync(kFull, z, b);
            double g = 0.;
            if (pj[r] < NB) {
                const double rr = WH_SQRT(dx * dx + dy * dy + dz * dz);
                g = WH_DIV(G, rr * rr * rr);
            }
            gx[r] = g * dx; gy[r] = g * dy; gz[r] = g * dz;
        }
        double ax = 0., ay = 0., az = 0.;
#pragma unroll
        for (int q = 0; q < NB; q++) {
            // partner q: its pair's term sits at row-order index p (round p / 32,
            // lane p % 32) and enters with -m_q for the pair's first body, +m_q
            // for the second
            const int a = lane < q ? lane : q, b = lane < q ? q : lane;
            const int p = a * (NB - 1) - a * (a - 1) / 2 + (b - a - 1);
            const double sgm = (lane == q || !on || (a == 0 && b == 1)) ? 0. : (lane < q ? -mj[q] : mj[q]);
            double tx = 0., ty = 0., tz = 0.;
#pragma unroll
            for (int r = 0; r < kRounds; r++) {
                const int sl = p - 32 * r;
                const double vx_ = __shfl_sync(kFull, gx[r], sl & 31), vy_ = __shfl_sync(kFull, gy[r], sl & 31),
                             vz_ = __shfl_sync(kFull, gz[r], sl & 31);
                if (sl >= 0 && sl < 32) { tx = vx_; ty = vy_; tz = vz_; }
            }
            ax += sgm * tx; ay += sgm * ty; az += sgm * tz;
        }
        // kick in Jacobi coordinates (src/transformations.c:147-176, src/integrator_whfast.c:447-472)
        {
            double S[3] = {m * ax, m * ay, m * az};
            lane_scan_multi<NB, 3, false>(S, lane);
            const double ex = __shfl_up_sync(kFull, S[0], 1), ey = __shfl_up_sync(kFull, S[1], 1),
                         ez = __shfl_up_sync(kFull, S[2], 1);
            const double Sx = lane == 0 ? 0. : ex, Sy = lane == 0 ? 0. : ey, Sz = lane == 0 ? 0. : ez;
            if (jac) {
                ux += h * (ax - Sx * ei); uy += h * (ay - Sy * ei); uz += h * (az - Sz * ei);
                if (lane > 1) {
                    const double rj2i = WH_RCP(qx * qx + qy * qy + qz * qz);
                    const double pf = h * (WH_SQRT(rj2i) * rj2i * G * eta_in);
                    ux += pf * qx; uy += pf * qy; uz += pf * qz;
                }
            }
        }
        opens = closes;
        if (!closes) {
            // this step's closing half drift and the next step's opening one
            if (jac) wh::kepler_solver(qx, qy, qz, ux, uy, uz, mu, h, status);
            else if (lane == 0) { qx += h * ux; qy += h * uy; qz += h * uz; }
            continue;
        }
        left = block;
        // drift dt/2
        if (jac) wh::kepler_solver(qx, qy, qz, ux, uy, uz, mu, h2, status);
        else if (lane == 0) { qx += h2 * ux; qy += h2 * uy; qz += h2 * uz; }
        // Jacobi -> inertial positions and velocities
        {
            const double Xc = __shfl_sync(kFull, qx, 0), Yc = __shfl_sync(kFull, qy, 0), Zc = __shfl_sync(kFull, qz, 0);
            const double Vx = __shfl_sync(kFull, ux, 0), Vy = __shfl_sync(kFull, uy, 0), Vz = __shfl_sync(kFull, uz, 0);
            double W[6] = {wf * qx, wf * qy, wf * qz, wf * ux, wf * uy, wf * uz};
            lane_scan_multi<NB, 6, true>(W, lane);
            const double Wx = W[0], Wy = W[1], Wz = W[2], Wvx = W[3], Wvy = W[4], Wvz = W[5];
            x = (jac ? qx : 0.) + Xc - Wx; y = (jac ? qy : 0.) + Yc - Wy; z = (jac ? qz : 0.) + Zc - Wz;
            vx = (jac ? ux : 0.) + Vx - Wvx; vy = (jac ? uy : 0.) + Vy - Wvy; vz = (jac ? uz : 0.) + Vz - Wvz;
        }
        if (!on) { x = y = z = vx = vy = vz = 0.; }
        done = k + 1;
        if (budget_ns > 0) {
            const long long el = (long long)(global_ns() - t_start);
            if (__shfl_sync(kFull, el, 0) >= budget_ns) break;
        }
    }
    if (on) {
        st[o] = x; st[f + o] = y; st[2 * f + o] = z;
        st[3 * f + o] = vx; st[4 * f + o] = vy; st[5 * f + o] = vz;
    }
    return done;
}

}  // namespace whw
