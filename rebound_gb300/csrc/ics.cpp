// Seeded synthetic workloads with the shapes of the reference's benchmark
// configurations, drawn with the reference's random-number conventions
// (glibc rand_r streams, src/tools.c:64-105).  Host code.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>
#include "../../include/rebound_gb300.h"

namespace {

struct Rng {
    unsigned int seed;
    // reb_random_uniform (src/tools.c:64-75)
    double uniform(double lo, double hi) { return ((double)rand_r(&seed)) / ((double)RAND_MAX) * (hi - lo) + lo; }
    // reb_random_powerlaw (src/tools.c:78-82)
    double powerlaw(double lo, double hi, double slope) {
        const double y = uniform(0., 1.);
        if (slope == -1) return exp(y * log(hi / lo) + log(lo));
        return pow((pow(hi, slope + 1.) - pow(lo, slope + 1.)) * y + pow(lo, slope + 1.), 1. / (slope + 1.));
    }
    // reb_random_normal (src/tools.c:84-100); the argument is the variance.
    double normal(double variance) {
        double v1 = 0., v2 = 0., rsq = 1.;
        while (rsq >= 1. || rsq < 1.0e-12) {
            v1 = 2. * ((double)rand_r(&seed)) / ((double)RAND_MAX) - 1.0;
            v2 = 2. * ((double)rand_r(&seed)) / ((double)RAND_MAX) - 1.0;
            rsq = v1 * v1 + v2 * v2;
        }
        return v1 * sqrt(-2. * log(rsq) / rsq * variance);
    }
    // reb_random_rayleigh (src/tools.c:102-105)
    double rayleigh(double sigma) { return sigma * sqrt(-2 * log(uniform(0., 1.))); }
};

inline double* rec(void* out, size_t stride, size_t i) { return (double*)((char*)out + i * stride); }

void put(double* r, double x, double y, double z, double vx, double vy, double vz, double m, double rad) {
    r[0] = x; r[1] = y; r[2] = z; r[3] = vx; r[4] = vy; r[5] = vz;
    r[6] = r[7] = r[8] = 0.; r[9] = m; r[10] = rad;
}

}  // namespace

extern "C" {

// Plummer sphere by the Aarseth, Henon & Wielen (1974) rejection method as in
// reb_simulation_add_plummer (src/tools.c:463-502), keeping in draw order only
// particles with r <= rmax, equal masses M/N.
int rgpu_ic_plummer(unsigned int seed, size_t N, double M, double R, double rmax, void* out, size_t stride) {
    if (!out || stride < 88) return RGPU_ERR_ARG;
    Rng g{seed};
    const double E = 3. / 64. * M_PI * M * M / R;
    size_t n = 0;
    while (n < N) {
        const double rr = pow(pow(g.uniform(0, 1), -2. / 3.) - 1., -1. / 2.);
        const double x2 = g.uniform(0, 1);
        const double x3 = g.uniform(0, 2. * M_PI);
        double z = (1. - 2. * x2) * rr;
        double x = sqrt(rr * rr - z * z) * cos(x3);
        double y = sqrt(rr * rr - z * z) * sin(x3);
        double x5, gg, q;
        do {
            x5 = g.uniform(0., 1.);
            q = g.uniform(0., 1.);
            gg = q * q * pow(1. - q * q, 7. / 2.);
        } while (0.1 * x5 > gg);
        const double ve = pow(2., 1. / 2.) * pow(1. + rr * rr, -1. / 4.);
        const double v = q * ve;
        const double x6 = g.uniform(0., 1.);
        const double x7 = g.uniform(0., 2. * M_PI);
        double vz = (1. - 2. * x6) * v;
        double vx = sqrt(v * v - vz * vz) * cos(x7);
        double vy = sqrt(v * v - vz * vz) * sin(x7);
        x *= 3. * M_PI / 64. * M * M / E;
        y *= 3. * M_PI / 64. * M * M / E;
        z *= 3. * M_PI / 64. * M * M / E;
        vx *= sqrt(E * 64. / 3. / M_PI / M);
        vy *= sqrt(E * 64. / 3. / M_PI / M);
        vz *= sqrt(E * 64. / 3. / M_PI / M);
        if (sqrt(x * x + y * y + z * z) > rmax) continue;
        put(rec(out, stride, n), x, y, z, vx, vy, vz, M / (double)N, 0.);
        n++;
    }
    return RGPU_OK;
}

// Planetary-ring patch in a shearing sheet: radii dN/dr ~ r^-3 on [rmin, rmax],
// x, y uniform in the box, z ~ N(0, sigma_z^2) redrawn until |z| < Lz/2,
// v = Keplerian shear -1.5*OMEGA*x plus N(0, sigma_v^2) per component, until
// the total mass reaches surface_density * Lx * Ly.  Returns the count in *n_out
// (at most cap records are written; RGPU_ERR_OVERFLOW if more were needed).
int rgpu_ic_ring_patch(unsigned int seed, double Lx, double Ly, double Lz, double OMEGA, double surface_density,
                       double particle_density, double rmin, double rmax, double sigma_z, double sigma_v,
                       void* out, size_t stride, size_t cap, size_t* n_out) {
    if (!n_out || stride < 88) return RGPU_ERR_ARG;
    Rng g{seed};
    double total = 0.;
    size_t n = 0;
    while (total < surface_density * Lx * Ly) {
        const double rad = g.powerlaw(rmin, rmax, -3.);
        const double x = g.uniform(-Lx / 2., Lx / 2.);
        const double y = g.uniform(-Ly / 2., Ly / 2.);
        double z;
        do { z = g.normal(sigma_z * sigma_z); } while (!(fabs(z) < Lz / 2.));
        const double vx = g.normal(sigma_v * sigma_v);
        const double vy = -1.5 * x * OMEGA + g.normal(sigma_v * sigma_v);
        const double vz = g.normal(sigma_v * sigma_v);
        const double m = particle_density * 4. / 3. * M_PI * rad * rad * rad;
        if (out && n < cap) put(rec(out, stride, n), x, y, z, vx, vy, vz, m, rad);
        n++;
        total += m;
    }
    *n_out = n;
    return (out && n > cap) ? RGPU_ERR_OVERFLOW : RGPU_OK;
}

// One planetary system: star of mass 1 plus k planets, m log-uniform in
// [mmin, mmax], a log-uniform in [amin, amax] sorted and redrawn until
// neighbours are >= hill_sep mutual Hill radii apart, e ~ Rayleigh(sig_e),
// inc ~ Rayleigh(sig_i), Omega, omega, f uniform; each planet is placed on its
// orbit about the centre of mass of the bodies before it (Murray & Dermott
// Eq. 2.122 and 2.36, as in reb_particle_from_orbit, src/tools.c:940-996), and
// the system is moved to its barycentre.  Writes k+1 records; returns the
// inner orbital period in *p_inner.
int rgpu_ic_planetary(unsigned int* seed, int k, double G, double mmin, double mmax, double amin, double amax,
                      double sig_e, double sig_i, double hill_sep, void* out, size_t stride, double* p_inner) {
    if (!seed || !out || k < 1 || k > 64 || stride < 88) return RGPU_ERR_ARG;
    Rng g{*seed};
    std::vector<double> ms(k), as(k);
    for (;;) {
        for (int j = 0; j < k; j++) ms[j] = exp(g.uniform(log(mmin), log(mmax)));
        for (int j = 0; j < k; j++) as[j] = exp(g.uniform(log(amin), log(amax)));
        std::vector<double> sorted(as);
        std::sort(sorted.begin(), sorted.end());
        as = sorted;
        bool ok = true;
        for (int j = 0; j + 1 < k; j++) {
            const double rh = cbrt((ms[j] + ms[j + 1]) / 3.) * (as[j] + as[j + 1]) / 2.;
            if (as[j + 1] - as[j] < hill_sep * rh) { ok = false; break; }
        }
        if (ok) break;
    }
    double* p0 = rec(out, stride, 0);
    put(p0, 0, 0, 0, 0, 0, 0, 1.0, 0.);
    double cm = 1.0, cx = 0, cy = 0, cz = 0, cvx = 0, cvy = 0, cvz = 0;
    for (int j = 0; j < k; j++) {
        const double e = g.rayleigh(sig_e), inc = g.rayleigh(sig_i);
        const double Om = g.uniform(0, 2 * M_PI), om = g.uniform(0, 2 * M_PI), f = g.uniform(0, 2 * M_PI);
        const double a = as[j], m = ms[j];
        const double r = a * (1 - e * e) / (1 + e * cos(f));
        const double v0 = sqrt(G * (m + cm) / a / (1. - e * e));
        const double cO = cos(Om), sO = sin(Om), co = cos(om), so = sin(om), cf = cos(f), sf = sin(f);
        const double ci = cos(inc), si = sin(inc);
        const double px = cx / cm, py = cy / cm, pz = cz / cm, pvx = cvx / cm, pvy = cvy / cm, pvz = cvz / cm;
        const double x = px + r * (cO * (co * cf - so * sf) - sO * (so * cf + co * sf) * ci);
        const double y = py + r * (sO * (co * cf - so * sf) + cO * (so * cf + co * sf) * ci);
        const double z = pz + r * (so * cf + co * sf) * si;
        const double vx = pvx + v0 * ((e + cf) * (-ci * co * sO - cO * so) - sf * (co * cO - ci * so * sO));
        const double vy = pvy + v0 * ((e + cf) * (ci * co * cO - sO * so) - sf * (co * sO + ci * so * cO));
        const double vz = pvz + v0 * ((e + cf) * co * si - sf * si * so);
        put(rec(out, stride, j + 1), x, y, z, vx, vy, vz, m, 0.);
        cm += m; cx += m * x; cy += m * y; cz += m * z; cvx += m * vx; cvy += m * vy; cvz += m * vz;
    }
    for (int j = 0; j <= k; j++) {
        double* r = rec(out, stride, j);
        r[0] -= cx / cm; r[1] -= cy / cm; r[2] -= cz / cm;
        r[3] -= cvx / cm; r[4] -= cvy / cm; r[5] -= cvz / cm;
    }
    if (p_inner) *p_inner = 2 * M_PI * sqrt(as[0] * as[0] * as[0] / (G * (1.0 + ms[0])));
    *seed = g.seed;
    return RGPU_OK;
}

}  // extern "C"
