/*
 * oracle.c -- CPU restatement of the REBOUND 5.0.0 force-and-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  Loaded by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg; the product
 * never touches it.  Build with -ffp-contract=off so every expression rounds
 * exactly like the reference's own parity build.
 *
 * Citations are REBOUND source paths (src/...:line).
 */
#include "oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static size_t n_active_of(const orc_sim* r) {
    return r->N_active == SIZE_MAX ? r->N : r->N_active;
}

/* N_active as WHFast reads it (src/integrator_whfast.c:1119): testparticle_type 1
 * puts every body into the coordinate transforms. */
static size_t wh_active_of(const orc_sim* r) {
    return (r->N_active == SIZE_MAX || r->testparticle_type == 1) ? r->N : r->N_active;
}

/* ------------------------------------------------------------------------
 * Boundary: src/boundary.c:35-141 (check) and :145-201 (ghost box offsets).
 * ---------------------------------------------------------------------- */
void orc_boundary_ghostbox(const orc_sim* r, int i, int j, int k, double gb[6]) {
    const double bx = r->root_size * (double)r->N_root_x;
    const double by = r->root_size * (double)r->N_root_y;
    const double bz = r->root_size * (double)r->N_root_z;
    gb[0] = gb[1] = gb[2] = gb[3] = gb[4] = gb[5] = 0.0;
    if (r->boundary == 1 || r->boundary == 2) {          /* open / periodic */
        gb[0] = bx * (double)i; gb[1] = by * (double)j; gb[2] = bz * (double)k;
    } else if (r->boundary == 3) {                       /* shear, :162-180 */
        const double vy = -1.5 * (double)i * r->OMEGA * bx;
        double shift;
        if (i == 0) shift = -fmod(vy * r->t, by);
        else if (i > 0) shift = -fmod(vy * r->t - by / 2., by) - by / 2.;
        else shift = -fmod(vy * r->t + by / 2., by) + by / 2.;
        gb[0] = bx * (double)i;
        gb[1] = by * (double)j - shift;
        gb[2] = bz * (double)k;
        gb[4] = vy;
    }
}

void orc_boundary_check(orc_sim* r) {
    const double bx = r->root_size * (double)r->N_root_x;
    const double by = r->root_size * (double)r->N_root_y;
    const double bz = r->root_size * (double)r->N_root_z;
    orc_particle* p = r->particles;
    if (r->boundary == 3) {                              /* :78-114 */
        const double O = r->OMEGA;
        const double offp1 = -fmod(-1.5 * O * bx * r->t + by / 2., by) - by / 2.;
        const double offm1 = -fmod(1.5 * O * bx * r->t - by / 2., by) + by / 2.;
        for (size_t i = 0; i < r->N; i++) {
            while (p[i].x > bx / 2.) { p[i].x -= bx; p[i].y += offp1; p[i].vy += 3. / 2. * O * bx; }
            while (p[i].x < -bx / 2.) { p[i].x += bx; p[i].y += offm1; p[i].vy -= 3. / 2. * O * bx; }
            while (p[i].y > by / 2.) p[i].y -= by;
            while (p[i].y < -by / 2.) p[i].y += by;
            while (p[i].z > bz / 2.) p[i].z -= bz;
            while (p[i].z < -bz / 2.) p[i].z += bz;
        }
    } else if (r->boundary == 2) {                       /* :115-135 */
        for (size_t i = 0; i < r->N; i++) {
            while (p[i].x > bx / 2.) p[i].x -= bx;
            while (p[i].x < -bx / 2.) p[i].x += bx;
            while (p[i].y > by / 2.) p[i].y -= by;
            while (p[i].y < -by / 2.) p[i].y += by;
            while (p[i].z > bz / 2.) p[i].z -= bz;
            while (p[i].z < -bz / 2.) p[i].z += bz;
        }
    }
}

/* ------------------------------------------------------------------------
 * Direct summation, BASIC: src/gravity.c:167-282.
 * ---------------------------------------------------------------------- */
void orc_gravity_basic_serial(orc_sim* r) {
    orc_particle* const P = r->particles;
    const size_t N = r->N, Na = n_active_of(r);
    const double G = r->G, eps2 = r->softening * r->softening;
    const int ign = r->gravity_ignore_terms;
    const size_t starti = ign == 0 ? 1 : 2;             /* :183-184 */
    const size_t startj = ign == 2 ? 1 : 0;
    for (size_t i = 0; i < N; i++) P[i].ax = P[i].ay = P[i].az = 0.;
    for (int gx = -r->N_ghost_x; gx <= r->N_ghost_x; gx++)
    for (int gy = -r->N_ghost_y; gy <= r->N_ghost_y; gy++)
    for (int gz = -r->N_ghost_z; gz <= r->N_ghost_z; gz++) {
        double gb[6];
        orc_boundary_ghostbox(r, gx, gy, gz, gb);
        for (size_t i = starti; i < Na; i++) {           /* pairwise, :195-214 */
            for (size_t j = startj; j < i; j++) {
                const double dx = (gb[0] + P[i].x) - P[j].x;
                const double dy = (gb[1] + P[i].y) - P[j].y;
                const double dz = (gb[2] + P[i].z) - P[j].z;
                const double rr = sqrt(dx * dx + dy * dy + dz * dz + eps2);
                const double pf = G / (rr * rr * rr);
                const double pfj = -pf * P[j].m;
                const double pfi = pf * P[i].m;
                P[i].ax += pfj * dx; P[i].ay += pfj * dy; P[i].az += pfj * dz;
                P[j].ax += pfi * dx; P[j].ay += pfi * dy; P[j].az += pfi * dz;
            }
        }
        const size_t st = Na > starti ? Na : starti;     /* test particles, :235-257 */
        for (size_t i = st; i < N; i++) {
            for (size_t j = startj; j < Na; j++) {
                const double dx = (gb[0] + P[i].x) - P[j].x;
                const double dy = (gb[1] + P[i].y) - P[j].y;
                const double dz = (gb[2] + P[i].z) - P[j].z;
                const double rr = sqrt(dx * dx + dy * dy + dz * dz + eps2);
                const double pf = G / (rr * rr * rr);
                const double pfj = -pf * P[j].m;
                P[i].ax += pfj * dx; P[i].ay += pfj * dy; P[i].az += pfj * dz;
                if (r->testparticle_type) {
                    const double pfi = pf * P[i].m;
                    P[j].ax += pfi * dx; P[j].ay += pfi * dy; P[j].az += pfi * dz;
                }
            }
        }
    }
}

/* One row block of the OpenMP gather loop (:215-233 and :258-277). */
static void basic_gather_rows(orc_sim* r, const double gb[6], size_t i0, size_t i1) {
    orc_particle* const P = r->particles;
    const size_t N = r->N, Na = n_active_of(r);
    const double G = r->G, eps2 = r->softening * r->softening;
    const int ign = r->gravity_ignore_terms;
#pragma omp parallel for schedule(guided)
    for (size_t i = i0; i < i1; i++) {
        double ax = P[i].ax, ay = P[i].ay, az = P[i].az;
        for (size_t j = 0; j < Na; j++) {
            if (ign == 1 && ((j == 1 && i == 0) || (i == 1 && j == 0))) continue;
            if (ign == 2 && (j == 0 || i == 0)) continue;
            if (i == j) continue;
            const double dx = (gb[0] + P[i].x) - P[j].x;
            const double dy = (gb[1] + P[i].y) - P[j].y;
            const double dz = (gb[2] + P[i].z) - P[j].z;
            const double rr = sqrt(dx * dx + dy * dy + dz * dz + eps2);
            const double pf = -G / (rr * rr * rr) * P[j].m;
            ax += pf * dx; ay += pf * dy; az += pf * dz;
        }
        P[i].ax = ax; P[i].ay = ay; P[i].az = az;
    }
    if (r->testparticle_type) {
#pragma omp parallel for
        for (size_t i = i0 < Na ? i0 : Na; i < (i1 < Na ? i1 : Na); i++) {
            double ax = P[i].ax, ay = P[i].ay, az = P[i].az;
            for (size_t j = Na; j < N; j++) {
                if (ign == 1 && (j == 1 && i == 0)) continue;
                if (ign == 2 && (j == 0 || i == 0)) continue;
                const double dx = (gb[0] + P[i].x) - P[j].x;
                const double dy = (gb[1] + P[i].y) - P[j].y;
                const double dz = (gb[2] + P[i].z) - P[j].z;
                const double rr = sqrt(dx * dx + dy * dy + dz * dz + eps2);
                const double pf = -G / (rr * rr * rr) * P[j].m;
                ax += pf * dx; ay += pf * dy; az += pf * dz;
            }
            P[i].ax = ax; P[i].ay = ay; P[i].az = az;
        }
    }
}

void orc_gravity_basic_omp_rows(orc_sim* r, size_t i0, size_t i1) {
    orc_particle* const P = r->particles;
    if (i1 > r->N) i1 = r->N;
    for (size_t i = i0; i < i1; i++) P[i].ax = P[i].ay = P[i].az = 0.;
    for (int gx = -r->N_ghost_x; gx <= r->N_ghost_x; gx++)
    for (int gy = -r->N_ghost_y; gy <= r->N_ghost_y; gy++)
    for (int gz = -r->N_ghost_z; gz <= r->N_ghost_z; gz++) {
        double gb[6];
        orc_boundary_ghostbox(r, gx, gy, gz, gb);
        basic_gather_rows(r, gb, i0, i1);
    }
}

void orc_gravity_basic_omp(orc_sim* r) { orc_gravity_basic_omp_rows(r, 0, r->N); }

/* ------------------------------------------------------------------------
 * Direct summation, COMPENSATED (Kahan per component): src/gravity.c:284-531.
 * ---------------------------------------------------------------------- */
#define KAHAN_ADD(acc, c, term) do { \
        const double y_ = (term) - (c); \
        const double t_ = (acc) + y_; \
        (c) = (t_ - (acc)) - y_; \
        (acc) = t_; } while (0)

void orc_gravity_compensated_serial(orc_sim* r) {
    orc_particle* const P = r->particles;
    const size_t N = r->N, Na = n_active_of(r);
    const double G = r->G, eps2 = r->softening * r->softening;
    const int ign = r->gravity_ignore_terms;
    double* cs = r->cs;
    for (size_t i = 0; i < N; i++) {
        P[i].ax = P[i].ay = P[i].az = 0.;
        cs[3 * i] = cs[3 * i + 1] = cs[3 * i + 2] = 0.;
    }
    for (size_t i = 0; i < Na; i++) {                    /* :416-469 */
        for (size_t j = i + 1; j < Na; j++) {
            if (ign == 1 && ((j == 1 && i == 0) || (i == 1 && j == 0))) continue;
            if (ign == 2 && (j == 0 || i == 0)) continue;
            const double dx = P[i].x - P[j].x, dy = P[i].y - P[j].y, dz = P[i].z - P[j].z;
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            const double rr = sqrt(r2);
            const double pf = G / (r2 * rr);
            const double pfi = pf * P[i].m, pfj = -pf * P[j].m;
            KAHAN_ADD(P[i].ax, cs[3 * i], pfj * dx);
            KAHAN_ADD(P[i].ay, cs[3 * i + 1], pfj * dy);
            KAHAN_ADD(P[i].az, cs[3 * i + 2], pfj * dz);
            KAHAN_ADD(P[j].ax, cs[3 * j], pfi * dx);
            KAHAN_ADD(P[j].ay, cs[3 * j + 1], pfi * dy);
            KAHAN_ADD(P[j].az, cs[3 * j + 2], pfi * dz);
        }
    }
    for (size_t i = Na; i < N; i++) {                    /* :472-528 */
        for (size_t j = 0; j < Na; j++) {
            if (ign == 1 && ((j == 1 && i == 0) || (i == 1 && j == 0))) continue;
            if (ign == 2 && (j == 0 || i == 0)) continue;
            const double dx = P[i].x - P[j].x, dy = P[i].y - P[j].y, dz = P[i].z - P[j].z;
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            const double rr = sqrt(r2);
            const double pf = G / (r2 * rr);
            const double pfj = -pf * P[j].m;
            KAHAN_ADD(P[i].ax, cs[3 * i], pfj * dx);
            KAHAN_ADD(P[i].ay, cs[3 * i + 1], pfj * dy);
            KAHAN_ADD(P[i].az, cs[3 * i + 2], pfj * dz);
            if (r->testparticle_type) {
                const double pfi = pf * P[i].m;
                KAHAN_ADD(P[j].ax, cs[3 * j], pfi * dx);
                KAHAN_ADD(P[j].ay, cs[3 * j + 1], pfi * dy);
                KAHAN_ADD(P[j].az, cs[3 * j + 2], pfi * dz);
            }
        }
    }
}

void orc_gravity_compensated_omp(orc_sim* r) {
    orc_particle* const P = r->particles;
    const size_t N = r->N, Na = n_active_of(r);
    const double G = r->G, eps2 = r->softening * r->softening;
    const int ign = r->gravity_ignore_terms;
    double* cs = r->cs;
    for (size_t i = 0; i < N; i++) {
        P[i].ax = P[i].ay = P[i].az = 0.;
        cs[3 * i] = cs[3 * i + 1] = cs[3 * i + 2] = 0.;
    }
#pragma omp parallel for schedule(guided)
    for (size_t i = 0; i < N; i++) {                     /* :308-343 and :346-378 */
        for (size_t j = 0; j < Na; j++) {
            if (ign == 1 && ((j == 1 && i == 0) || (i == 1 && j == 0))) continue;
            if (ign == 2 && (j == 0 || i == 0)) continue;
            if (i == j) continue;
            const double dx = P[i].x - P[j].x, dy = P[i].y - P[j].y, dz = P[i].z - P[j].z;
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            const double rr = sqrt(r2);
            const double pf = G / (r2 * rr);
            const double pfj = -pf * P[j].m;
            KAHAN_ADD(P[i].ax, cs[3 * i], pfj * dx);
            KAHAN_ADD(P[i].ay, cs[3 * i + 1], pfj * dy);
            KAHAN_ADD(P[i].az, cs[3 * i + 2], pfj * dz);
        }
    }
    if (r->testparticle_type) {                          /* :379-413 */
#pragma omp parallel for schedule(guided)
        for (size_t j = 0; j < Na; j++) {
            for (size_t i = Na; i < N; i++) {
                if (ign == 1 && ((j == 1 && i == 0) || (i == 1 && j == 0))) continue;
                if (ign == 2 && (j == 0 || i == 0)) continue;
                const double dx = P[i].x - P[j].x, dy = P[i].y - P[j].y, dz = P[i].z - P[j].z;
                const double r2 = dx * dx + dy * dy + dz * dz + eps2;
                const double rr = sqrt(r2);
                const double pf = G / (r2 * rr);
                const double pfi = pf * P[i].m;
                KAHAN_ADD(P[j].ax, cs[3 * j], pfi * dx);
                KAHAN_ADD(P[j].ay, cs[3 * j + 1], pfi * dy);
                KAHAN_ADD(P[j].az, cs[3 * j + 2], pfi * dz);
            }
        }
    }
}

/* ------------------------------------------------------------------------
 * Octree: src/tree.c.  One particle per leaf, cubic root boxes on an
 * N_root_x x N_root_y x N_root_z grid, recursive insertion in index order.
 * ---------------------------------------------------------------------- */
typedef struct ocell {
    double x, y, z, w, m, mx, my, mz;
    double mxx, mxy, mxz, myy, myz, mzz;     /* mass quadrupole (QUADRUPOLE builds) */
    struct ocell* oct[8];
    long pt;                /* >=0 leaf particle, <0 minus particle count */
} ocell;

typedef struct otree {
    ocell** root;
    size_t n_root;
} otree;

static int octant_of(const orc_particle* p, const ocell* c) {   /* tree.c:136-142 */
    int o = 0;
    if (p->x < c->x) o += 1;
    if (p->y < c->y) o += 2;
    if (p->z < c->z) o += 4;
    return o;
}

static ocell* cell_insert(orc_sim* r, ocell* node, long pt, const ocell* parent, int o) {
    const orc_particle* P = r->particles;
    if (!node) {                                                 /* tree.c:83-115 */
        node = (ocell*)calloc(1, sizeof(ocell));
        if (!parent) {
            const double bx = r->root_size * (double)r->N_root_x;
            const double by = r->root_size * (double)r->N_root_y;
            const double bz = r->root_size * (double)r->N_root_z;
            node->w = r->root_size;
            const int i = ((int)floor((P[pt].x + bx / 2.) / r->root_size)) % r->N_root_x;
            const int j = ((int)floor((P[pt].y + by / 2.) / r->root_size)) % r->N_root_y;
            const int k = ((int)floor((P[pt].z + bz / 2.) / r->root_size)) % r->N_root_z;
            node->x = -bx / 2. + r->root_size * (0.5 + (double)i);
            node->y = -by / 2. + r->root_size * (0.5 + (double)j);
            node->z = -bz / 2. + r->root_size * (0.5 + (double)k);
        } else {
            node->w = parent->w / 2.;
            node->x = parent->x + node->w / 2. * ((o >> 0) % 2 == 0 ? 1. : -1);
            node->y = parent->y + node->w / 2. * ((o >> 1) % 2 == 0 ? 1. : -1);
            node->z = parent->z + node->w / 2. * ((o >> 2) % 2 == 0 ? 1. : -1);
        }
        if (node->w <= 0.0) { r->error = 2; free(node); return NULL; }
        node->pt = pt;
        return node;
    }
    if (node->pt >= 0) {                                         /* tree.c:117-128 */
        const int o1 = octant_of(&P[node->pt], node);
        const int o2 = octant_of(&P[pt], node);
        if (o1 == o2 && P[pt].x == P[node->pt].x && P[pt].y == P[node->pt].y && P[pt].z == P[node->pt].z) {
            r->error = 3;   /* two particles with the same coordinates */
            return node;
        }
        node->oct[o1] = cell_insert(r, node->oct[o1], node->pt, node, o1);
        node->oct[o2] = cell_insert(r, node->oct[o2], pt, node, o2);
        node->pt = -2;
    } else {
        node->pt--;
        const int oo = octant_of(&P[pt], node);
        node->oct[oo] = cell_insert(r, node->oct[oo], pt, node, oo);
    }
    return node;
}

static void cell_free(ocell* c) {
    if (!c) return;
    for (int o = 0; o < 8; o++) cell_free(c->oct[o]);
    free(c);
}

static void tree_free(otree* t) {
    for (size_t i = 0; i < t->n_root; i++) cell_free(t->root[i]);
    free(t->root);
    t->root = NULL;
}

static int root_of(const orc_sim* r, const orc_particle* p) {  /* particle.c:119-126 */
    const int i = ((int)floor((p->x + r->root_size * (double)r->N_root_x / 2.) / r->root_size) + r->N_root_x) % r->N_root_x;
    const int j = ((int)floor((p->y + r->root_size * (double)r->N_root_y / 2.) / r->root_size) + r->N_root_y) % r->N_root_y;
    const int k = ((int)floor((p->z + r->root_size * (double)r->N_root_z / 2.) / r->root_size) + r->N_root_z) % r->N_root_z;
    return (k * r->N_root_y + j) * r->N_root_x + i;
}

static int tree_build(orc_sim* r, otree* t) {                  /* tree.c:254-271, :65-78 */
    t->n_root = (size_t)r->N_root_x * r->N_root_y * r->N_root_z;
    t->root = (ocell**)calloc(t->n_root, sizeof(ocell*));
    for (size_t i = 0; i < r->N; i++) {
        const orc_particle* p = &r->particles[i];
        if (fabs(p->x) > r->root_size * (double)r->N_root_x / 2. ||
            fabs(p->y) > r->root_size * (double)r->N_root_y / 2. ||
            fabs(p->z) > r->root_size * (double)r->N_root_z / 2.) { r->error = 4; return 4; }
        if (!isfinite(p->x) || !isfinite(p->y) || !isfinite(p->z)) { r->error = 5; return 5; }
        const int rb = root_of(r, p);
        t->root[rb] = cell_insert(r, t->root[rb], (long)i, NULL, 0);
        if (r->error) return r->error;
    }
    return 0;
}

static void cell_gravity_data(const orc_sim* r, ocell* c) {     /* tree.c:147-207 */
    c->mxx = c->mxy = c->mxz = c->myy = c->myz = c->mzz = 0.;
    if (c->pt < 0) {
        c->m = 0; c->mx = 0; c->my = 0; c->mz = 0;
        for (int o = 0; o < 8; o++) {
            ocell* d = c->oct[o];
            if (d) {
                cell_gravity_data(r, d);
                const double dm = d->m;
                c->mx += d->mx * dm;
                c->my += d->my * dm;
                c->mz += d->mz * dm;
                c->m += dm;
            }
        }
        const double mt = c->m;
        if (mt > 0) { c->mx /= mt; c->my /= mt; c->mz /= mt; }
        if (r->tree_quadrupole) {                                   /* tree.c:180-198, Hernquist 1987 */
            for (int o = 0; o < 8; o++) {
                const ocell* d = c->oct[o];
                if (!d) continue;
                const double dm = d->m;
                const double qx = d->mx - c->mx, qy = d->my - c->my, qz = d->mz - c->mz;
                const double qr2 = qx * qx + qy * qy + qz * qz;
                c->mxx += d->mxx + dm * (3. * qx * qx - qr2);
                c->mxy += d->mxy + dm * 3. * qx * qy;
                c->mxz += d->mxz + dm * 3. * qx * qz;
                c->myy += d->myy + dm * (3. * qy * qy - qr2);
                c->myz += d->myz + dm * 3. * qy * qz;
            }
            c->mzz = -c->mxx - c->myy;
        }
    } else {
        const orc_particle* p = &r->particles[c->pt];
        c->m = p->m; c->mx = p->x; c->my = p->y; c->mz = p->z;
    }
}

static void cell_accel(const orc_sim* r, long pt, const ocell* c, const double gx, const double gy, const double gz,
                       double* ax, double* ay, double* az) {      /* tree.c:275-318 */
    const double G = r->G, eps2 = r->softening * r->softening;
    const double dx = gx - c->mx, dy = gy - c->my, dz = gz - c->mz;
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (c->pt < 0) {
        if (c->w * c->w > r->opening_angle2 * r2) {
            for (int o = 0; o < 8; o++)
                if (c->oct[o]) cell_accel(r, pt, c->oct[o], gx, gy, gz, ax, ay, az);
        } else if (r->tree_quadrupole) {                            /* tree.c:293-306 */
            const double rr = sqrt(r2 + eps2);
            const double pf = -G / (rr * rr * rr) * c->m;
            double qpf = G / (rr * rr * rr * rr * rr);
            *ax += qpf * (dx * c->mxx + dy * c->mxy + dz * c->mxz);
            *ay += qpf * (dx * c->mxy + dy * c->myy + dz * c->myz);
            *az += qpf * (dx * c->mxz + dy * c->myz + dz * c->mzz);
            const double mrr = dx * dx * c->mxx + dy * dy * c->myy + dz * dz * c->mzz
                             + 2. * dx * dy * c->mxy + 2. * dx * dz * c->mxz + 2. * dy * dz * c->myz;
            qpf *= -5.0 / (2.0 * rr * rr) * mrr;
            *ax += (qpf + pf) * dx; *ay += (qpf + pf) * dy; *az += (qpf + pf) * dz;
        } else {
            const double rr = sqrt(r2 + eps2);
            const double pf = -G / (rr * rr * rr) * c->m;
            *ax += pf * dx; *ay += pf * dy; *az += pf * dz;
        }
    } else {
        if (c->pt == pt) return;
        const double rr = sqrt(r2 + eps2);
        const double pf = -G / (rr * rr * rr) * c->m;
        *ax += pf * dx; *ay += pf * dy; *az += pf * dz;
    }
}

void orc_gravity_tree(orc_sim* r) {                                /* gravity.c:47-106 */
    orc_boundary_check(r);
    otree t = {0};
    if (tree_build(r, &t)) { tree_free(&t); return; }
    for (size_t i = 0; i < t.n_root; i++) if (t.root[i]) cell_gravity_data(r, t.root[i]);
    orc_particle* const P = r->particles;
    const size_t N = r->N;
    for (size_t i = 0; i < N; i++) P[i].ax = P[i].ay = P[i].az = 0.;
    for (int gx = -r->N_ghost_x; gx <= r->N_ghost_x; gx++)
    for (int gy = -r->N_ghost_y; gy <= r->N_ghost_y; gy++)
    for (int gz = -r->N_ghost_z; gz <= r->N_ghost_z; gz++) {
        double gb[6];
        orc_boundary_ghostbox(r, gx, gy, gz, gb);
#pragma omp parallel for schedule(guided)
        for (size_t i = 0; i < N; i++) {
            const double sx = gb[0] + P[i].x, sy = gb[1] + P[i].y, sz = gb[2] + P[i].z;
            double ax = P[i].ax, ay = P[i].ay, az = P[i].az;
            for (size_t k = 0; k < t.n_root; k++)
                if (t.root[k]) cell_accel(r, (long)i, t.root[k], sx, sy, sz, &ax, &ay, &az);
            P[i].ax = ax; P[i].ay = ay; P[i].az = az;
        }
    }
    tree_free(&t);
}

static void cell_export(const ocell* c, int root, int depth, uint64_t path,
                        orc_cell* out, size_t cap, size_t* n) {
    if (*n < cap) {
        orc_cell* e = &out[*n];
        e->root = root; e->depth = depth; e->path = path;
        e->x = c->x; e->y = c->y; e->z = c->z; e->w = c->w;
        e->m = c->m; e->mx = c->mx; e->my = c->my; e->mz = c->mz;
        e->pt = c->pt;
    }
    (*n)++;
    for (int o = 0; o < 8; o++)
        if (c->oct[o]) cell_export(c->oct[o], root, depth + 1, (path << 3) | (uint64_t)o, out, cap, n);
}

int orc_tree_export(orc_sim* r, orc_cell* out, size_t cap, size_t* n_out) {
    otree t = {0};
    int err = tree_build(r, &t);
    *n_out = 0;
    if (!err) {
        for (size_t i = 0; i < t.n_root; i++) if (t.root[i]) cell_gravity_data(r, t.root[i]);
        for (size_t i = 0; i < t.n_root; i++)
            if (t.root[i]) cell_export(t.root[i], (int)i, 0, 0, out, cap, n_out);
    }
    tree_free(&t);
    return err;
}

/* ------------------------------------------------------------------------
 * Collision search: src/collision.c:49-124 (DIRECT), :197-269 and :422-503
 * (TREE).  Pairs are emitted in discovery order; the caller sorts.
 * ---------------------------------------------------------------------- */
typedef struct pairbuf { orc_collision* out; size_t cap, n; int grow; } pairbuf;

static void pair_push(pairbuf* b, size_t p1, size_t p2, const double gb[6], size_t ri) {
    if (b->grow && b->n == b->cap) {            /* growable per-thread buffers of the OpenMP search */
        const size_t nc = b->cap ? 2 * b->cap : 1024;
        orc_collision* o = (orc_collision*)realloc(b->out, nc * sizeof(orc_collision));
        if (o) { b->out = o; b->cap = nc; }
    }
    if (b->n < b->cap) {
        orc_collision* c = &b->out[b->n];
        c->p1 = p1; c->p2 = p2; c->ri = ri;
        memcpy(c->gb, gb, sizeof(double) * 6);
    }
    b->n++;
}

size_t orc_collision_search_direct(orc_sim* r, orc_collision* out, size_t cap) {
    const orc_particle* P = r->particles;
    pairbuf b = {out, cap, 0};
    const int nx = r->N_ghost_x > 1 ? 1 : r->N_ghost_x;
    const int ny = r->N_ghost_y > 1 ? 1 : r->N_ghost_y;
    const int nz = r->N_ghost_z > 1 ? 1 : r->N_ghost_z;
    for (int gx = -nx; gx <= nx; gx++)
    for (int gy = -ny; gy <= ny; gy++)
    for (int gz = -nz; gz <= nz; gz++) {
        double g0[6];
        orc_boundary_ghostbox(r, gx, gy, gz, g0);
        for (size_t i = 0; i < r->N; i++) {
            const orc_particle p1 = P[i];
            const double sx = g0[0] + p1.x, sy = g0[1] + p1.y, sz = g0[2] + p1.z;
            const double svx = g0[3] + p1.vx, svy = g0[4] + p1.vy, svz = g0[5] + p1.vz;
            for (size_t j = 0; j < r->N; j++) {
                if (i == j) continue;
                const orc_particle p2 = P[j];
                const double dx = sx - p2.x, dy = sy - p2.y, dz = sz - p2.z;
                const double sr = p1.r + p2.r;
                const double r2 = dx * dx + dy * dy + dz * dz;
                if (r2 > sr * sr) continue;
                const double dvx = svx - p2.vx, dvy = svy - p2.vy, dvz = svz - p2.vz;
                if (dvx * dx + dvy * dy + dvz * dz > 0) continue;
                pair_push(&b, i, j, g0, 0);
            }
        }
    }
    return b.n;
}

static void tree_nn(const orc_sim* r, const double s[6], const double g0[6], int ri, double p1r, double r2nd,
                    size_t p1, const ocell* c, pairbuf* b) {     /* collision.c:422-503 */
    const orc_particle* P = r->particles;
    if (c->pt >= 0) {
        if ((size_t)c->pt == p1) return;
        const orc_particle p2 = P[c->pt];
        const double dx = s[0] - p2.x, dy = s[1] - p2.y, dz = s[2] - p2.z;
        const double r2 = dx * dx + dy * dy + dz * dz;
        const double rp = p1r + p2.r;
        if (r2 > rp * rp) return;
        const double dvx = s[3] - p2.vx, dvy = s[4] - p2.vy, dvz = s[5] - p2.vz;
        if (dvx * dx + dvy * dy + dvz * dz > 0) return;
        pair_push(b, p1, (size_t)c->pt, g0, (size_t)ri);
    } else {
        const double dx = s[0] - c->x, dy = s[1] - c->y, dz = s[2] - c->z;
        const double r2 = dx * dx + dy * dy + dz * dz;
        const double rp = p1r + r2nd + 0.86602540378443 * c->w;
        if (r2 < rp * rp)
            for (int o = 0; o < 8; o++)
                if (c->oct[o]) tree_nn(r, s, g0, ri, p1r, r2nd, p1, c->oct[o], b);
    }
}

static double second_largest_radius(const orc_sim* r) {   /* simulation.c:718-800, serial branch */
    double l1 = -1.0, l2 = -1.0;
    size_t i1 = SIZE_MAX, i2 = SIZE_MAX;
    for (size_t i = 0; i < r->N; i++) {
        const double rad = r->particles[i].r;
        if (rad > l1) { l2 = l1; i2 = i1; l1 = rad; i1 = i; }
        else if (rad > l2) { l2 = rad; i2 = i; }
    }
    return i2 == SIZE_MAX ? 0.0 : r->particles[i2].r;
}

size_t orc_collision_search_tree(orc_sim* r, orc_collision* out, size_t cap) {
    pairbuf b = {out, cap, 0};
    otree t = {0};
    if (tree_build(r, &t)) { tree_free(&t); return 0; }
    const int nx = r->N_ghost_x > 1 ? 1 : r->N_ghost_x;
    const int ny = r->N_ghost_y > 1 ? 1 : r->N_ghost_y;
    const int nz = r->N_ghost_z > 1 ? 1 : r->N_ghost_z;
    const double r2nd = second_largest_radius(r);
    const orc_particle* P = r->particles;
    for (size_t i = 0; i < r->N; i++) {
        const orc_particle p1 = P[i];
        for (int gx = -nx; gx <= nx; gx++)
        for (int gy = -ny; gy <= ny; gy++)
        for (int gz = -nz; gz <= nz; gz++) {
            double g0[6], s[6];
            orc_boundary_ghostbox(r, gx, gy, gz, g0);
            s[0] = g0[0] + p1.x; s[1] = g0[1] + p1.y; s[2] = g0[2] + p1.z;
            s[3] = g0[3] + p1.vx; s[4] = g0[4] + p1.vy; s[5] = g0[5] + p1.vz;
            for (size_t k = 0; k < t.n_root; k++)
                if (t.root[k]) tree_nn(r, s, g0, (int)k, p1.r, r2nd, i, t.root[k], &b);
        }
    }
    tree_free(&t);
    return b.n;
}

/* The same search with the particle loop split over OpenMP threads: thread t
 * takes a contiguous block of particles in increasing order and collects its
 * pairs in its own buffer, and the buffers are joined in thread order, so the
 * list (and its order) equals the serial search above. */
size_t orc_collision_search_tree_omp(orc_sim* r, orc_collision* out, size_t cap) {
    otree t = {0};
    if (tree_build(r, &t)) { tree_free(&t); return 0; }
    const int nx = r->N_ghost_x > 1 ? 1 : r->N_ghost_x;
    const int ny = r->N_ghost_y > 1 ? 1 : r->N_ghost_y;
    const int nz = r->N_ghost_z > 1 ? 1 : r->N_ghost_z;
    const double r2nd = second_largest_radius(r);
    const orc_particle* P = r->particles;
    int nt = 1;
#ifdef _OPENMP
    nt = omp_get_max_threads();
#endif
    pairbuf* bufs = (pairbuf*)calloc((size_t)nt, sizeof(pairbuf));
    if (!bufs) { tree_free(&t); return 0; }
#pragma omp parallel num_threads(nt)
    {
        int th = 0, T = 1;
#ifdef _OPENMP
        th = omp_get_thread_num();
        T = omp_get_num_threads();
#endif
        pairbuf* b = &bufs[th];
        b->grow = 1;
        const size_t lo = r->N * (size_t)th / (size_t)T, hi = r->N * (size_t)(th + 1) / (size_t)T;
        for (size_t i = lo; i < hi; i++) {
            const orc_particle p1 = P[i];
            for (int gx = -nx; gx <= nx; gx++)
            for (int gy = -ny; gy <= ny; gy++)
            for (int gz = -nz; gz <= nz; gz++) {
                double g0[6], s[6];
                orc_boundary_ghostbox(r, gx, gy, gz, g0);
                s[0] = g0[0] + p1.x; s[1] = g0[1] + p1.y; s[2] = g0[2] + p1.z;
                s[3] = g0[3] + p1.vx; s[4] = g0[4] + p1.vy; s[5] = g0[5] + p1.vz;
                for (size_t k = 0; k < t.n_root; k++)
                    if (t.root[k]) tree_nn(r, s, g0, (int)k, p1.r, r2nd, i, t.root[k], b);
            }
        }
    }
    size_t n = 0;
    for (int th = 0; th < nt; th++) {
        for (size_t k = 0; k < bufs[th].n && k < bufs[th].cap; k++)
            if (n + k < cap) out[n + k] = bufs[th].out[k];
        n += bufs[th].n;
        free(bufs[th].out);
    }
    free(bufs);
    tree_free(&t);
    return n;
}

/* Do two straight paths over the last step (relative position d at its end,
 * relative velocity dv, step dtl) come within rsum?  src/collision.c:149-173 and
 * :512-534: the distances at the end, at the start and, when it falls inside
 * the step, at closest approach. */
static int paths_touch(double dx, double dy, double dz, double dvx, double dvy, double dvz, double dtl,
                       double rsum) {
    const double r_end = dx * dx + dy * dy + dz * dz;
    const double sx = dx - dtl * dvx, sy = dy - dtl * dvy, sz = dz - dtl * dvz;
    const double r_start = sx * sx + sy * sy + sz * sz;
    const double tc = (dx * dvx + dy * dvy + dz * dvz) / (dvx * dvx + dvy * dvy + dvz * dvz);
    double rmin2 = r_end < r_start ? r_end : r_start;
    if (tc / dtl >= 0. && tc / dtl <= 1.) {
        const double cx = dx - tc * dvx, cy = dy - tc * dvy, cz = dz - tc * dvz;
        const double r_close = cx * cx + cy * cy + cz * cz;
        rmin2 = rmin2 < r_close ? rmin2 : r_close;
    }
    return !(rmin2 > rsum * rsum);
}

/* REB_COLLISION_LINE (src/collision.c:125-196): ghost boxes of the inner ring,
 * then i, then j > i. */
size_t orc_collision_search_line(orc_sim* r, double dtl, orc_collision* out, size_t cap) {
    const orc_particle* P = r->particles;
    pairbuf b = {out, cap, 0};
    const int nx = r->N_ghost_x > 1 ? 1 : r->N_ghost_x;
    const int ny = r->N_ghost_y > 1 ? 1 : r->N_ghost_y;
    const int nz = r->N_ghost_z > 1 ? 1 : r->N_ghost_z;
    for (int gx = -nx; gx <= nx; gx++)
    for (int gy = -ny; gy <= ny; gy++)
    for (int gz = -nz; gz <= nz; gz++) {
        double g0[6];
        orc_boundary_ghostbox(r, gx, gy, gz, g0);
        for (size_t i = 0; i < r->N; i++) {
            const orc_particle p1 = P[i];
            const double sx = g0[0] + p1.x, sy = g0[1] + p1.y, sz = g0[2] + p1.z;
            const double svx = g0[3] + p1.vx, svy = g0[4] + p1.vy, svz = g0[5] + p1.vz;
            for (size_t j = i + 1; j < r->N; j++) {
                const orc_particle p2 = P[j];
                if (paths_touch(sx - p2.x, sy - p2.y, sz - p2.z, svx - p2.vx, svy - p2.vy, svz - p2.vz, dtl,
                                p1.r + p2.r))
                    pair_push(&b, i, j, g0, 0);
            }
        }
    }
    return b.n;
}

static void tree_paths(const orc_sim* r, const double s[6], const double g0[6], int ri, double p1r,
                       double p1r_dtv, double maxdrift, double dtl, size_t p1, const ocell* c,
                       pairbuf* b) {                              /* collision.c:506-572 */
    const orc_particle* P = r->particles;
    if (c->pt >= 0) {
        if ((size_t)c->pt == p1) return;
        const orc_particle p2 = P[c->pt];
        if (paths_touch(s[0] - p2.x, s[1] - p2.y, s[2] - p2.z, s[3] - p2.vx, s[4] - p2.vy, s[5] - p2.vz, dtl,
                        p1r + p2.r))
            pair_push(b, p1, (size_t)c->pt, g0, (size_t)ri);
    } else {
        const double dx = s[0] - c->x, dy = s[1] - c->y, dz = s[2] - c->z;
        const double r2 = dx * dx + dy * dy + dz * dz;
        const double rp = p1r_dtv + maxdrift + 0.86602540378443 * c->w;
        if (r2 < rp * rp)
            for (int o = 0; o < 8; o++)
                if (c->oct[o]) tree_paths(r, s, g0, ri, p1r, p1r_dtv, maxdrift, dtl, p1, c->oct[o], b);
    }
}

/* REB_COLLISION_LINETREE (src/collision.c:270-330): i, then ghost boxes, then roots. */
size_t orc_collision_search_linetree(orc_sim* r, double dtl, orc_collision* out, size_t cap) {
    pairbuf b = {out, cap, 0};
    const orc_particle* P = r->particles;
    double vmax2 = 0.;
    for (size_t i = 0; i < r->N; i++) {
        const double v2 = P[i].vx * P[i].vx + P[i].vy * P[i].vy + P[i].vz * P[i].vz;
        vmax2 = vmax2 > v2 ? vmax2 : v2;
    }
    const double maxdrift = dtl * sqrt(vmax2);
    otree t = {0};
    if (tree_build(r, &t)) { tree_free(&t); return 0; }
    const int nx = r->N_ghost_x > 1 ? 1 : r->N_ghost_x;
    const int ny = r->N_ghost_y > 1 ? 1 : r->N_ghost_y;
    const int nz = r->N_ghost_z > 1 ? 1 : r->N_ghost_z;
    for (size_t i = 0; i < r->N; i++) {
        const orc_particle p1 = P[i];
        const double p1r_dtv = p1.r + dtl * sqrt(p1.vx * p1.vx + p1.vy * p1.vy + p1.vz * p1.vz);
        for (int gx = -nx; gx <= nx; gx++)
        for (int gy = -ny; gy <= ny; gy++)
        for (int gz = -nz; gz <= nz; gz++) {
            double g0[6], s[6];
            orc_boundary_ghostbox(r, gx, gy, gz, g0);
            s[0] = g0[0] + p1.x; s[1] = g0[1] + p1.y; s[2] = g0[2] + p1.z;
            s[3] = g0[3] + p1.vx; s[4] = g0[4] + p1.vy; s[5] = g0[5] + p1.vz;
            for (size_t k = 0; k < t.n_root; k++)
                if (t.root[k]) tree_paths(r, s, g0, (int)k, p1.r, p1r_dtv, maxdrift, dtl, i, t.root[k], &b);
        }
    }
    tree_free(&t);
    return b.n;
}

/* Hardsphere resolution, src/collision.c:573-665, constant restitution eps. */
void orc_collision_resolve_hardsphere(orc_sim* r, const orc_collision* c, double eps, double minvel) {
    orc_particle* P = r->particles;
    const orc_particle p1 = P[c->p1], p2 = P[c->p2];
    const double* gb = c->gb;
    const double x21 = p1.x + gb[0] - p2.x, y21 = p1.y + gb[1] - p2.y, z21 = p1.z + gb[2] - p2.z;
    const double rp = p1.r + p2.r;
    if (rp * rp < x21 * x21 + y21 * y21 + z21 * z21) return;
    const double vx21 = p1.vx + gb[3] - p2.vx, vy21 = p1.vy + gb[4] - p2.vy, vz21 = p1.vz + gb[5] - p2.vz;
    if (vx21 * x21 + vy21 * y21 + vz21 * z21 > 0) return;
    const double th = atan2(z21, y21), sth = sin(th), cth = cos(th);
    const double vy21n = cth * vy21 + sth * vz21;
    const double y21n = cth * y21 + sth * z21;
    const double ph = atan2(y21n, x21), cph = cos(ph), sph = sin(ph);
    const double vx21nn = cph * vx21 + sph * vy21n;
    double dvx2 = -(1.0 + eps) * vx21nn;
    const double minr = (p1.r > p2.r) ? p2.r : p1.r;
    const double maxr = (p1.r < p2.r) ? p2.r : p1.r;
    double mindv = minr * minvel;
    const double rr = sqrt(x21 * x21 + y21 * y21 + z21 * z21);
    mindv *= 1. - (rr - maxr) / minr;
    if (mindv > maxr * minvel) mindv = maxr * minvel;
    if (dvx2 < mindv) dvx2 = mindv;
    const double dvx2n = cph * dvx2, dvy2n = sph * dvx2;
    const double dvy2nn = cth * dvy2n, dvz2nn = sth * dvy2n;
    const double p2pf = p1.m / (p1.m + p2.m);
    P[c->p2].vx -= p2pf * dvx2n; P[c->p2].vy -= p2pf * dvy2nn; P[c->p2].vz -= p2pf * dvz2nn;
    const double p1pf = p2.m / (p1.m + p2.m);
    P[c->p1].vx += p1pf * dvx2n; P[c->p1].vy += p1pf * dvy2nn; P[c->p1].vz += p1pf * dvz2nn;
}

/* ------------------------------------------------------------------------
 * Leapfrog order 2: src/integrator_leapfrog.c:72-107.
 * ---------------------------------------------------------------------- */
static void update_accel(orc_sim* r, int gravity) {      /* simulation.c:640-689 */
    switch (gravity) {
        case 0: for (size_t i = 0; i < r->N; i++) r->particles[i].ax = r->particles[i].ay = r->particles[i].az = 0.; break;
        case 1: orc_gravity_basic_serial(r); break;
        case 2: orc_gravity_compensated_serial(r); break;
        case 3: orc_gravity_tree(r); break;
        case 101: orc_gravity_basic_omp(r); break;
        case 102: orc_gravity_compensated_omp(r); break;
        default: r->error = 1; break;
    }
}

static void lf_drift(orc_sim* r, double dt) {
    orc_particle* P = r->particles;
    for (size_t i = 0; i < r->N; i++) {
        P[i].x += dt * P[i].vx; P[i].y += dt * P[i].vy; P[i].z += dt * P[i].vz;
    }
    r->t += dt;
}

static void lf_kick(orc_sim* r, double dt) {
    orc_particle* P = r->particles;
    for (size_t i = 0; i < r->N; i++) {
        P[i].vx += dt * P[i].ax; P[i].vy += dt * P[i].ay; P[i].vz += dt * P[i].az;
    }
}

void orc_leapfrog_step(orc_sim* r, int gravity) {
    r->gravity_ignore_terms = 0;
    const double dt = r->dt;
    lf_drift(r, dt * 0.5);
    update_accel(r, gravity);
    lf_kick(r, dt);
    lf_drift(r, dt * 0.5);
}

/* Orders 4, 6 and 8: src/integrator_leapfrog.c:68-70 (coefficients) and :111-196
 * (stage sequences), restated as a drift, then per stage accelerations, kick and
 * drift, with the same expression for every drift and kick length. */
static const double orc_lf4_a = 0.675603595979828817023843904485;
static const double orc_lf6_a[5] = {0.1867, 0.5554970237124784, 0.1294669489134754, -0.843265623387734,
                                    0.9432033015235604};
static const double orc_lf8_a[9] = {0.128865979381443, 0.581514087105251, -0.410175371469850, 0.1851469357165877,
                                    -0.4095523434208514, 0.1444059410800120, 0.2783355003936797,
                                    0.3149566839162949, -0.6269948254051343979};

int orc_leapfrog_step_order(orc_sim* r, int gravity, int order) {
    if (order == 2) { orc_leapfrog_step(r, gravity); return 0; }
    r->gravity_ignore_terms = 0;
    const double dt = r->dt;
    if (order == 4) {
        const double a = orc_lf4_a;
        lf_drift(r, dt * a);
        update_accel(r, gravity); lf_kick(r, dt * 2. * a); lf_drift(r, dt * (0.5 - a));
        update_accel(r, gravity); lf_kick(r, dt * (1. - 4. * a)); lf_drift(r, dt * (0.5 - a));
        update_accel(r, gravity); lf_kick(r, dt * 2. * a); lf_drift(r, dt * a);
        return 0;
    }
    if (order != 6 && order != 8) return 1;
    const double* a = order == 6 ? orc_lf6_a : orc_lf8_a;
    const int m = order == 6 ? 5 : 9;
    lf_drift(r, dt * a[0] * 0.5);
    /* up the coefficient list and back down: kicks a0..a[m-1]..a0 */
    for (int i = 0; i < m; i++) {
        update_accel(r, gravity);
        lf_kick(r, dt * a[i]);
        if (i + 1 < m) lf_drift(r, dt * (a[i] + a[i + 1]) * 0.5);
    }
    for (int i = m - 2; i >= 0; i--) {
        lf_drift(r, dt * (a[i] + a[i + 1]) * 0.5);
        update_accel(r, gravity);
        lf_kick(r, dt * a[i]);
    }
    lf_drift(r, dt * a[0] * 0.5);
    return 0;
}

/* ------------------------------------------------------------------------
 * SEI: src/integrator_sei.c:86-174.
 * ---------------------------------------------------------------------- */
static void sei_h012(const orc_sim* r, orc_particle* p) {
    const double O = r->OMEGA, OZ = r->OMEGAZ;
    const double zx = p->z * OZ, zy = p->vz;
    const double zt1 = zx - r->sei_tandtz * zy;
    const double zyt = r->sei_sindtz * zt1 + zy;
    const double zxt = zt1 - r->sei_tandtz * zyt;
    p->z = zxt / OZ;
    p->vz = zyt;
    const double aO = 2. * p->vy + 4. * p->x * O;
    const double bO = p->y * O - 2. * p->vx;
    const double ys = (p->y * O - bO) / 2.;
    const double xs = (p->x * O - aO);
    const double xst1 = xs - r->sei_tandt * ys;
    const double yst = r->sei_sindt * xst1 + ys;
    const double xst = xst1 - r->sei_tandt * yst;
    p->x = (xst + aO) / O;
    p->y = (yst * 2. + bO) / O - 3. / 4. * aO * r->dt;
    p->vx = yst;
    p->vy = -xst * 2. - 3. / 2. * aO;
}

void orc_sei_step(orc_sim* r, int gravity) {
    r->gravity_ignore_terms = 0;
    if (r->sei_lastdt != r->dt) {
        if (r->OMEGAZ == -1) r->OMEGAZ = r->OMEGA;
        r->sei_sindt = sin(r->OMEGA * (-r->dt / 2.));
        r->sei_tandt = tan(r->OMEGA * (-r->dt / 4.));
        r->sei_sindtz = sin(r->OMEGAZ * (-r->dt / 2.));
        r->sei_tandtz = tan(r->OMEGAZ * (-r->dt / 4.));
        r->sei_lastdt = r->dt;
    }
    for (size_t i = 0; i < r->N; i++) sei_h012(r, &r->particles[i]);
    r->t += r->dt / 2.;
    update_accel(r, gravity);
    for (size_t i = 0; i < r->N; i++) {
        orc_particle* p = &r->particles[i];
        p->vx += p->ax * r->dt; p->vy += p->ay * r->dt; p->vz += p->az * r->dt;
        sei_h012(r, p);
    }
    r->t += r->dt / 2.;
}

/* ------------------------------------------------------------------------
 * WHFast, Jacobi coordinates, DEFAULT kernel: src/integrator_whfast.c.
 * ---------------------------------------------------------------------- */
static const double ifact[16] = {1., 1., 1. / 2., 1. / 6., 1. / 24., 1. / 120., 1. / 720., 1. / 5040.,
    1. / 40320., 1. / 362880., 1. / 3628800., 1. / 39916800., 1. / 479001600., 1. / 6227020800.,
    1. / 87178291200., 1. / 1307674368000.};

static void stumpff_c3(double* cs, double z) {           /* :189-212 */
    unsigned n = 0;
    while (fabs(z) > 0.1) { z = z / 4.; n++; }
    const int nmax = 13;
    double co = ifact[nmax], ce = ifact[nmax - 1];
    for (int np = nmax - 2; np >= 3; np -= 2) {
        co = ifact[np] - z * co;
        ce = ifact[np - 1] - z * ce;
    }
    cs[3] = co; cs[2] = ce;
    cs[1] = ifact[1] - z * co;
    cs[0] = ifact[0] - z * ce;
    for (; n > 0; n--) {
        cs[3] = (cs[2] + cs[0] * cs[3]) * 0.25;
        cs[2] = cs[1] * cs[1] * 0.5;
        cs[1] = cs[0] * cs[1];
        cs[0] = 2. * cs[0] * cs[0] - 1.;
    }
}

static void stiefel_g3(double* Gs, double beta, double X) {  /* :226-232 */
    const double X2 = X * X;
    stumpff_c3(Gs, beta * X2);
    Gs[1] *= X;
    Gs[2] *= X2;
    Gs[3] *= X2 * X;
}

void orc_whfast_kepler_solver(orc_particle* p, double mu, double dt) {   /* :241-427 */
    const orc_particle p1 = *p;
    const double r0 = sqrt(p1.x * p1.x + p1.y * p1.y + p1.z * p1.z);
    const double r0i = 1. / r0;
    const double v2 = p1.vx * p1.vx + p1.vy * p1.vy + p1.vz * p1.vz;
    const double beta = 2. * mu * r0i - v2;
    const double eta0 = p1.x * p1.vx + p1.y * p1.vy + p1.z * p1.vz;
    const double zeta0 = mu - beta * r0;
    double X, Gs[4], invperiod = 0, X_per_period = nan("");
    if (beta > 0.) {
        const double sb = sqrt(beta);
        invperiod = sb * beta / (2. * M_PI * mu);
        X_per_period = 2. * M_PI / sb;
        const double dtr0i = dt * r0i;
        X = dtr0i * (1. - dtr0i * eta0 * 0.5 * r0i);
    } else {
        X = 0.;
    }
    int converged = 0;
    double oldX = X;
    stiefel_g3(Gs, beta, X);
    const double e1 = eta0 * Gs[1] + zeta0 * Gs[2];
    double ri = 1. / (r0 + e1);
    X = ri * (X * e1 - eta0 * Gs[2] - zeta0 * Gs[3] + dt);
    if (fabs(X - oldX) > 0.01 * X_per_period) {
        X = beta * dt / mu;
        double prevX[65];
        for (int nl = 1; nl < 64; nl++) {
            stiefel_g3(Gs, beta, X);
            const double f = r0 * X + eta0 * Gs[2] + zeta0 * Gs[3] - dt;
            const double fp = r0 + eta0 * Gs[1] + zeta0 * Gs[2];
            const double fpp = eta0 * Gs[0] + zeta0 * Gs[1];
            const double den = fp + sqrt(fabs(16. * fp * fp - 20. * f * fpp));
            X = (X * den - 5. * f) / den;
            for (int i = 1; i < nl; i++) {
                if (X == prevX[i]) { nl = 64; converged = 1; break; }
            }
            prevX[nl] = X;
        }
        const double e2 = eta0 * Gs[1] + zeta0 * Gs[2];
        ri = 1. / (r0 + e2);
    } else {
        double oldX2 = nan("");
        for (int nh = 1; nh < 32; nh++) {
            oldX2 = oldX;
            oldX = X;
            stiefel_g3(Gs, beta, X);
            const double e2 = eta0 * Gs[1] + zeta0 * Gs[2];
            ri = 1. / (r0 + e2);
            X = ri * (X * e2 - eta0 * Gs[2] - zeta0 * Gs[3] + dt);
            if (X == oldX || X == oldX2) { converged = 1; break; }
        }
    }
    if (!converged) {                                    /* bisection, :333-370 */
        double Xmin, Xmax;
        if (beta > 0.) {
            Xmin = X_per_period * floor(dt * invperiod);
            Xmax = Xmin + X_per_period;
        } else {
            const double h2 = r0 * r0 * v2 - eta0 * eta0;
            const double q = h2 / mu / (1. + sqrt(1. - h2 * beta / (mu * mu)));
            const double vq = copysign(sqrt(h2) / q, dt);
            Xmin = dt / (fabs(vq * dt) + r0);
            Xmax = dt / q;
            if (dt < 0.) { const double tmp = Xmin; Xmin = Xmax; Xmax = tmp; }
        }
        X = (Xmax + Xmin) / 2.;
        do {
            stiefel_g3(Gs, beta, X);
            const double s = r0 * X + eta0 * Gs[2] + zeta0 * Gs[3] - dt;
            if (s >= 0.) Xmax = X; else Xmin = X;
            X = (Xmax + Xmin) / 2.;
        } while (fabs(Xmax - Xmin) > fabs((Xmax + Xmin) * 1e-15));
        const double e2 = eta0 * Gs[1] + zeta0 * Gs[2];
        ri = 1. / (r0 + e2);
    }
    if (isnan(ri)) { ri = 0.; Gs[1] = 0.; Gs[2] = 0.; Gs[3] = 0.; }
    const double f = -mu * Gs[2] * r0i;
    const double g = dt - mu * Gs[3];
    const double fd = -mu * Gs[1] * r0i * ri;
    const double gd = -mu * Gs[2] * ri;
    p->x += f * p1.x + g * p1.vx;
    p->y += f * p1.y + g * p1.vy;
    p->z += f * p1.z + g * p1.vz;
    p->vx += fd * p1.x + gd * p1.vx;
    p->vy += fd * p1.y + gd * p1.vy;
    p->vz += fd * p1.z + gd * p1.vz;
}

void orc_inertial_to_jacobi_posvel(const orc_particle* ps, orc_particle* pj, const orc_particle* pm, size_t N, size_t Na) {
    /* src/transformations.c:34-81 */
    double eta = pm[0].m;
    double sx = eta * ps[0].x, sy = eta * ps[0].y, sz = eta * ps[0].z;
    double svx = eta * ps[0].vx, svy = eta * ps[0].vy, svz = eta * ps[0].vz;
    for (size_t i = 1; i < Na; i++) {
        const double ei = 1. / eta;
        const orc_particle pi = ps[i];
        eta += pm[i].m;
        const double pme = eta * ei;
        pj[i].m = pi.m;
        pj[i].x = pi.x - sx * ei; pj[i].y = pi.y - sy * ei; pj[i].z = pi.z - sz * ei;
        pj[i].vx = pi.vx - svx * ei; pj[i].vy = pi.vy - svy * ei; pj[i].vz = pi.vz - svz * ei;
        sx = sx * pme + pm[i].m * pj[i].x; sy = sy * pme + pm[i].m * pj[i].y; sz = sz * pme + pm[i].m * pj[i].z;
        svx = svx * pme + pm[i].m * pj[i].vx; svy = svy * pme + pm[i].m * pj[i].vy; svz = svz * pme + pm[i].m * pj[i].vz;
    }
    const double ei = 1. / eta;
    for (size_t i = Na; i < N; i++) {
        const orc_particle pi = ps[i];
        pj[i].m = pi.m;
        pj[i].x = pi.x - sx * ei; pj[i].y = pi.y - sy * ei; pj[i].z = pi.z - sz * ei;
        pj[i].vx = pi.vx - svx * ei; pj[i].vy = pi.vy - svy * ei; pj[i].vz = pi.vz - svz * ei;
    }
    const double mti = 1. / eta;
    pj[0].m = eta;
    pj[0].x = sx * mti; pj[0].y = sy * mti; pj[0].z = sz * mti;
    pj[0].vx = svx * mti; pj[0].vy = svy * mti; pj[0].vz = svz * mti;
}

void orc_jacobi_to_inertial_posvel(orc_particle* ps, const orc_particle* pj, const orc_particle* pm, size_t N, size_t Na) {
    /* src/transformations.c:178-226 */
    double eta = pj[0].m;
    double sx = pj[0].x * eta, sy = pj[0].y * eta, sz = pj[0].z * eta;
    double svx = pj[0].vx * eta, svy = pj[0].vy * eta, svz = pj[0].vz * eta;
    for (size_t i = N - 1; i >= Na; i--) {
        const orc_particle q = pj[i];
        const double ei = 1. / eta;
        ps[i].x = q.x + sx * ei; ps[i].y = q.y + sy * ei; ps[i].z = q.z + sz * ei;
        ps[i].vx = q.vx + svx * ei; ps[i].vy = q.vy + svy * ei; ps[i].vz = q.vz + svz * ei;
        if (i == 0) break;
    }
    for (size_t i = Na - 1; i > 0; i--) {
        const orc_particle q = pj[i];
        const double ei = 1. / eta;
        sx = (sx - pm[i].m * q.x) * ei; sy = (sy - pm[i].m * q.y) * ei; sz = (sz - pm[i].m * q.z) * ei;
        svx = (svx - pm[i].m * q.vx) * ei; svy = (svy - pm[i].m * q.vy) * ei; svz = (svz - pm[i].m * q.vz) * ei;
        ps[i].x = q.x + sx; ps[i].y = q.y + sy; ps[i].z = q.z + sz;
        ps[i].vx = q.vx + svx; ps[i].vy = q.vy + svy; ps[i].vz = q.vz + svz;
        eta -= pm[i].m;
        sx *= eta; sy *= eta; sz *= eta; svx *= eta; svy *= eta; svz *= eta;
    }
    const double mi = 1. / eta;
    ps[0].x = sx * mi; ps[0].y = sy * mi; ps[0].z = sz * mi;
    ps[0].vx = svx * mi; ps[0].vy = svy * mi; ps[0].vz = svz * mi;
}

static void inertial_to_jacobi_acc(const orc_particle* ps, orc_particle* pj, const orc_particle* pm, size_t N, size_t Na) {
    /* src/transformations.c:147-176 */
    double eta = pm[0].m;
    double sx = eta * ps[0].ax, sy = eta * ps[0].ay, sz = eta * ps[0].az;
    for (size_t i = 1; i < Na; i++) {
        const double ei = 1. / eta;
        const orc_particle pi = ps[i];
        eta += pm[i].m;
        const double pme = eta * ei;
        pj[i].ax = pi.ax - sx * ei; pj[i].ay = pi.ay - sy * ei; pj[i].az = pi.az - sz * ei;
        sx = sx * pme + pm[i].m * pj[i].ax; sy = sy * pme + pm[i].m * pj[i].ay; sz = sz * pme + pm[i].m * pj[i].az;
    }
    const double ei = 1. / eta;
    for (size_t i = Na; i < N; i++) {
        const orc_particle pi = ps[i];
        pj[i].ax = pi.ax - sx * ei; pj[i].ay = pi.ay - sy * ei; pj[i].az = pi.az - sz * ei;
    }
    const double mti = 1. / eta;
    pj[0].ax = sx * mti; pj[0].ay = sy * mti; pj[0].az = sz * mti;
}

/* Democratic heliocentric, WHDS and barycentric coordinates
 * (src/transformations.c:295-644); coordinates = 0 Jacobi, 1 democratic
 * heliocentric, 2 WHDS, 3 barycentric. */
static void inertial_to_helio(const orc_particle* P, orc_particle* h, size_t N, size_t Na, int whds) {
    double x0 = 0., y0 = 0., z0 = 0., vx0 = 0., vy0 = 0., vz0 = 0., m0 = 0.;   /* :388-425, :295-345 */
    for (size_t i = 0; i < Na; i++) {
        const double m = P[i].m;
        x0 += P[i].x * m; y0 += P[i].y * m; z0 += P[i].z * m;
        vx0 += P[i].vx * m; vy0 += P[i].vy * m; vz0 += P[i].vz * m;
        m0 += m;
    }
    h[0].x = x0 / m0; h[0].y = y0 / m0; h[0].z = z0 / m0;
    h[0].vx = vx0 / m0; h[0].vy = vy0 / m0; h[0].vz = vz0 / m0;
    h[0].m = m0;
    const double ms = P[0].m;
    for (size_t i = 1; i < N; i++) {
        h[i].x = P[i].x - P[0].x; h[i].y = P[i].y - P[0].y; h[i].z = P[i].z - P[0].z;
        if (whds && i < Na) {
            const double mf = (ms + P[i].m) / ms;
            h[i].vx = mf * (P[i].vx - h[0].vx); h[i].vy = mf * (P[i].vy - h[0].vy); h[i].vz = mf * (P[i].vz - h[0].vz);
        } else {
            h[i].vx = P[i].vx - h[0].vx; h[i].vy = P[i].vy - h[0].vy; h[i].vz = P[i].vz - h[0].vz;
        }
        h[i].m = P[i].m;
    }
}

static void helio_to_inertial(orc_particle* P, const orc_particle* h, size_t N, size_t Na, int whds) {
    const double mtot = h[0].m;                                      /* :427-473, :347-381 */
    double x0 = 0., y0 = 0., z0 = 0.;
    for (size_t i = 1; i < Na; i++) {
        const double m = h[i].m;
        x0 += h[i].x * m / mtot; y0 += h[i].y * m / mtot; z0 += h[i].z * m / mtot;
        P[i].m = m;
    }
    P[0].x = h[0].x - x0; P[0].y = h[0].y - y0; P[0].z = h[0].z - z0;
    for (size_t i = 1; i < N; i++) {
        P[i].x = h[i].x + P[0].x; P[i].y = h[i].y + P[0].y; P[i].z = h[i].z + P[0].z;
    }
    const double m0 = P[0].m;
    for (size_t i = 1; i < N; i++) {
        if (whds && i < Na) {
            const double mf = (m0 + P[i].m) / m0;
            P[i].vx = h[i].vx / mf + h[0].vx; P[i].vy = h[i].vy / mf + h[0].vy; P[i].vz = h[i].vz / mf + h[0].vz;
        } else {
            P[i].vx = h[i].vx + h[0].vx; P[i].vy = h[i].vy + h[0].vy; P[i].vz = h[i].vz + h[0].vz;
        }
    }
    double vx0 = 0., vy0 = 0., vz0 = 0.;
    for (size_t i = 1; i < Na; i++) {
        const double m = P[i].m;
        if (whds) { vx0 += h[i].vx * m / (m0 + m); vy0 += h[i].vy * m / (m0 + m); vz0 += h[i].vz * m / (m0 + m); }
        else { vx0 += h[i].vx * m / m0; vy0 += h[i].vy * m / m0; vz0 += h[i].vz * m / m0; }
    }
    P[0].vx = h[0].vx - vx0; P[0].vy = h[0].vy - vy0; P[0].vz = h[0].vz - vz0;
}

static void inertial_to_bary(const orc_particle* P, orc_particle* b, size_t N, size_t Na) {   /* :595-644 */
    b[0].x = P[0].m * P[0].x; b[0].y = P[0].m * P[0].y; b[0].z = P[0].m * P[0].z;
    b[0].vx = P[0].m * P[0].vx; b[0].vy = P[0].m * P[0].vy; b[0].vz = P[0].m * P[0].vz;
    b[0].m = P[0].m;
    double sx = 0., sy = 0., sz = 0., svx = 0., svy = 0., svz = 0., sm = 0.;
    for (size_t i = 1; i < Na; i++) {
        const double m = P[i].m;
        b[i].m = m;
        sx += P[i].x * m; sy += P[i].y * m; sz += P[i].z * m;
        svx += P[i].vx * m; svy += P[i].vy * m; svz += P[i].vz * m;
        sm += m;
    }
    b[0].x += sx; b[0].y += sy; b[0].z += sz; b[0].vx += svx; b[0].vy += svy; b[0].vz += svz; b[0].m += sm;
    const double mi = 1.0 / b[0].m;
    b[0].x *= mi; b[0].y *= mi; b[0].z *= mi; b[0].vx *= mi; b[0].vy *= mi; b[0].vz *= mi;
    for (size_t i = 1; i < N; i++) {
        if (i >= Na) b[i].m = P[i].m;
        b[i].x = P[i].x - b[0].x; b[i].y = P[i].y - b[0].y; b[i].z = P[i].z - b[0].z;
        b[i].vx = P[i].vx - b[0].vx; b[i].vy = P[i].vy - b[0].vy; b[i].vz = P[i].vz - b[0].vz;
    }
}

static void bary_to_inertial(orc_particle* P, const orc_particle* b, size_t N, size_t Na) {   /* :544-593 */
    P[0].x = b[0].m * b[0].x; P[0].y = b[0].m * b[0].y; P[0].z = b[0].m * b[0].z;
    P[0].vx = b[0].m * b[0].vx; P[0].vy = b[0].m * b[0].vy; P[0].vz = b[0].m * b[0].vz;
    P[0].m = b[0].m;
    double sx = 0., sy = 0., sz = 0., svx = 0., svy = 0., svz = 0., sm = 0.;
    for (size_t i = 1; i < N; i++) {
        P[i].x = b[i].x + b[0].x; P[i].y = b[i].y + b[0].y; P[i].z = b[i].z + b[0].z;
        P[i].vx = b[i].vx + b[0].vx; P[i].vy = b[i].vy + b[0].vy; P[i].vz = b[i].vz + b[0].vz;
        if (i < Na) {
            const double m = b[i].m;
            P[i].m = m;
            sx += P[i].x * m; sy += P[i].y * m; sz += P[i].z * m;
            svx += P[i].vx * m; svy += P[i].vy * m; svz += P[i].vz * m;
            sm += m;
        }
    }
    P[0].x -= sx; P[0].y -= sy; P[0].z -= sz; P[0].vx -= svx; P[0].vy -= svy; P[0].vz -= svz; P[0].m -= sm;
    const double m0i = 1. / P[0].m;
    P[0].x *= m0i; P[0].y *= m0i; P[0].z *= m0i; P[0].vx *= m0i; P[0].vy *= m0i; P[0].vz *= m0i;
}

/* reb_integrator_whfast_from_inertial / _to_inertial (src/integrator_whfast.c:950-1024) */
static void whfast_from_inertial(orc_sim* r) {
    const size_t N = r->N, Na = wh_active_of(r);
    switch (r->whfast_coordinates) {
        case 1: inertial_to_helio(r->particles, r->p_jh, N, Na, 0); break;
        case 2: inertial_to_helio(r->particles, r->p_jh, N, Na, 1); break;
        case 3: inertial_to_bary(r->particles, r->p_jh, N, Na); break;
        default: orc_inertial_to_jacobi_posvel(r->particles, r->p_jh, r->particles, N, Na);
    }
}

static void whfast_to_inertial(orc_sim* r) {
    const size_t N = r->N, Na = wh_active_of(r);
    switch (r->whfast_coordinates) {
        case 1: helio_to_inertial(r->particles, r->p_jh, N, Na, 0); break;
        case 2: helio_to_inertial(r->particles, r->p_jh, N, Na, 1); break;
        case 3: bary_to_inertial(r->particles, r->p_jh, N, Na); break;
        default: orc_jacobi_to_inertial_posvel(r->particles, r->p_jh, r->particles, N, Na);
    }
}

static void whfast_kepler_step(orc_sim* r, double dt) {           /* :589-636, serial branch */
    const double m0 = r->particles[0].m;
    const size_t N = r->N, Na = wh_active_of(r);
    double eta = m0;
    for (size_t i = 1; i < N; i++) {
        double e;
        switch (r->whfast_coordinates) {
            case 1: e = m0; break;
            case 2: e = i < Na ? m0 + r->p_jh[i].m : m0; break;
            case 3: e = r->p_jh[0].m; break;
            default: if (i < Na) eta += r->p_jh[i].m; e = eta;
        }
        orc_whfast_kepler_solver(&r->p_jh[i], e * r->G, dt);
    }
}

/* reb_integrator_whfast_jump_step (:526-584): democratic heliocentric and WHDS only. */
static void whfast_jump_step(orc_sim* r, double dt) {
    const int c = r->whfast_coordinates;
    if (c != 1 && c != 2) return;
    orc_particle* h = r->p_jh;
    const orc_particle* P = r->particles;
    const size_t N = r->N, Na = wh_active_of(r);
    const double m0 = P[0].m;
    double px = 0., py = 0., pz = 0.;
    for (size_t i = 1; i < Na; i++) {
        const double m = P[i].m;
        if (c == 1) { px += m * h[i].vx; py += m * h[i].vy; pz += m * h[i].vz; }
        else { px += m * h[i].vx / (m0 + m); py += m * h[i].vy / (m0 + m); pz += m * h[i].vz / (m0 + m); }
    }
    for (size_t i = 1; i < N; i++) {
        if (c == 1) {
            h[i].x += dt * (px / m0); h[i].y += dt * (py / m0); h[i].z += dt * (pz / m0);
        } else if (i < Na) {
            const double m = P[i].m;
            h[i].x += dt * (px - (m * h[i].vx / (m0 + m)));
            h[i].y += dt * (py - (m * h[i].vy / (m0 + m)));
            h[i].z += dt * (pz - (m * h[i].vz / (m0 + m)));
        } else {
            h[i].x += dt * px; h[i].y += dt * py; h[i].z += dt * pz;
        }
    }
}

static void whfast_com_step(orc_sim* r, double dt) {              /* :638-651 */
    r->p_jh[0].x += dt * r->p_jh[0].vx;
    r->p_jh[0].y += dt * r->p_jh[0].vy;
    r->p_jh[0].z += dt * r->p_jh[0].vz;
}

static void whfast_interaction_step_jacobi(orc_sim* r, double dt);

static void whfast_interaction_step(orc_sim* r, double dt) {      /* :431-524 */
    const int c = r->whfast_coordinates;
    if (c == 0) { whfast_interaction_step_jacobi(r, dt); return; }
    orc_particle* h = r->p_jh;
    const orc_particle* P = r->particles;
    const size_t N = r->N, Na = wh_active_of(r);
    const double m0 = P[0].m;
    for (size_t i = 1; i < N; i++) {
        if (c == 2 && i < Na) {                                    /* :502-508 */
            const double mi = P[i].m;
            h[i].vx += dt * (m0 + mi) * P[i].ax / m0;
            h[i].vy += dt * (m0 + mi) * P[i].ay / m0;
            h[i].vz += dt * (m0 + mi) * P[i].az / m0;
        } else if (c == 3) {                                       /* :517-524 */
            const double dr = sqrt(h[i].x * h[i].x + h[i].y * h[i].y + h[i].z * h[i].z);
            const double pf = r->G * h[0].m / (dr * dr * dr);
            h[i].vx += dt * (pf * h[i].x + P[i].ax);
            h[i].vy += dt * (pf * h[i].y + P[i].ay);
            h[i].vz += dt * (pf * h[i].z + P[i].az);
        } else {                                                   /* :494-500 */
            h[i].vx += dt * P[i].ax; h[i].vy += dt * P[i].ay; h[i].vz += dt * P[i].az;
        }
    }
}

static void whfast_interaction_step_jacobi(orc_sim* r, double dt) {  /* :431-492 */
    const size_t N = r->N, Na = wh_active_of(r);
    orc_particle* pj = r->p_jh;
    /* kernels MODIFIEDKICK and LAZY run with gravity = JACOBI: the Jacobi term is
     * already in the accelerations (:458) */
    const int jacobi_term = r->whfast_kernel != 1 && r->whfast_kernel != 3;
    inertial_to_jacobi_acc(r->particles, pj, r->particles, N, Na);
    double eta = r->particles[0].m;
    for (size_t i = 1; i < N; i++) {
        const orc_particle q = pj[i];
        if (i < Na) eta += q.m;
        pj[i].vx += dt * q.ax; pj[i].vy += dt * q.ay; pj[i].vz += dt * q.az;
        if (jacobi_term && i > 1) {
            const double rj2i = 1. / (q.x * q.x + q.y * q.y + q.z * q.z);
            const double rji = sqrt(rj2i);
            const double rj3iM = rji * rj2i * r->G * eta;
            const double pf = dt * rj3iM;
            pj[i].vx += pf * q.x; pj[i].vy += pf * q.y; pj[i].vz += pf * q.z;
        }
    }
}

/* reb_gravity_jacobi_calculate_acceleration (src/gravity.c:108-162). */
static void gravity_jacobi(orc_sim* r) {
    orc_particle* const P = r->particles;
    const size_t N = r->N;
    const double G = r->G;
    double Rx = 0., Ry = 0., Rz = 0., M = 0.;
    for (size_t j = 0; j < N; j++) {
        P[j].ax = 0.; P[j].ay = 0.; P[j].az = 0.;
        for (size_t i = 0; i < j + 1; i++) {
            if (j > 1) {
                const double Qx = P[j].x - Rx / M, Qy = P[j].y - Ry / M, Qz = P[j].z - Rz / M;
                const double dr = sqrt(Qx * Qx + Qy * Qy + Qz * Qz);
                const double dQ = i < j ? -P[j].m : M;
                const double pf = G * dQ / (dr * dr * dr);
                P[i].ax += pf * Qx; P[i].ay += pf * Qy; P[i].az += pf * Qz;
            }
            if (i != j && (i != 0 || j != 1)) {
                const double dx = P[i].x - P[j].x, dy = P[i].y - P[j].y, dz = P[i].z - P[j].z;
                const double dr = sqrt(dx * dx + dy * dy + dz * dz);
                const double pf = G / (dr * dr * dr);
                const double pfi = pf * P[i].m, pfj = pf * P[j].m;
                P[i].ax -= pfj * dx; P[i].ay -= pfj * dy; P[i].az -= pfj * dz;
                P[j].ax += pfi * dx; P[j].ay += pfi * dy; P[j].az += pfi * dz;
            }
        }
        Rx += P[j].m * P[j].x; Ry += P[j].m * P[j].y; Rz += P[j].m * P[j].z;
        M += P[j].m;
    }
}

/* reb_simulation_update_acceleration for WHFast: BASIC with the 0-1 pair
 * skipped, or JACOBI for kernels MODIFIEDKICK and LAZY (:929-931). */
static void whfast_update_acceleration(orc_sim* r) {
    if (r->whfast_kernel == 1 || r->whfast_kernel == 3) { gravity_jacobi(r); return; }
    switch (r->whfast_gravity) {                                   /* the simulation's gravity */
        case 1: orc_gravity_compensated_serial(r); break;
        case 2: for (size_t i = 0; i < r->N; i++) r->particles[i].ax = r->particles[i].ay = r->particles[i].az = 0.;
                break;
        default: orc_gravity_basic_serial(r);
    }
}

/* reb_integrator_whfast_calculate_jerk (:786-870) into jx, jy, jz. */
static void whfast_jerk(const orc_sim* r, double* jx, double* jy, double* jz) {
    const orc_particle* const P = r->particles;
    const size_t N = r->N;
    const double G = r->G;
    double Rx = 0., Ry = 0., Rz = 0., M = 0., Ax = 0., Ay = 0., Az = 0.;
    for (size_t j = 0; j < N; j++) {
        jx[j] = 0.; jy[j] = 0.; jz[j] = 0.;
        for (size_t i = 0; i < j + 1; i++) {
            if (j > 1) {
                const double dQ = i < j ? -P[j].m : M;
                const double Qx = P[j].x - Rx / M, Qy = P[j].y - Ry / M, Qz = P[j].z - Rz / M;
                const double dax = P[j].ax - Ax / M, day = P[j].ay - Ay / M, daz = P[j].az - Az / M;
                const double dr = sqrt(Qx * Qx + Qy * Qy + Qz * Qz);
                const double pf2 = G * dQ / (dr * dr * dr);
                jx[i] += pf2 * dax; jy[i] += pf2 * day; jz[i] += pf2 * daz;
                const double alpha = dax * Qx + day * Qy + daz * Qz;
                const double pf1 = 3. * alpha * pf2 / (dr * dr);
                jx[i] -= pf1 * Qx; jy[i] -= pf1 * Qy; jz[i] -= pf1 * Qz;
            }
            if (j != i && (i != 0 || j != 1)) {
                const double dx = P[j].x - P[i].x, dy = P[j].y - P[i].y, dz = P[j].z - P[i].z;
                const double dax = P[j].ax - P[i].ax, day = P[j].ay - P[i].ay, daz = P[j].az - P[i].az;
                const double dr = sqrt(dx * dx + dy * dy + dz * dz);
                const double alpha = dax * dx + day * dy + daz * dz;
                const double pf2 = G / (dr * dr * dr);
                const double pf2i = pf2 * P[i].m, pf2j = pf2 * P[j].m;
                jx[j] -= dax * pf2i; jy[j] -= day * pf2i; jz[j] -= daz * pf2i;
                jx[i] += dax * pf2j; jy[i] += day * pf2j; jz[i] += daz * pf2j;
                const double pf1 = 3. * alpha * pf2 / (dr * dr);
                const double pf1i = pf1 * P[i].m, pf1j = pf1 * P[j].m;
                jx[j] += dx * pf1i; jy[j] += dy * pf1i; jz[j] += dz * pf1i;
                jx[i] -= dx * pf1j; jy[i] -= dy * pf1j; jz[i] -= dz * pf1j;
            }
        }
        Ax += P[j].ax * P[j].m; Ay += P[j].ay * P[j].m; Az += P[j].az * P[j].m;
        Rx += P[j].x * P[j].m; Ry += P[j].y * P[j].m; Rz += P[j].z * P[j].m;
        M += P[j].m;
    }
}

/* Corrector coefficients (src/integrator_whfast.c:124-158). */
static const double corr_a[9] = {0.,
    0.41833001326703777398908601289259374469640768464934,
    0.83666002653407554797817202578518748939281536929867,
    1.2549900398011133219672580386777812340892230539480,
    1.6733200530681510959563440515703749787856307385973,
    2.0916500663351888699454300644629687234820384232467,
    2.5099800796022266439345160773555624681784461078960,
    2.9283100928692644179236020902481562128748537925454,
    3.3466401061363021919126881031407499575712614771947};
static const double corr_b3[1] = {-0.024900596027799867499350357910273437184309981229127};
static const double corr_b5[2] = {-0.0083001986759332891664501193034244790614366604097090,
                                  0.041500993379666445832250596517122395307183302048545};
static const double corr_b7[3] = {0.0024926811426922105779030593952776964450539008582219,
                                  -0.018270923246702131478062356884535264841652263842597,
                                  0.053964399093127498721765893493510877532452806339655};
static const double corr_b11[5] = {0.00020361579647854651301632818774633716473696537436847,
                                   -0.0023487215292295354188307328851055489876255097419754,
                                   0.012309078592019946317544564763237909911330686448336,
                                   -0.038121613681288650508647613260247372125243616270670,
                                   0.072593394748842738674253180742744961827622366521517};
static const double corr_b17[8] = {-0.0000043347415473373580190650223498124944896789841432241,
                                   0.000076436355227935738363241846979413475106795392377415,
                                   -0.00063599983075817658983166881625078545864140848560259,
                                   0.0033132577069380655655490196833451994080066801611459,
                                   -0.012071760822342291062449751726959664253913904872527,
                                   0.032422198864713580293681523029577130832258806467604,
                                   -0.065192863576377893658290760803725762027864651086787,
                                   0.093056103771425958591541059067553547100903397724386};
static const double corr2_b = 0.03486083443891981449909050107438281205803;

/* Jacobi -> inertial, then the accelerations, then a kick of dt. */
static void whfast_evaluate_kick(orc_sim* r, double dt) {
    whfast_to_inertial(r);
    whfast_update_acceleration(r);
    whfast_interaction_step(r, dt);
}

static void corrector_z(orc_sim* r, double a, double b) {          /* :653-694 */
    whfast_kepler_step(r, a);
    whfast_evaluate_kick(r, -b);
    whfast_kepler_step(r, -2. * a);
    whfast_evaluate_kick(r, b);
    whfast_kepler_step(r, a);
}

static void apply_corrector(orc_sim* r, double inv, int order) {   /* :696-751 */
    const double dt = r->dt;
    if (order == 3) {
        corrector_z(r, corr_a[1] * dt, -inv * corr_b3[0] * dt);
        corrector_z(r, -corr_a[1] * dt, inv * corr_b3[0] * dt);
        return;
    }
    const double* b = order == 5 ? corr_b5 : order == 7 ? corr_b7 : order == 11 ? corr_b11 : corr_b17;
    const int h = order == 5 ? 2 : order == 7 ? 3 : order == 11 ? 5 : 8;
    for (int k = 0; k < h; k++) corrector_z(r, -corr_a[h - k] * dt, -inv * b[k] * dt);
    for (int k = h - 1; k >= 0; k--) corrector_z(r, corr_a[h - k] * dt, inv * b[k] * dt);
}

static void operator_c(orc_sim* r, double a, double b) {           /* :753-768 */
    whfast_kepler_step(r, a);
    whfast_evaluate_kick(r, b);
    whfast_kepler_step(r, -a);
}
static void operator_y(orc_sim* r, double a, double b) { operator_c(r, a, b); operator_c(r, -a, -b); }
static void operator_u(orc_sim* r, double a, double b) {
    whfast_kepler_step(r, a);
    operator_y(r, a, b);
    operator_y(r, a, -b);
    whfast_kepler_step(r, -a);
}
static void apply_corrector2(orc_sim* r, double inv) {             /* :779-785 */
    const double a = 0.5 * inv * r->dt;
    const double b = corr2_b * inv * r->dt;
    operator_u(r, a, b);
    operator_u(r, -a, b);
}

void orc_whfast_synchronize(orc_sim* r) {                         /* :1051-1111 */
    if (r->whfast_is_synchronized == 0) {
        orc_particle* keep = NULL;
        if (r->whfast_keep_unsynchronized) {
            keep = (orc_particle*)malloc(sizeof(orc_particle) * r->N);
            memcpy(keep, r->p_jh, sizeof(orc_particle) * r->N);
        }
        const double d = r->whfast_kernel == 2 ? 3. * r->dt / 8. : r->dt / 2.;
        whfast_kepler_step(r, d);
        whfast_com_step(r, d);
        if (r->whfast_corrector2) apply_corrector2(r, -1.);
        if (r->whfast_corrector) apply_corrector(r, -1., r->whfast_corrector);
        whfast_to_inertial(r);
        if (keep) {
            memcpy(r->p_jh, keep, sizeof(orc_particle) * r->N);
            free(keep);
        } else {
            r->whfast_is_synchronized = 1;
        }
    }
}

void orc_whfast_step(orc_sim* r) {                                /* :1113-1259 */
    const double dt = r->dt;
    const size_t N = r->N, Na = wh_active_of(r);
    const int coords = r->whfast_coordinates;
    r->gravity_ignore_terms = coords == 0 ? 1 : coords == 3 ? 0 : 2;   /* :929-938 */
    if (r->whfast_safe_mode || r->whfast_did_modify) {
        if (r->whfast_is_synchronized == 0) orc_whfast_synchronize(r);
        whfast_from_inertial(r);
        r->whfast_did_modify = 0;
    }
    if (r->whfast_is_synchronized) {
        if (r->whfast_corrector) apply_corrector(r, 1., r->whfast_corrector);
        if (r->whfast_corrector2) apply_corrector2(r, 1.);
        const double d = r->whfast_kernel == 2 ? 5. * dt / 8. : dt / 2.;
        whfast_kepler_step(r, d);
        whfast_com_step(r, d);
    } else {
        whfast_kepler_step(r, dt);
        whfast_com_step(r, dt);
    }
    whfast_jump_step(r, dt / 2.);
    whfast_to_inertial(r);
    r->t += dt / 2.;
    whfast_update_acceleration(r);
    switch (r->whfast_kernel) {
        case 1: {                                                  /* MODIFIEDKICK (:1192-1203) */
            double* j = (double*)malloc(sizeof(double) * 3 * N);
            whfast_jerk(r, j, j + N, j + 2 * N);
            const double pf = dt * dt / 12.;
            for (size_t i = 0; i < N; i++) {
                r->particles[i].ax += pf * j[i];
                r->particles[i].ay += pf * j[N + i];
                r->particles[i].az += pf * j[2 * N + i];
            }
            free(j);
            whfast_interaction_step(r, dt);
            break;
        }
        case 2:                                                    /* COMPOSITION (:1205-1231) */
            whfast_interaction_step(r, -dt / 6.);
            whfast_kepler_step(r, -dt / 4.); whfast_com_step(r, -dt / 4.);
            whfast_evaluate_kick(r, dt / 6.);
            whfast_kepler_step(r, dt / 8.); whfast_com_step(r, dt / 8.);
            whfast_evaluate_kick(r, dt);
            whfast_kepler_step(r, -dt / 8.); whfast_com_step(r, -dt / 8.);
            whfast_evaluate_kick(r, -dt / 6.);
            whfast_kepler_step(r, dt / 4.); whfast_com_step(r, dt / 4.);
            whfast_evaluate_kick(r, dt / 6.);
            break;
        case 3: {                                                  /* LAZY (:1233-1247) */
            const double pf = dt * dt / 12.;
            for (size_t i = 1; i < N; i++) {
                r->particles[i].x += pf * r->particles[i].ax;
                r->particles[i].y += pf * r->particles[i].ay;
                r->particles[i].z += pf * r->particles[i].az;
            }
            whfast_update_acceleration(r);
            whfast_interaction_step(r, dt);
            break;
        }
        default:                                                   /* DEFAULT */
            whfast_interaction_step(r, dt);
            whfast_jump_step(r, dt / 2.);
    }
    r->whfast_is_synchronized = 0;
    if (r->whfast_safe_mode) orc_whfast_synchronize(r);
    r->t += dt / 2.;
}

/* n WHFast steps in a row (one foreign call for a whole timing sample). */
void orc_whfast_steps(orc_sim* r, long n) {
    for (long k = 0; k < n; k++) orc_whfast_step(r);
}

/* ------------------------------------------------------------------------
 * Energy: src/tools.c:108-162 (no softening, test-particle aware).
 * ---------------------------------------------------------------------- */
double orc_energy(const orc_sim* r) {
    const size_t N = r->N, Na = n_active_of(r);
    const orc_particle* P = r->particles;
    const size_t Ni = r->testparticle_type == 0 ? Na : N;
    double ek = 0., ep = 0.;
    for (size_t i = 0; i < Ni; i++)
        ek += 0.5 * P[i].m * (P[i].vx * P[i].vx + P[i].vy * P[i].vy + P[i].vz * P[i].vz);
    for (size_t i = 0; i < Na; i++) {
        const orc_particle pi = P[i];
        for (size_t j = i + 1; j < Ni; j++) {
            const double dx = pi.x - P[j].x, dy = pi.y - P[j].y, dz = pi.z - P[j].z;
            ep -= r->G * P[j].m * pi.m / sqrt(dx * dx + dy * dy + dz * dz);
        }
    }
    return ek + ep;
}

/* ------------------------------------------------------------------------
 * Seeded Plummer sphere: reb_simulation_add_plummer (src/tools.c:463-502)
 * with the reference RNG (reb_random_uniform, src/tools.c:64-75, glibc rand_r),
 * keeping in draw order only particles with r <= rmax; masses M/N.
 * ---------------------------------------------------------------------- */
static double orc_uniform(unsigned int* seed, double lo, double hi) {
    return ((double)rand_r(seed)) / ((double)RAND_MAX) * (hi - lo) + lo;
}

void orc_ic_plummer(unsigned int seed, size_t N, double M, double R, double rmax, orc_particle* out) {
    const double E = 3. / 64. * M_PI * M * M / R;
    size_t n = 0;
    while (n < N) {
        const double rr = pow(pow(orc_uniform(&seed, 0, 1), -2. / 3.) - 1., -1. / 2.);
        const double x2 = orc_uniform(&seed, 0, 1);
        const double x3 = orc_uniform(&seed, 0, 2. * M_PI);
        orc_particle p;
        memset(&p, 0, sizeof(p));
        p.z = (1. - 2. * x2) * rr;
        p.x = sqrt(rr * rr - p.z * p.z) * cos(x3);
        p.y = sqrt(rr * rr - p.z * p.z) * sin(x3);
        double x5, g, q;
        do {
            x5 = orc_uniform(&seed, 0., 1.);
            q = orc_uniform(&seed, 0., 1.);
            g = q * q * pow(1. - q * q, 7. / 2.);
        } while (0.1 * x5 > g);
        const double ve = pow(2., 1. / 2.) * pow(1. + rr * rr, -1. / 4.);
        const double v = q * ve;
        const double x6 = orc_uniform(&seed, 0., 1.);
        const double x7 = orc_uniform(&seed, 0., 2. * M_PI);
        p.vz = (1. - 2. * x6) * v;
        p.vx = sqrt(v * v - p.vz * p.vz) * cos(x7);
        p.vy = sqrt(v * v - p.vz * p.vz) * sin(x7);
        p.x *= 3. * M_PI / 64. * M * M / E;
        p.y *= 3. * M_PI / 64. * M * M / E;
        p.z *= 3. * M_PI / 64. * M * M / E;
        p.vx *= sqrt(E * 64. / 3. / M_PI / M);
        p.vy *= sqrt(E * 64. / 3. / M_PI / M);
        p.vz *= sqrt(E * 64. / 3. / M_PI / M);
        if (sqrt(p.x * p.x + p.y * p.y + p.z * p.z) > rmax) continue;
        p.m = M / (double)N;
        out[n++] = p;
    }
}

/* Rows [i0, i1) of the OpenMP COMPENSATED gather (src/gravity.c:308-343),
 * no ghost boxes, all particles active: an accurate reference for a sample of
 * rows at sizes where the full O(N^2) sum is too slow on the host. */
void orc_gravity_compensated_omp_rows(orc_sim* r, size_t i0, size_t i1) {
    orc_particle* const P = r->particles;
    const size_t N = r->N;
    const double G = r->G, eps2 = r->softening * r->softening;
    if (i1 > N) i1 = N;
#pragma omp parallel for schedule(guided)
    for (size_t i = i0; i < i1; i++) {
        double ax = 0., ay = 0., az = 0., cx = 0., cy = 0., cz = 0.;
        for (size_t j = 0; j < N; j++) {
            if (i == j) continue;
            const double dx = P[i].x - P[j].x, dy = P[i].y - P[j].y, dz = P[i].z - P[j].z;
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            const double rr = sqrt(r2);
            const double pf = G / (r2 * rr);
            const double pfj = -pf * P[j].m;
            KAHAN_ADD(ax, cx, pfj * dx);
            KAHAN_ADD(ay, cy, pfj * dy);
            KAHAN_ADD(az, cz, pfj * dz);
        }
        P[i].ax = ax; P[i].ay = ay; P[i].az = az;
    }
}

/* Tree gravity (src/gravity.c:47-106) for rows [i0, i1) only: same tree and
 * walk, so a sample of particles can be checked at sizes where the full walk
 * is too slow on the host. */
void orc_gravity_tree_rows(orc_sim* r, size_t i0, size_t i1) {
    otree t = {0};
    if (tree_build(r, &t)) { tree_free(&t); return; }
    for (size_t i = 0; i < t.n_root; i++) if (t.root[i]) cell_gravity_data(r, t.root[i]);
    orc_particle* const P = r->particles;
    if (i1 > r->N) i1 = r->N;
#pragma omp parallel for schedule(dynamic)
    for (size_t i = i0; i < i1; i++) {
        double ax = 0., ay = 0., az = 0.;
        for (int gx = -r->N_ghost_x; gx <= r->N_ghost_x; gx++)
        for (int gy = -r->N_ghost_y; gy <= r->N_ghost_y; gy++)
        for (int gz = -r->N_ghost_z; gz <= r->N_ghost_z; gz++) {
            double gb[6];
            orc_boundary_ghostbox(r, gx, gy, gz, gb);
            const double sx = gb[0] + P[i].x, sy = gb[1] + P[i].y, sz = gb[2] + P[i].z;
            for (size_t k = 0; k < t.n_root; k++)
                if (t.root[k]) cell_accel(r, (long)i, t.root[k], sx, sy, sz, &ax, &ay, &az);
        }
        P[i].ax = ax; P[i].ay = ay; P[i].az = az;
    }
    tree_free(&t);
}
