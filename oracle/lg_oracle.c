/*
 * lg_oracle.c -- CPU FP64 restatement of libgran's pair-force + integration hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the oracle that the GPU engine is checked against and
 * the CPU baseline that bench.py times beside it. Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load it. The product (libgran_gb300) never links, loads or calls it.
 *
 * What it restates (paths inside the libgran project):
 *   contact_force_functor::operator()             contact_force/contact_force.h:57-96
 *   contact_force_functor::compute_shear_contribution contact_force/contact_force.h:105-147
 *   alt_sinter_functor (ctor bond detection, bonded branch)  sinter_bridge/alt_sinter_bridge.h:19-156
 *   alt_breaking_sinter_functor                   sinter_bridge/alt_breaking_sinter_bridge.h:17-131
 *   sinter_functor (ctor connectors, bonded branch) sinter_bridge/sinter_bridge.h:100-268
 *   sinter_step_handler (connector increments)     sinter_bridge/sinter_bridge.h:14-94
 *   hamaker_functor                               hamaker_force/hamaker_force.h:28-43
 *   limited_range_hamaker_functor                 hamaker_force/limited_range_hamaker_force.h:29-47
 *   simplified_hamaker_functor                    hamaker_force/simplified_hamaker_force.h:18-31
 *   surface_contact_force_functor                 contact_force/surface_contact_force.h:57-145
 *   surface_hamaker_functor                       hamaker_force/surface_hamaker_force.h:18-30
 *   triangular_facet (closest point, fold, move)  surface_force/triangular_facet.h:18-137
 *   binary/unary functor container folds          granular_system/binary_force_container.h:20-32,
 *                                                 granular_system/unary_force_container.h:20-32
 *                                                 (a right fold: f0 + (f1 + (... + fN)))
 *   central_attraction_functor (body force)       Custom-unary-force-model.md:108-118
 *   fixed_particle_step_handler (held increments) Custom-step-handler.md:82-97
 *   observables                                   test/compute_energy.cpp:7-58,
 *                                                 test/mass_distribution.cpp:7-27
 * The system loop and the rotational velocity-Verlet integrator live in libtimestep, which the
 * libgran tree references as a git submodule but does not contain. They are restated here from
 * the textbook kick-drift-kick scheme and libgran's documentation of the loop (Overview.md:26-45)
 * and step-handler increments (Custom-step-handler.md:82-145):
 *
 *   construction:  (a, alpha) = F(x0, v0, theta0, omega0)          one force evaluation
 *   do_step(dt):   v += a*(dt/2);  omega += alpha*(dt/2)            half kick
 *                  x += v*dt;      theta += omega*dt                drift (per particle: x, then
 *                                                                   theta; with the 5-connector
 *                                                                   sinter model these are the step
 *                                                                   handler's increment_x and
 *                                                                   increment_theta)
 *                  (a, alpha) = F(x, v, theta, omega)               one force evaluation
 *                  v += a*(dt/2);  omega += alpha*(dt/2)            half kick
 *   F: for each i, acc = 0; for each j != i in ascending order (or in i's Verlet row, ascending):
 *      acc += fold_of_binary_functors(i, j); then acc += fold_of_unary_functors(i).
 *
 * Vector arithmetic follows Eigen's component-wise semantics: norm() = sqrt((x*x + y*y) + z*z),
 * normalized() = v / norm (v itself when the squared norm is 0), dot = (x*x' + y*y') + z*z'.
 * Build with -ffp-contract=off so that no multiply-add is fused.
 */
#include "lg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------------------------------------
 * 3-vectors with Eigen's evaluation order
 * ------------------------------------------------------------------------------------------- */
typedef struct { double x, y, z; } v3;

static inline v3 mk(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static inline v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 scl(double s, v3 a) { return mk(s * a.x, s * a.y, s * a.z); }
static inline v3 dvs(v3 a, double s) { return mk(a.x / s, a.y / s, a.z / s); }
static inline v3 neg(v3 a) { return mk(-a.x, -a.y, -a.z); }
static inline double dot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline double sqn(v3 a) { return (a.x * a.x + a.y * a.y) + a.z * a.z; }
static inline double nrm(v3 a) { return sqrt(sqn(a)); }
static inline v3 nrmz(v3 a) {
    double z = sqn(a);
    if (z > 0.0) return dvs(a, sqrt(z));
    return a;
}
static inline v3 crs(v3 a, v3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static const v3 ZERO = {0.0, 0.0, 0.0};

static inline v3 ld(const double *p, int64_t i) { return mk(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
static inline void stv(double *p, int64_t i, v3 a) { p[3 * i] = a.x; p[3 * i + 1] = a.y; p[3 * i + 2] = a.z; }

/* ---------------------------------------------------------------------------------------------
 * System state
 * ------------------------------------------------------------------------------------------- */
typedef struct {
    int32_t j;
    v3 xi[3]; /* contact springs (contact functor, or the sintered functor's inner contact copy) */
} entry;

typedef struct {
    int32_t j;
    int32_t intact;  /* bonded_contacts[i*n+j] */
    double strength; /* neck strength read for (i, j) */
    v3 xi[3];        /* alt_sinter contact_springs[i*n+j] (bond springs) */
    v3 cn[5];        /* sinter_functor spring_connectors[i*n+j]: the five connectors on particle i */
    int32_t rev;     /* index of the bond (j, i) in row j (5-connector model) */
} bond;

typedef struct {
    entry *e;
    int32_t n, cap;
    bond *b;
    int32_t nb;
} row;

struct lgo_system {
    lg_system_desc d;
    int64_t n;
    double *x, *v, *th, *om, *a, *al; /* AoS double[3n] */
    row *rows;
    lg_facet_desc *facets;
    double *facet_area;   /* [nf] */
    double *facet_normal; /* [3nf] */
    v3 *surf_xi;          /* [nf * n * 3] surface contact springs, surface_contact_force.h:53-54 */
    int64_t step_index;
    int64_t n_bonds_initial;
    int threads;
    uint8_t *hold;        /* [n] LG_HOLD_* bits, or NULL */
    double centre[3];     /* LG_BODY_CENTRAL centre */
};

/* ---------------------------------------------------------------------------------------------
 * Shear contributions
 * ------------------------------------------------------------------------------------------- */

/* contact_force.h:105-147 (also surface_contact_force.h:103-145): rotate the spring onto the
 * tangent plane keeping its magnitude, test force, Coulomb static/dynamic choice. */
static v3 shear_coulomb(v3 *xi, v3 n, double stiffness, double damping, double normal_force,
                        double mu_static, double phi_dynamic, v3 rel, double dt) {
    double mu_dynamic = mu_static * phi_dynamic;
    v3 xi_new = sub(*xi, scl(dot(*xi, n), n));
    if (nrm(xi_new) > 0.0) {
        double z = sqn(xi_new);
        if (z > 0.0) xi_new = dvs(xi_new, sqrt(z)); /* normalize() */
        double old = nrm(*xi);
        xi_new = scl(old, xi_new); /* *= xi.norm() (component * scalar, same product) */
    }
    *xi = xi_new;
    v3 f0 = sub(scl(-stiffness, *xi), scl(damping, rel));
    double static_friction = mu_static * normal_force;
    double dynamic_friction = mu_dynamic * normal_force;
    v3 t;
    if (nrm(f0) > 0.0)
        t = nrmz(f0);
    else
        t = ZERO;
    double f_selected;
    if (nrm(f0) <= static_friction) {
        *xi = add(*xi, scl(dt, rel)); /* rel * dt */
        f_selected = static_friction;
    } else {
        *xi = scl(-1.0 / stiffness, add(scl(dynamic_friction, t), scl(damping, rel)));
        f_selected = dynamic_friction;
    }
    double f0n = nrm(f0);
    double m = (f0n < f_selected) ? f0n : f_selected; /* std::min(f_selected, f0n) */
    return scl(m, t);
}

/* alt_sinter_bridge.h:137-156: same rotation, uncapped test force, spring always stretches. */
static v3 shear_bond(v3 *xi, v3 n, double stiffness, double damping, v3 rel, double dt) {
    v3 xi_new = sub(*xi, scl(dot(*xi, n), n));
    if (nrm(xi_new) > 0.0) {
        double z = sqn(xi_new);
        if (z > 0.0) xi_new = dvs(xi_new, sqrt(z));
        double old = nrm(*xi);
        xi_new = scl(old, xi_new);
    }
    *xi = xi_new;
    v3 f0 = sub(scl(-stiffness, *xi), scl(damping, rel));
    *xi = add(*xi, scl(dt, rel));
    return f0;
}

/* ---------------------------------------------------------------------------------------------
 * Binary functors. Each writes (translational acc, angular acc) of particle i due to j.
 * ------------------------------------------------------------------------------------------- */

/* contact_force.h:57-96 */
static void contact_functor(const lg_contact_params *p, v3 xi_, v3 xj_, v3 vi, v3 vj, v3 wi, v3 wj,
                            v3 *springs, v3 *oa, v3 *oal) {
    v3 dx = sub(xi_, xj_);
    v3 n = nrmz(dx);
    double overlap = 2.0 * p->r_part - dot(dx, n);
    if (overlap <= 0) {
        springs[0] = springs[1] = springs[2] = ZERO; /* reset_springs, :99-101 */
        *oa = ZERO;
        *oal = ZERO;
        return;
    }
    double rp = p->r_part - overlap / 2.0;
    double v_n = -dot(sub(vi, vj), n);
    double f_n = p->k * overlap + p->gamma_n * v_n;
    v3 nwi = crs(n, wi), nwj = crs(n, wj);
    v3 v_ij = add(add(sub(vi, vj), scl(rp, nwi)), scl(rp, nwj));
    v3 v_t = sub(v_ij, scl(dot(v_ij, n), n));
    v3 v_r = scl(-rp, sub(nwi, nwj));
    v3 v_o = scl(p->r_part * (dot(n, wi) - dot(n, wj)), n);
    v3 f_t = shear_coulomb(&springs[0], n, p->k_t, p->gamma_t, f_n, p->mu_s, p->phi_d, v_t, p->dt);
    v3 f_r = shear_coulomb(&springs[1], n, p->k_r, p->gamma_r, f_n, p->mu_r, p->phi_r, v_r, p->dt);
    v3 f_o = shear_coulomb(&springs[2], n, p->k_o, p->gamma_o, f_n, p->mu_o, p->phi_o, v_o, p->dt);
    v3 tau_t = scl(rp, crs(n, f_t));
    v3 tau_r = scl(p->r_part, crs(n, f_r));
    v3 tau_o = scl(p->r_part, f_o);
    *oa = dvs(add(scl(f_n, n), f_t), p->mass);
    *oal = dvs(add(add(neg(tau_t), tau_r), tau_o), p->inertia);
}

/* alt_sinter_bridge.h:103-128 and alt_breaking_sinter_bridge.h:89-121 (bonded branch).
 * Returns 1 when the breaking variant decides to break the (i, j) bond. */
static int bond_functor(const lg_sinter_params *p, v3 xi_, v3 xj_, v3 vi, v3 vj, v3 wi, v3 wj,
                        v3 *springs, int breaking, double strength, v3 *oa, v3 *oal) {
    v3 dx = sub(xi_, xj_);
    v3 n = nrmz(dx);
    double overlap = 2.0 * p->r_part - dot(dx, n);
    double rp = p->r_part - overlap / 2.0;
    double v_n = -dot(sub(vi, vj), n);
    double f_n = p->k * overlap + p->gamma_n * v_n;
    v3 nwi = crs(n, wi), nwj = crs(n, wj);
    v3 v_ij = add(add(sub(vi, vj), scl(rp, nwi)), scl(rp, nwj));
    v3 v_t = sub(v_ij, scl(dot(v_ij, n), n));
    v3 v_r = scl(-rp, sub(nwi, nwj));
    v3 v_o = scl(p->r_part * (dot(n, wi) - dot(n, wj)), n);
    v3 f_t = shear_bond(&springs[0], n, p->k_t, p->gamma_t, v_t, p->dt);
    v3 f_r = shear_bond(&springs[1], n, p->k_r, p->gamma_r, v_r, p->dt);
    v3 f_o = shear_bond(&springs[2], n, p->k_o, p->gamma_o, v_o, p->dt);
    v3 tau_t = scl(rp, crs(n, f_t));
    v3 tau_r = scl(p->r_part, crs(n, f_r));
    v3 tau_o = scl(p->r_part, f_o);
    v3 f_tot = add(scl(f_n, n), f_t);
    v3 tau_tot = add(add(neg(tau_t), tau_r), tau_o);
    int brk = 0;
    if (breaking && nrm(f_tot) > strength) brk = 1; /* alt_breaking_sinter_bridge.h:118-119 */
    *oa = dvs(f_tot, p->mass);
    *oal = dvs(tau_tot, p->inertia);
    return brk;
}

/* sinter_functor::bonded_contact_accelerations, sinter_bridge.h:238-266: five connector springs
 * between the connectors of i (ci) and of j (cj); rest lengths 2 r for the four side springs and 0
 * for the centre spring (sinter_bridge.h:201-206). */
static void connector_functor(const lg_connector_params *cp, double r, double mass, double inertia, v3 xi_, v3 xj_,
                              v3 vi, v3 vj, v3 wi, v3 wj, const v3 *ci, const v3 *cj, v3 *pa, v3 *pal) {
    v3 force = ZERO, torque = ZERO;
    for (int k = 0; k < 5; ++k) {
        v3 spring = sub(cj[k], ci[k]);
        double len = nrm(spring);
        double eq = k < 4 ? 2.0 * r : 0.0;
        v3 cvi = add(vi, crs(wi, sub(ci[k], xi_)));
        v3 cvj = add(vj, crs(wj, sub(cj[k], xj_)));
        v3 rel = sub(cvj, cvi);
        v3 df = add(scl(-(eq - len) * cp->k_d, nrmz(spring)), scl(cp->gamma_d, rel));
        force = add(force, df);
        torque = add(torque, crs(sub(ci[k], xi_), df));
    }
    *pa = dvs(force, mass);
    *pal = dvs(torque, inertia);
}

static inline double square_(double x) { return x * x; }
static inline double cube_(double x) { return x * x * x; }

/* hamaker_force.h:28-43 (mode FULL), limited_range_hamaker_force.h:29-47 (LIMITED),
 * simplified_hamaker_force.h:18-31 (SIMPLIFIED). Angular part is zero. */
static v3 hamaker_functor(int mode, const lg_hamaker_params *p, v3 xi_, v3 xj_) {
    if (mode == LG_HAMAKER_LIMITED) {
        if (nrm(sub(xi_, xj_)) > p->r_cutoff) return ZERO;
    }
    v3 r = sub(xj_, xi_);
    double h = nrm(r) - 2.0 * p->r_part;
    if (h < p->h0) h = p->h0;
    double rp = p->r_part;
    double s;
    if (mode == LG_HAMAKER_SIMPLIFIED) {
        s = 2.0 * p->A * rp / square_(h);
    } else {
        double br = (4.0 * rp + 2.0 * h) / (4.0 * rp + h) / h
                    - 2.0 / (2.0 * rp + h)
                    - 4.0 * square_(rp) / cube_(2.0 * rp + h)
                    - 2.0 * square_(rp) * (4.0 * rp + 2.0 * h) / square_(4.0 * rp + h) / square_(h);
        s = -p->A / 6.0 * br;
    }
    v3 f = scl(s, nrmz(r));
    return dvs(f, p->mass);
}

/* ---------------------------------------------------------------------------------------------
 * Unary functors: triangular facet with surface contact and surface Hamaker
 * ------------------------------------------------------------------------------------------- */

/* triangular_facet.h:73-137 */
static v3 closest_point_on_triangle(const double *vt, double area, v3 N, v3 p) {
    v3 v0 = mk(vt[0], vt[1], vt[2]), v1 = mk(vt[3], vt[4], vt[5]), v2 = mk(vt[6], vt[7], vt[8]);
    v3 off = scl(dot(v0, N), N);
    v3 proj = sub(p, scl(dot(p, N), N));
    v3 cp = add(proj, off);
    double s = 0.0;
    v3 pa = sub(v0, cp), pb = sub(v1, cp), pc = sub(v2, cp);
    s += 1.0 / 2.0 * nrm(crs(pa, pb));
    s += 1.0 / 2.0 * nrm(crs(pb, pc));
    s += 1.0 / 2.0 * nrm(crs(pc, pa));
    if (!(s > area)) return cp;
    v3 vv[3] = {v0, v1, v2};
    v3 e[3];
    for (int k = 0; k < 3; ++k) {
        v3 a = vv[k], b = vv[(k + 1) % 3];
        v3 L = sub(b, a);
        v3 uL = nrmz(L);
        v3 tp = sub(p, a);
        double len = nrm(L);
        double pr = dot(tp, uL);
        if (pr < 0.0)
            e[k] = a;
        else if (pr > len)
            e[k] = b;
        else
            e[k] = add(a, scl(pr, uL));
    }
    double d1 = sqn(sub(p, e[0])), d2 = sqn(sub(p, e[1])), d3 = sqn(sub(p, e[2]));
    if (d1 < d2) {
        if (d1 < d3) return e[0];
    } else {
        if (d2 < d3) return e[1];
    }
    return e[2];
}

/* surface_contact_force.h:57-96 */
static void surface_contact(const lg_contact_params *p, v3 xf, v3 vf, v3 xi_, v3 vi, v3 wi, v3 *springs,
                            v3 *oa, v3 *oal) {
    v3 dx = sub(xi_, xf);
    v3 n = nrmz(dx);
    double overlap = p->r_part - dot(dx, n);
    if (overlap <= 0) {
        springs[0] = springs[1] = springs[2] = ZERO;
        *oa = ZERO;
        *oal = ZERO;
        return;
    }
    double rp = p->r_part - overlap;
    double v_n = -dot(sub(vi, vf), n);
    double f_n = p->k * overlap + p->gamma_n * v_n;
    v3 nwi = crs(n, wi);
    v3 v_ij = add(sub(vi, vf), scl(rp, nwi));
    v3 v_t = sub(v_ij, scl(dot(v_ij, n), n));
    v3 v_r = scl(-rp, nwi);
    v3 v_o = scl(p->r_part * dot(n, wi), n);
    v3 f_t = shear_coulomb(&springs[0], n, p->k_t, p->gamma_t, f_n, p->mu_s, p->phi_d, v_t, p->dt);
    v3 f_r = shear_coulomb(&springs[1], n, p->k_r, p->gamma_r, f_n, p->mu_r, p->phi_r, v_r, p->dt);
    v3 f_o = shear_coulomb(&springs[2], n, p->k_o, p->gamma_o, f_n, p->mu_o, p->phi_o, v_o, p->dt);
    v3 tau_t = scl(rp, crs(n, f_t));
    v3 tau_r = scl(p->r_part, crs(n, f_r));
    v3 tau_o = scl(p->r_part, f_o);
    *oa = dvs(add(scl(f_n, n), f_t), p->mass);
    *oal = dvs(add(add(neg(tau_t), tau_r), tau_o), p->inertia);
}

/* surface_hamaker_force.h:18-30 */
static v3 surface_hamaker(const lg_hamaker_params *p, v3 xf, v3 xi_) {
    v3 r = sub(xf, xi_);
    double h = nrm(r) - p->r_part;
    if (h < p->h0) h = p->h0;
    double s = 2.0 * p->A / 3.0 * (cube_(p->r_part) / square_(h) / square_(h + 2.0 * p->r_part));
    return dvs(scl(s, nrmz(r)), p->mass);
}

/* ---------------------------------------------------------------------------------------------
 * Construction helpers
 * ------------------------------------------------------------------------------------------- */
static int cmp_i32(const void *a, const void *b) {
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

static bond *find_bond(row *r, int32_t j) {
    int lo = 0, hi = r->nb - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        if (r->b[mid].j == j) return &r->b[mid];
        if (r->b[mid].j < j) lo = mid + 1; else hi = mid - 1;
    }
    return NULL;
}

static entry *find_entry(entry *e, int32_t n, int32_t j) {
    int lo = 0, hi = n - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        if (e[mid].j == j) return &e[mid];
        if (e[mid].j < j) lo = mid + 1; else hi = mid - 1;
    }
    return NULL;
}

typedef struct { int32_t i, j; } ipair;

/* Bond detection in the order of the reference double loop, alt_sinter_bridge.h:67-89 (cycle
 * prevention by subset relabelling) and alt_breaking_sinter_bridge.h:65-76 (no cycle check).
 * The test is |(|x_i - x_j| - 2 r)| < critical_separation. */
static int64_t detect_bonds(const lg_system_desc *d, const double *x0, int64_t n, ipair **out) {
    const double r = d->sinter.r_part, dc = d->sinter.critical_separation;
    int cyc = (d->binary_model == LG_BINARY_SINTER);
    int64_t cap = 16, nb = 0;
    ipair *pr = (ipair *)malloc(sizeof(ipair) * cap);
    int64_t *subset = (int64_t *)malloc(sizeof(int64_t) * (n > 0 ? n : 1));
    for (int64_t i = 0; i < n; ++i) subset[i] = i;
    for (int64_t i = 0; i + 1 < n; ++i) {
        v3 xi_ = ld(x0, i);
        for (int64_t j = i + 1; j < n; ++j) {
            double g = nrm(sub(xi_, ld(x0, j))) - 2.0 * r;
            if (fabs(g) < dc) {
                if (cyc) {
                    if (subset[i] == subset[j]) continue;
                    int64_t sj = subset[j], si = subset[i];
                    for (int64_t q = 0; q < n; ++q)
                        if (subset[q] == sj) subset[q] = si;
                }
                if (nb == cap) { cap *= 2; pr = (ipair *)realloc(pr, sizeof(ipair) * cap); }
                pr[nb].i = (int32_t)i;
                pr[nb].j = (int32_t)j;
                ++nb;
            }
        }
    }
    free(subset);
    *out = pr;
    return nb;
}

/* sinter_functor ctor bond test, sinter_bridge.h:146-160: every pair i < j (i ascending, then j)
 * with |(|x_j - x_i| - 2 r)| <= critical_separation; no cycle check. */
static int64_t detect_bonds_connectors(const lg_system_desc *d, const double *x0, int64_t n, ipair **out) {
    const double r = d->contact.r_part, dc = d->connector.critical_separation;
    int64_t cap = 16, nb = 0;
    ipair *pr = (ipair *)malloc(sizeof(ipair) * cap);
    for (int64_t i = 0; i + 1 < n; ++i) {
        v3 xi_ = ld(x0, i);
        for (int64_t j = i + 1; j < n; ++j) {
            double g = nrm(sub(ld(x0, j), xi_)) - 2.0 * r;
            if (fabs(g) > dc) continue;
            if (nb == cap) { cap *= 2; pr = (ipair *)realloc(pr, sizeof(ipair) * cap); }
            pr[nb].i = (int32_t)i;
            pr[nb].j = (int32_t)j;
            ++nb;
        }
    }
    *out = pr;
    return nb;
}

static int cmp_bond(const void *a, const void *b) {
    int32_t x = ((const bond *)a)->j, y = ((const bond *)b)->j;
    return (x > y) - (x < y);
}

/* ---------------------------------------------------------------------------------------------
 * Verlet list: j != i with squared centre distance < r_verlet^2, ascending j. Built through a
 * uniform cell grid; rows keep the springs of pairs present before and after.
 * ------------------------------------------------------------------------------------------- */
static void build_rows(lgo_system *s, int carry) {
    const int64_t n = s->n;
    const int all = (s->d.pairs == LG_PAIRS_ALL);
    if (all) {
        for (int64_t i = 0; i < n; ++i) {
            row *r = &s->rows[i];
            if (r->e) continue; /* all-pairs rows never change */
            r->cap = (int32_t)(n > 1 ? n - 1 : 1);
            r->e = (entry *)calloc((size_t)r->cap, sizeof(entry));
            int32_t c = 0;
            for (int64_t j = 0; j < n; ++j)
                if (j != i) r->e[c++].j = (int32_t)j;
            r->n = c;
        }
        return;
    }
    const double rv = s->d.r_verlet, rv2 = rv * rv;
    double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
    for (int64_t i = 0; i < n; ++i)
        for (int c = 0; c < 3; ++c) {
            double q = s->x[3 * i + c];
            if (q < lo[c]) lo[c] = q;
            if (q > hi[c]) hi[c] = q;
        }
    /* cells of edge >= r_verlet, so the 27-cell stencil covers every pair; the edge grows until
     * the grid has at most max(64, 4n) cells */
    double edge = rv;
    int64_t dim[3];
    for (;;) {
        for (int c = 0; c < 3; ++c) {
            int64_t m = (int64_t)floor((hi[c] - lo[c]) / edge) + 1;
            dim[c] = m < 1 ? 1 : m;
        }
        double cells = (double)dim[0] * (double)dim[1] * (double)dim[2];
        if (cells <= (double)(4 * n > 64 ? 4 * n : 64)) break;
        edge *= 1.25;
    }
    int64_t ncell = dim[0] * dim[1] * dim[2];
    int64_t *head = (int64_t *)malloc(sizeof(int64_t) * ncell);
    int64_t *next = (int64_t *)malloc(sizeof(int64_t) * (n > 0 ? n : 1));
    int64_t *cid = (int64_t *)malloc(sizeof(int64_t) * 3 * (n > 0 ? n : 1));
    for (int64_t c = 0; c < ncell; ++c) head[c] = -1;
    for (int64_t i = n - 1; i >= 0; --i) {
        int64_t cc[3];
        for (int c = 0; c < 3; ++c) {
            int64_t k = (int64_t)floor((s->x[3 * i + c] - lo[c]) / edge);
            if (k < 0) k = 0;
            if (k >= dim[c]) k = dim[c] - 1;
            cc[c] = k;
            cid[3 * i + c] = k;
        }
        int64_t lin = (cc[2] * dim[1] + cc[1]) * dim[0] + cc[0];
        next[i] = head[lin];
        head[lin] = i;
    }
#pragma omp parallel for schedule(dynamic, 64) num_threads(s->threads)
    for (int64_t i = 0; i < n; ++i) {
        int32_t cap = 64, cnt = 0;
        int32_t *js = (int32_t *)malloc(sizeof(int32_t) * cap);
        v3 xi_ = ld(s->x, i);
        const int64_t reach[3] = {1, 1, 1};
        for (int64_t cz = cid[3 * i + 2] - reach[2]; cz <= cid[3 * i + 2] + reach[2]; ++cz) {
            if (cz < 0 || cz >= dim[2]) continue;
            for (int64_t cy = cid[3 * i + 1] - reach[1]; cy <= cid[3 * i + 1] + reach[1]; ++cy) {
                if (cy < 0 || cy >= dim[1]) continue;
                for (int64_t cx = cid[3 * i] - reach[0]; cx <= cid[3 * i] + reach[0]; ++cx) {
                    if (cx < 0 || cx >= dim[0]) continue;
                    for (int64_t j = head[(cz * dim[1] + cy) * dim[0] + cx]; j >= 0; j = next[j]) {
                        if (j == i) continue;
                        if (sqn(sub(xi_, ld(s->x, j))) < rv2) {
                            if (cnt == cap) { cap *= 2; js = (int32_t *)realloc(js, sizeof(int32_t) * cap); }
                            js[cnt++] = (int32_t)j;
                        }
                    }
                }
            }
        }
        qsort(js, (size_t)cnt, sizeof(int32_t), cmp_i32);
        row *r = &s->rows[i];
        entry *ne = (entry *)calloc((size_t)(cnt > 0 ? cnt : 1), sizeof(entry));
        for (int32_t k = 0; k < cnt; ++k) {
            ne[k].j = js[k];
            if (carry && r->e) {
                entry *old = find_entry(r->e, r->n, js[k]);
                if (old) memcpy(ne[k].xi, old->xi, sizeof(old->xi));
            }
        }
        free(r->e);
        r->e = ne;
        r->n = cnt;
        r->cap = cnt > 0 ? cnt : 1;
        free(js);
    }
    free(head);
    free(next);
    free(cid);
}

/* ---------------------------------------------------------------------------------------------
 * Force evaluation
 * ------------------------------------------------------------------------------------------- */
static void eval_forces(lgo_system *s) {
    const int64_t n = s->n;
    const lg_system_desc *d = &s->d;
    const int bm = d->binary_model, hm = d->hamaker_model;
    const int breaking = (bm == LG_BINARY_BREAKING_SINTER);
#pragma omp parallel for schedule(dynamic, 16) num_threads(s->threads)
    for (int64_t i = 0; i < n; ++i) {
        v3 acc = ZERO, accw = ZERO;
        v3 xi_ = ld(s->x, i), vi = ld(s->v, i), wi = ld(s->om, i);
        row *r = &s->rows[i];
        for (int32_t k = 0; k < r->n; ++k) {
            entry *e = &r->e[k];
            int64_t j = e->j;
            v3 xj_ = ld(s->x, j), vj = ld(s->v, j), wj = ld(s->om, j);
            v3 pa = ZERO, pal = ZERO;
            int have = 0;
            if (bm != LG_BINARY_NONE) {
                bond *b = (bm == LG_BINARY_SINTER || bm == LG_BINARY_BREAKING_SINTER || bm == LG_BINARY_SINTER_CONNECTORS)
                              ? find_bond(r, (int32_t)j) : NULL;
                if (b && b->intact && bm == LG_BINARY_SINTER_CONNECTORS) {
                    const bond *bj = &s->rows[j].b[b->rev];
                    connector_functor(&d->connector, d->contact.r_part, d->contact.mass, d->contact.inertia, xi_, xj_,
                                      vi, vj, wi, wj, b->cn, bj->cn, &pa, &pal);
                } else if (b && b->intact) {
                    int brk = bond_functor(&d->sinter, xi_, xj_, vi, vj, wi, wj, b->xi, breaking, b->strength, &pa, &pal);
                    if (brk) b->intact = 0;
                } else {
                    contact_functor(&d->contact, xi_, xj_, vi, vj, wi, wj, e->xi, &pa, &pal);
                }
                have = 1;
            }
            if (hm != LG_HAMAKER_NONE) {
                v3 ha = hamaker_functor(hm, &d->hamaker, xi_, xj_);
                if (have) {
                    pa = add(pa, ha);
                    pal = add(pal, ZERO);
                } else {
                    pa = ha;
                    pal = ZERO;
                }
            }
            acc = add(acc, pa);
            accw = add(accw, pal);
        }
        /* unary functors: the facets, then the body force, folded as the container folds them,
         * f0 + (f1 + (... + body)) (unary_force_container.h:27-29) */
        {
            v3 ua = ZERO, ual = ZERO;
            int have = 0;
            if (d->body.model == LG_BODY_CENTRAL) {
                /* central_attraction_functor (Custom-unary-force-model.md:108-118) */
                const double kam = d->body.k_a / d->body.mass;
                ua = scl(kam, sub(mk(s->centre[0], s->centre[1], s->centre[2]), xi_));
                ual = ZERO;
                have = 1;
            }
            for (int32_t f = d->n_facets - 1; f >= 0; --f) {
                const lg_facet_desc *fd = &s->facets[f];
                v3 N = ld(s->facet_normal, f);
                v3 xf = closest_point_on_triangle(fd->vertices, s->facet_area[f], N, xi_);
                v3 vf = mk(fd->v_facet[0], fd->v_facet[1], fd->v_facet[2]);
                v3 fa = ZERO, fal = ZERO;
                int hv = 0;
                if (fd->has_contact) {
                    surface_contact(&fd->contact, xf, vf, xi_, vi, wi, &s->surf_xi[((int64_t)f * n + i) * 3], &fa, &fal);
                    hv = 1;
                }
                if (fd->has_hamaker) {
                    v3 ha = surface_hamaker(&fd->hamaker, xf, xi_);
                    if (hv) { fa = add(fa, ha); fal = add(fal, ZERO); } else { fa = ha; fal = ZERO; }
                }
                if (have) { ua = add(fa, ua); ual = add(fal, ual); } else { ua = fa; ual = fal; have = 1; }
            }
            if (have) {
                acc = add(acc, ua);
                accw = add(accw, ual);
            }
        }
        stv(s->a, i, acc);
        stv(s->al, i, accw);
    }
}

/* ---------------------------------------------------------------------------------------------
 * Public API
 * ------------------------------------------------------------------------------------------- */
static void facet_geometry(lgo_system *s) {
    for (int32_t f = 0; f < s->d.n_facets; ++f) {
        const double *vt = s->facets[f].vertices;
        v3 v0 = mk(vt[0], vt[1], vt[2]), v1 = mk(vt[3], vt[4], vt[5]), v2 = mk(vt[6], vt[7], vt[8]);
        v3 u = sub(v1, v0), w = sub(v2, v0);
        s->facet_area[f] = 1.0 / 2.0 * nrm(crs(u, w)); /* triangular_facet.h:23-27 */
        stv(s->facet_normal, f, nrmz(crs(u, w)));
    }
}

lgo_system *lgo_create(const lg_system_desc *d, const double *x0, const double *v0, const double *th0,
                       const double *om0, const lg_facet_desc *facets, const double *neck, int64_t n_neck,
                       int threads) {
    if (!d || d->n_part < 0) return NULL;
    lgo_system *s = (lgo_system *)calloc(1, sizeof(lgo_system));
    s->d = *d;
    s->n = d->n_part;
    s->threads = threads > 0 ? threads : 1;
    s->d.hold_mask = NULL;
    if (d->hold_mask) {
        s->hold = (uint8_t *)malloc((size_t)(s->n > 0 ? s->n : 1));
        memcpy(s->hold, d->hold_mask, (size_t)s->n);
    }
    if (d->body.model == LG_BODY_CENTRAL)
        for (int c = 0; c < 3; ++c) s->centre[c] = d->body.centre[c];
    size_t bytes = sizeof(double) * 3 * (size_t)(s->n > 0 ? s->n : 1);
    s->x = (double *)malloc(bytes); s->v = (double *)malloc(bytes);
    s->th = (double *)malloc(bytes); s->om = (double *)malloc(bytes);
    s->a = (double *)calloc(1, bytes); s->al = (double *)calloc(1, bytes);
    memcpy(s->x, x0, bytes); memcpy(s->v, v0, bytes); memcpy(s->th, th0, bytes); memcpy(s->om, om0, bytes);
    s->rows = (row *)calloc((size_t)(s->n > 0 ? s->n : 1), sizeof(row));
    if (d->n_facets > 0) {
        s->facets = (lg_facet_desc *)malloc(sizeof(lg_facet_desc) * d->n_facets);
        memcpy(s->facets, facets, sizeof(lg_facet_desc) * d->n_facets);
        s->facet_area = (double *)malloc(sizeof(double) * d->n_facets);
        s->facet_normal = (double *)malloc(sizeof(double) * 3 * d->n_facets);
        s->surf_xi = (v3 *)calloc((size_t)d->n_facets * (size_t)(s->n > 0 ? s->n : 1) * 3, sizeof(v3));
        facet_geometry(s);
    }
    /* bonds */
    if (d->binary_model == LG_BINARY_SINTER || d->binary_model == LG_BINARY_BREAKING_SINTER) {
        ipair *pr = NULL;
        int64_t nb = detect_bonds(d, x0, s->n, &pr);
        s->n_bonds_initial = 2 * nb;
        /* particle-indexed strengths of the reference (alt_breaking_sinter_bridge.h:70-73) */
        double *pstr = (double *)calloc((size_t)(s->n > 0 ? s->n : 1), sizeof(double));
        for (int64_t b = 0; b < nb; ++b) {
            double sv = (neck && n_neck == nb) ? neck[b] : INFINITY;
            pstr[pr[b].i] = sv;
            pstr[pr[b].j] = sv;
        }
        int32_t *cnt = (int32_t *)calloc((size_t)(s->n > 0 ? s->n : 1), sizeof(int32_t));
        for (int64_t b = 0; b < nb; ++b) { cnt[pr[b].i]++; cnt[pr[b].j]++; }
        for (int64_t i = 0; i < s->n; ++i) {
            s->rows[i].b = (bond *)calloc((size_t)(cnt[i] > 0 ? cnt[i] : 1), sizeof(bond));
            s->rows[i].nb = 0;
        }
        for (int64_t b = 0; b < nb; ++b) {
            double sv = (neck && n_neck == nb) ? neck[b] : INFINITY;
            int32_t i = pr[b].i, j = pr[b].j;
            bond *bi = &s->rows[i].b[s->rows[i].nb++];
            bond *bj = &s->rows[j].b[s->rows[j].nb++];
            bi->j = j; bi->intact = 1;
            bj->j = i; bj->intact = 1;
            if (d->neck_mode == LG_NECK_REFERENCE_INDEXING) {
                /* neck_strengths[i*n + j] is nonzero only where i*n + j < n, i.e. i == 0 */
                bi->strength = (i == 0) ? pstr[j] : 0.0;
                bj->strength = (j == 0) ? pstr[i] : 0.0;
            } else {
                bi->strength = sv;
                bj->strength = sv;
            }
        }
        for (int64_t i = 0; i < s->n; ++i)
            if (s->rows[i].nb > 1) qsort(s->rows[i].b, (size_t)s->rows[i].nb, sizeof(bond), cmp_bond);
        free(cnt);
        free(pstr);
        free(pr);
    }
    if (d->binary_model == LG_BINARY_SINTER_CONNECTORS) {
        ipair *pr = NULL;
        int64_t nb = detect_bonds_connectors(d, x0, s->n, &pr);
        if (!d->connector_axes || d->n_connector_axes != nb) {
            free(pr);
            lgo_destroy(s);
            return NULL;
        }
        s->n_bonds_initial = 2 * nb;
        int32_t *cnt = (int32_t *)calloc((size_t)(s->n > 0 ? s->n : 1), sizeof(int32_t));
        for (int64_t b = 0; b < nb; ++b) { cnt[pr[b].i]++; cnt[pr[b].j]++; }
        for (int64_t i = 0; i < s->n; ++i) {
            s->rows[i].b = (bond *)calloc((size_t)(cnt[i] > 0 ? cnt[i] : 1), sizeof(bond));
            s->rows[i].nb = 0;
        }
        const double r = d->contact.r_part;
        for (int64_t b = 0; b < nb; ++b) {  /* connectors, sinter_bridge.h:163-197 */
            const int32_t i = pr[b].i, j = pr[b].j;
            v3 pi = ld(x0, i), pj = ld(x0, j);
            v3 ni = nrmz(sub(pj, pi)), nj = neg(ni);
            v3 v = ld(d->connector_axes, b);
            v3 db = crs(v, nj);
            if (nrm(db) == 0.0) {  /* the reference draws again; the caller's axis must not be parallel */
                free(pr);
                free(cnt);
                lgo_destroy(s);
                return NULL;
            }
            v3 ds = sub(v, scl(dot(v, ni), ni));
            db = nrmz(db);
            ds = nrmz(ds);
            bond *bi = &s->rows[i].b[s->rows[i].nb++];
            bond *bj = &s->rows[j].b[s->rows[j].nb++];
            bi->j = j; bi->intact = 1; bi->strength = INFINITY;
            bj->j = i; bj->intact = 1; bj->strength = INFINITY;
            bi->cn[0] = add(pi, scl(r, ds)); bi->cn[1] = sub(pi, scl(r, ds));
            bi->cn[2] = add(pi, scl(r, db)); bi->cn[3] = sub(pi, scl(r, db));
            bi->cn[4] = add(pi, scl(r, ni));
            bj->cn[0] = add(pj, scl(r, ds)); bj->cn[1] = sub(pj, scl(r, ds));
            bj->cn[2] = add(pj, scl(r, db)); bj->cn[3] = sub(pj, scl(r, db));
            bj->cn[4] = add(pj, scl(r, nj));
        }
        for (int64_t i = 0; i < s->n; ++i)
            if (s->rows[i].nb > 1) qsort(s->rows[i].b, (size_t)s->rows[i].nb, sizeof(bond), cmp_bond);
        for (int64_t i = 0; i < s->n; ++i)
            for (int32_t q = 0; q < s->rows[i].nb; ++q) {
                bond *bq = &s->rows[i].b[q];
                bq->rev = (int32_t)(find_bond(&s->rows[bq->j], (int32_t)i) - s->rows[bq->j].b);
            }
        free(cnt);
        free(pr);
    }
    build_rows(s, 0);
    eval_forces(s);
    return s;
}

void lgo_destroy(lgo_system *s) {
    if (!s) return;
    for (int64_t i = 0; i < s->n; ++i) { free(s->rows[i].e); free(s->rows[i].b); }
    free(s->rows);
    free(s->x); free(s->v); free(s->th); free(s->om); free(s->a); free(s->al);
    free(s->facets); free(s->facet_area); free(s->facet_normal); free(s->surf_xi); free(s->hold);
    free(s);
}

int lgo_update_neighbor_list(lgo_system *s) {
    if (s->d.pairs != LG_PAIRS_VERLET) return 0;
    build_rows(s, 1);
    return 0;
}

static void facet_move(lgo_system *s, int32_t f, double dt) {
    lg_facet_desc *fd = &s->facets[f];
    for (int k = 0; k < 3; ++k)
        for (int c = 0; c < 3; ++c) fd->vertices[3 * k + c] += fd->v_facet[c] * dt; /* v_facet * dt */
}

int lgo_step(lgo_system *s, double dt, int64_t nsteps, int64_t rebuild_every) {
    const int64_t n = s->n;
    const double hdt = dt / 2.0;
    for (int64_t st = 0; st < nsteps; ++st) {
        if (s->d.pairs == LG_PAIRS_VERLET && rebuild_every > 0 && (s->step_index % rebuild_every) == 0)
            build_rows(s, 1);
        /* half kick; a step handler's held increments are skipped (Custom-step-handler.md:82-97) */
        for (int64_t i = 0; i < n; ++i) {
            const unsigned h = s->hold ? s->hold[i] : 0u;
            for (int c = 0; c < 3; ++c) {
                if (!(h & LG_HOLD_V)) s->v[3 * i + c] += s->a[3 * i + c] * hdt;
                if (!(h & LG_HOLD_OMEGA)) s->om[3 * i + c] += s->al[3 * i + c] * hdt;
            }
        }
        if (s->d.binary_model == LG_BINARY_SINTER_CONNECTORS) {
            /* sinter_step_handler: increment_x moves the particle and its connectors by dx,
             * increment_theta turns the connectors by dtheta about the (moved) centre
             * (sinter_bridge.h:24-42, 55-75); a held increment skips the whole call */
            for (int64_t i = 0; i < n; ++i) {
                const unsigned h = s->hold ? s->hold[i] : 0u;
                row *r = &s->rows[i];
                v3 xn = ld(s->x, i);
                if (!(h & LG_HOLD_X)) {
                    v3 dx = mk(s->v[3 * i] * dt, s->v[3 * i + 1] * dt, s->v[3 * i + 2] * dt);
                    xn = add(xn, dx);
                    stv(s->x, i, xn);
                    for (int32_t q = 0; q < r->nb; ++q)
                        for (int k = 0; k < 5; ++k) r->b[q].cn[k] = add(r->b[q].cn[k], dx);
                }
                if (!(h & LG_HOLD_THETA)) {
                    v3 dth = mk(s->om[3 * i] * dt, s->om[3 * i + 1] * dt, s->om[3 * i + 2] * dt);
                    stv(s->th, i, add(ld(s->th, i), dth));
                    for (int32_t q = 0; q < r->nb; ++q)
                        for (int k = 0; k < 5; ++k) r->b[q].cn[k] = add(r->b[q].cn[k], crs(dth, sub(r->b[q].cn[k], xn)));
                }
            }
        } else {
            for (int64_t i = 0; i < n; ++i) {
                const unsigned h = s->hold ? s->hold[i] : 0u;
                for (int c = 0; c < 3; ++c) {
                    if (!(h & LG_HOLD_X)) s->x[3 * i + c] += s->v[3 * i + c] * dt;
                    if (!(h & LG_HOLD_THETA)) s->th[3 * i + c] += s->om[3 * i + c] * dt;
                }
            }
        }
        eval_forces(s);
        for (int64_t i = 0; i < n; ++i) {
            const unsigned h = s->hold ? s->hold[i] : 0u;
            for (int c = 0; c < 3; ++c) {
                if (!(h & LG_HOLD_V)) s->v[3 * i + c] += s->a[3 * i + c] * hdt;
                if (!(h & LG_HOLD_OMEGA)) s->om[3 * i + c] += s->al[3 * i + c] * hdt;
            }
        }
        if (s->d.facet_auto_move)
            for (int32_t f = 0; f < s->d.n_facets; ++f) facet_move(s, f, dt);
        s->step_index++;
    }
    return 0;
}

/* Connector points of every bond end: particle i ascending, partner j ascending, 5 points each
 * (spring_connectors[i * n + j] of sinter_bridge.h:139). Returns the number of points. */
int64_t lgo_get_connectors(lgo_system *s, double *out, int64_t cap) {
    int64_t k = 0;
    if (s->d.binary_model != LG_BINARY_SINTER_CONNECTORS) return 0;
    for (int64_t i = 0; i < s->n; ++i) {
        row *r = &s->rows[i];
        int32_t order[256];
        int32_t m = r->nb < 256 ? r->nb : 256;
        for (int32_t q = 0; q < m; ++q) order[q] = q;
        for (int32_t a = 1; a < m; ++a) /* insertion sort by partner */
            for (int32_t b = a; b > 0 && r->b[order[b]].j < r->b[order[b - 1]].j; --b) {
                int32_t t = order[b]; order[b] = order[b - 1]; order[b - 1] = t;
            }
        for (int32_t q = 0; q < m; ++q)
            for (int c = 0; c < 5; ++c, ++k)
                if (out && k < cap) {
                    out[3 * k] = r->b[order[q]].cn[c].x;
                    out[3 * k + 1] = r->b[order[q]].cn[c].y;
                    out[3 * k + 2] = r->b[order[q]].cn[c].z;
                }
    }
    return k;
}

int lgo_set_hold_mask(lgo_system *s, const uint8_t *mask) {
    free(s->hold);
    s->hold = NULL;
    if (mask) {
        s->hold = (uint8_t *)malloc((size_t)(s->n > 0 ? s->n : 1));
        memcpy(s->hold, mask, (size_t)s->n);
    }
    return 0;
}

int lgo_set_body_force(lgo_system *s, const lg_body_force *f) {
    lg_body_force none;
    memset(&none, 0, sizeof(none));
    s->d.body = f ? *f : none;
    if (f && f->model == LG_BODY_CENTRAL)
        for (int c = 0; c < 3; ++c) s->centre[c] = f->centre[c];
    return 0;
}

int lgo_set_body_centre(lgo_system *s, const double *c) {
    for (int k = 0; k < 3; ++k) s->centre[k] = c[k];
    return 0;
}

int lgo_facet_update_positions(lgo_system *s, int32_t f, double dt) {
    if (f < 0 || f >= s->d.n_facets) return -1;
    facet_move(s, f, dt);
    return 0;
}

int lgo_facet_get_vertices(lgo_system *s, int32_t f, double *out9) {
    if (f < 0 || f >= s->d.n_facets) return -1;
    memcpy(out9, s->facets[f].vertices, sizeof(double) * 9);
    return 0;
}

int lgo_get(lgo_system *s, int field, double *out) {
    double *src = NULL;
    switch (field) {
        case LG_FIELD_X: src = s->x; break;
        case LG_FIELD_V: src = s->v; break;
        case LG_FIELD_THETA: src = s->th; break;
        case LG_FIELD_OMEGA: src = s->om; break;
        case LG_FIELD_A: src = s->a; break;
        case LG_FIELD_ALPHA: src = s->al; break;
        default: return -1;
    }
    memcpy(out, src, sizeof(double) * 3 * (size_t)s->n);
    return 0;
}

int lgo_set(lgo_system *s, int field, const double *in) {
    double *dst = NULL;
    switch (field) {
        case LG_FIELD_X: dst = s->x; break;
        case LG_FIELD_V: dst = s->v; break;
        case LG_FIELD_THETA: dst = s->th; break;
        case LG_FIELD_OMEGA: dst = s->om; break;
        case LG_FIELD_A: dst = s->a; break;
        case LG_FIELD_ALPHA: dst = s->al; break;
        default: return -1;
    }
    memcpy(dst, in, sizeof(double) * 3 * (size_t)s->n);
    return 0;
}

int lgo_get_pair_springs(lgo_system *s, int64_t i, int64_t j, double *out9) {
    memset(out9, 0, sizeof(double) * 9);
    if (i < 0 || j < 0 || i >= s->n || j >= s->n) return -1;
    row *r = &s->rows[i];
    bond *b = r->b ? find_bond(r, (int32_t)j) : NULL;
    v3 *src = NULL;
    if (b && b->intact) src = b->xi;
    else {
        entry *e = find_entry(r->e, r->n, (int32_t)j);
        if (e) src = e->xi;
    }
    if (src)
        for (int k = 0; k < 3; ++k) { out9[3 * k] = src[k].x; out9[3 * k + 1] = src[k].y; out9[3 * k + 2] = src[k].z; }
    return 0;
}

int64_t lgo_count_bonds(lgo_system *s, int64_t *pairs, int64_t cap) {
    int64_t c = 0;
    for (int64_t i = 0; i < s->n; ++i)
        for (int32_t k = 0; k < s->rows[i].nb; ++k)
            if (s->rows[i].b[k].intact) {
                if (pairs && c < cap) { pairs[2 * c] = i; pairs[2 * c + 1] = s->rows[i].b[k].j; }
                ++c;
            }
    return c;
}

int64_t lgo_row_length(lgo_system *s, int64_t i) {
    if (i < 0 || i >= s->n) return -1;
    return s->rows[i].n;
}

int64_t lgo_row(lgo_system *s, int64_t i, int32_t *out, int64_t cap) {
    if (i < 0 || i >= s->n) return -1;
    int64_t m = s->rows[i].n < cap ? s->rows[i].n : cap;
    for (int64_t k = 0; k < m; ++k) out[k] = s->rows[i].e[k].j;
    return s->rows[i].n;
}

/* Hamaker interaction energy between two equal spheres at surface separation h (the potential of
 * the force in hamaker_force.h:36-40; libgran's README states it), evaluated at max(h, h0). */
/* Pair potential of the Hamaker functors, the exact integral of the force they apply (the
 * reference has no energy bookkeeping; this definition is the project's). The full form is
 *   U(h) = -A/6 [2r^2/((4r+h)h) + 2r^2/(2r+h)^2 + ln((4r+h)h/(2r+h)^2)],
 * whose derivative is the bracket of hamaker_force.h:36-40; the simplified form (force 2Ar/h^2,
 * simplified_hamaker_force.h:18-31) has U(h) = -2Ar/h. Below the saturation distance h0 the force
 * stays at its value at h0, so U continues linearly with that slope; the limited form cuts the
 * force at the centre distance r_cutoff, so its U is shifted to vanish there. */
static double hamaker_u0(int mode, double A, double r, double h) {
    if (mode == LG_HAMAKER_SIMPLIFIED) return -2.0 * A * r / h;
    return -A / 6.0 * (2.0 * r * r / ((4.0 * r + h) * h) + 2.0 * r * r / ((2.0 * r + h) * (2.0 * r + h))
                       + log((4.0 * r + h) * h / ((2.0 * r + h) * (2.0 * r + h))));
}
static double hamaker_slope(int mode, double A, double r, double h) {
    if (mode == LG_HAMAKER_SIMPLIFIED) return 2.0 * A * r / (h * h);
    double br = (4.0 * r + 2.0 * h) / (4.0 * r + h) / h - 2.0 / (2.0 * r + h) - 4.0 * r * r / ((2.0 * r + h) * (2.0 * r + h) * (2.0 * r + h))
                - 2.0 * r * r * (4.0 * r + 2.0 * h) / ((4.0 * r + h) * (4.0 * r + h)) / (h * h);
    return -A / 6.0 * br;
}
static double hamaker_energy(int mode, const lg_hamaker_params *p, double dist) {
    const double r = p->r_part, h = dist - 2.0 * r;
    double u = h < p->h0 ? hamaker_u0(mode, p->A, r, p->h0) + hamaker_slope(mode, p->A, r, p->h0) * (h - p->h0)
                         : hamaker_u0(mode, p->A, r, h);
    if (mode == LG_HAMAKER_LIMITED) {
        const double hc = p->r_cutoff - 2.0 * r;
        u -= hc < p->h0 ? hamaker_u0(mode, p->A, r, p->h0) + hamaker_slope(mode, p->A, r, p->h0) * (hc - p->h0)
                        : hamaker_u0(mode, p->A, r, hc);
    }
    return u;
}

/* test/compute_energy.cpp:7-58, test/mass_distribution.cpp:7-27, plus potential energy. */
int lgo_observables(lgo_system *s, lg_observables *o) {
    memset(o, 0, sizeof(*o));
    const int64_t n = s->n;
    const lg_system_desc *d = &s->d;
    double m, I;
    if (d->binary_model == LG_BINARY_SINTER || d->binary_model == LG_BINARY_BREAKING_SINTER) {
        m = d->sinter.mass; I = d->sinter.inertia;
    } else if (d->binary_model == LG_BINARY_CONTACT || d->binary_model == LG_BINARY_SINTER_CONNECTORS) {
        m = d->contact.mass; I = d->contact.inertia;
    } else {
        m = d->hamaker.mass; I = d->contact.inertia;
    }
    double e_tot = 0.0, e_tr = 0.0, e_rot = 0.0;
    v3 P = ZERO, L = ZERO, Lx = ZERO, c = ZERO;
    for (int64_t i = 0; i < n; ++i) {
        v3 v = ld(s->v, i), w = ld(s->om, i), x = ld(s->x, i);
        e_tot += m * dot(v, v) / 2.0;
        e_tot += I * dot(w, w) / 2.0;
        e_tr += m * dot(v, v);
        e_rot += I * dot(w, w);
        P = add(P, v);
        L = add(L, scl(I, w));
        c = add(c, x);
    }
    for (int64_t i = 0; i < n; ++i) Lx = add(Lx, crs(ld(s->x, i), scl(m, ld(s->v, i))));
    L = add(L, Lx);
    o->ke_total = e_tot;
    o->ke_translational = e_tr / 2.0;
    o->ke_rotational = e_rot / 2.0;
    o->linear_momentum = m * nrm(P);
    o->angular_momentum = nrm(L);
    c = dvs(c, (double)n);
    o->center_of_mass[0] = c.x; o->center_of_mass[1] = c.y; o->center_of_mass[2] = c.z;
    double rg = 0.0;
    for (int64_t i = 0; i < n; ++i) { v3 q = sub(ld(s->x, i), c); rg += dot(q, q); }
    o->radius_of_gyration = sqrt(rg / (double)n);
    /* potential energy, halved over ordered pairs */
    double pe = 0.0;
    int64_t ncont = 0, nbond = 0;
    for (int64_t i = 0; i < n; ++i) {
        row *r = &s->rows[i];
        v3 xi_ = ld(s->x, i);
        for (int32_t k = 0; k < r->n; ++k) {
            entry *e = &r->e[k];
            v3 xj_ = ld(s->x, e->j);
            double dist = nrm(sub(xi_, xj_));
            bond *b = r->b ? find_bond(r, e->j) : NULL;
            double u = 0.0;
            if (b && b->intact && d->binary_model == LG_BINARY_SINTER_CONNECTORS) {
                const bond *bj = &s->rows[e->j].b[b->rev];
                for (int k = 0; k < 5; ++k) {
                    double dl = (k < 4 ? 2.0 * d->contact.r_part : 0.0) - nrm(sub(bj->cn[k], b->cn[k]));
                    u += 0.5 * d->connector.k_d * dl * dl;
                }
                nbond++;
            } else if (b && b->intact) {
                double dl = 2.0 * d->sinter.r_part - dist;
                u += 0.5 * d->sinter.k * dl * dl;
                u += 0.5 * d->sinter.k_t * sqn(b->xi[0]) + 0.5 * d->sinter.k_r * sqn(b->xi[1]) + 0.5 * d->sinter.k_o * sqn(b->xi[2]);
                nbond++;
            } else if (d->binary_model != LG_BINARY_NONE) {
                double dl = 2.0 * d->contact.r_part - dist;
                if (dl > 0) {
                    u += 0.5 * d->contact.k * dl * dl;
                    ncont++;
                }
                u += 0.5 * d->contact.k_t * sqn(e->xi[0]) + 0.5 * d->contact.k_r * sqn(e->xi[1]) + 0.5 * d->contact.k_o * sqn(e->xi[2]);
            }
            if (d->hamaker_model == LG_HAMAKER_FULL || d->hamaker_model == LG_HAMAKER_SIMPLIFIED ||
                (d->hamaker_model == LG_HAMAKER_LIMITED && !(dist > d->hamaker.r_cutoff)))
                u += hamaker_energy(d->hamaker_model, &d->hamaker, dist);
            pe += 0.5 * u;
        }
    }
    o->potential_energy = pe;
    o->n_contacts = ncont;
    o->n_bonds = nbond;
    o->n_bonds_initial = s->n_bonds_initial;
    return 0;
}

int64_t lgo_step_index(lgo_system *s) { return s->step_index; }

/* Helper used by tests: evaluate the reference known-answer set-ups as independent systems in
 * parallel threads (each system single threaded). */
int lgo_run_many(lgo_system **systems, const double *dts, const int64_t *nsteps, const int64_t *rebuild,
                 int count) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int k = 0; k < count; ++k) lgo_step(systems[k], dts[k], nsteps[k], rebuild[k]);
    return 0;
}

/* ---------------------------------------------------------------------------------------------
 * Seeded workload generator (project-defined; libgran has none). Same algorithm and arithmetic as
 * the engine's lg_generate_rsa_aggregate / lg_generate_velocities, restated here so that the timed
 * CPU baseline builds its inputs without the engine library: SplitMix64 draws, a parent chosen
 * uniformly among the spheres placed so far, a direction uniform on the unit sphere (rejection
 * from the cube), the candidate at distance 2r from the parent, rejected when any other sphere is
 * closer than 2r - 1e-12 r. Whether a candidate is accepted does not depend on the order in which
 * the neighbouring spheres are visited, so the spatial hash below gives the engine's bits.
 */
typedef struct {
    uint64_t s;
} lgo_splitmix;

static uint64_t sm_next(lgo_splitmix *g) {
    uint64_t z = (g->s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double sm_uniform(lgo_splitmix *g) { return (double)(sm_next(g) >> 11) * 0x1.0p-53; }
static v3 sm_unit(lgo_splitmix *g) {
    for (;;) {
        double a = 2.0 * sm_uniform(g) - 1.0, b = 2.0 * sm_uniform(g) - 1.0, c = 2.0 * sm_uniform(g) - 1.0;
        double s2 = (a * a + b * b) + c * c;
        if (s2 > 1e-6 && s2 <= 1.0) {
            double s = sqrt(s2);
            return mk(a / s, b / s, c / s);
        }
    }
}

/* open-addressing table: cell key -> head of a singly linked list of sphere indices */
typedef struct {
    int64_t *key;
    int32_t *head;
    uint64_t mask;
} lgo_cellmap;

static uint64_t cell_hash(int64_t k) {
    uint64_t z = (uint64_t)k * 0x9E3779B97F4A7C15ull;
    return z ^ (z >> 29);
}
static int32_t *cell_slot(lgo_cellmap *m, int64_t k, int insert) {
    uint64_t h = cell_hash(k) & m->mask;
    for (;;) {
        if (m->head[h] == -2) {
            if (!insert) return NULL;
            m->key[h] = k;
            m->head[h] = -1;
            return &m->head[h];
        }
        if (m->key[h] == k) return &m->head[h];
        h = (h + 1) & m->mask;
    }
}

int lgo_generate_rsa_aggregate(uint64_t seed, int64_t n, double r, double *x) {
    if (n < 1 || !x || !(r > 0)) return -1;
    lgo_splitmix rng = {seed};
    const double edge = 2.0 * r;
    const double lim = 2.0 * r - 1e-12 * r;
    const double lim2 = lim * lim;
    uint64_t cap = 16;
    while (cap < 4 * (uint64_t)n) cap <<= 1;
    lgo_cellmap m = {(int64_t *)malloc(sizeof(int64_t) * cap), (int32_t *)malloc(sizeof(int32_t) * cap), cap - 1};
    int32_t *next = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    if (!m.key || !m.head || !next) {
        free(m.key);
        free(m.head);
        free(next);
        return -1;
    }
    for (uint64_t q = 0; q < cap; ++q) m.head[q] = -2;
#define LGO_KEY(a, b, c) ((((a) + 1048576) * 2097152 + ((b) + 1048576)) * 2097152 + ((c) + 1048576))
    x[0] = x[1] = x[2] = 0.0;
    {
        int32_t *h = cell_slot(&m, LGO_KEY((int64_t)floor(0.0 / edge), (int64_t)floor(0.0 / edge),
                                          (int64_t)floor(0.0 / edge)), 1);
        next[0] = *h;
        *h = 0;
    }
    int rc = 0;
    for (int64_t k = 1; k < n && rc == 0; ++k) {
        for (int attempt = 0;; ++attempt) {
            if (attempt > 100000) {
                rc = -1;
                break;
            }
            int64_t p = (int64_t)(sm_uniform(&rng) * (double)k);
            if (p >= k) p = k - 1;
            v3 dir = sm_unit(&rng);
            v3 c = add(ld(x, p), scl(2.0 * r, dir));
            int64_t cc[3] = {(int64_t)floor(c.x / edge), (int64_t)floor(c.y / edge), (int64_t)floor(c.z / edge)};
            int ok = 1;
            for (int64_t dz = -1; dz <= 1 && ok; ++dz)
                for (int64_t dy = -1; dy <= 1 && ok; ++dy)
                    for (int64_t dx = -1; dx <= 1 && ok; ++dx) {
                        int32_t *h = cell_slot(&m, LGO_KEY(cc[0] + dx, cc[1] + dy, cc[2] + dz), 0);
                        for (int32_t q = h ? *h : -1; q >= 0; q = next[q]) {
                            if (q == p) continue;
                            if (sqn(sub(c, ld(x, q))) < lim2) {
                                ok = 0;
                                break;
                            }
                        }
                    }
            if (!ok) continue;
            stv(x, k, c);
            int32_t *h = cell_slot(&m, LGO_KEY(cc[0], cc[1], cc[2]), 1);
            next[k] = *h;
            *h = (int32_t)k;
            break;
        }
    }
#undef LGO_KEY
    free(m.key);
    free(m.head);
    free(next);
    return rc;
}

int lgo_generate_velocities(uint64_t seed, int64_t n, double vmax, double *v) {
    if (n < 0 || !v) return -1;
    lgo_splitmix rng = {seed ^ 0x5DEECE66Dull};
    for (int64_t q = 0; q < 3 * n; ++q) v[q] = (2.0 * sm_uniform(&rng) - 1.0) * vmax;
    return 0;
}
