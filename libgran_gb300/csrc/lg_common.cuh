// lg_common.cuh -- device-side data layout and FP64 pair functors of the GB300 engine.
//
// The functors restate libgran's force models (paths inside the libgran project):
//   contact      contact_force/contact_force.h:57-147
//   bond         sinter_bridge/alt_sinter_bridge.h:103-156, alt_breaking_sinter_bridge.h:89-131
//   Hamaker      hamaker_force/hamaker_force.h:28-43, limited_range_hamaker_force.h:29-47,
//                simplified_hamaker_force.h:18-31
//   surface      contact_force/surface_contact_force.h:57-145, surface_hamaker_force.h:18-30,
//                surface_force/triangular_facet.h:32-137
// Every FP64 expression keeps the evaluation order of the reference (Eigen component-wise
// semantics: norm = sqrt((x*x + y*y) + z*z), normalized = v / norm). Translation units that include
// this header for the FP64 path are compiled with --fmad=false, so a thread that walks a row in
// ascending j produces the same bits as a sequential CPU evaluation built with -ffp-contract=off.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/libgran_gb300.h"

namespace lg {

// ------------------------------------------------------------------------------------------------
// Small FP64 vector with the reference's evaluation order
// ------------------------------------------------------------------------------------------------
struct d3 {
    double x, y, z;
};
__host__ __device__ __forceinline__ d3 mk3(double x, double y, double z) { return d3{x, y, z}; }
__host__ __device__ __forceinline__ d3 add(d3 a, d3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ d3 sub(d3 a, d3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ d3 scl(double s, d3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
__host__ __device__ __forceinline__ d3 dvs(d3 a, double s) { return mk3(a.x / s, a.y / s, a.z / s); }
__host__ __device__ __forceinline__ d3 neg(d3 a) { return mk3(-a.x, -a.y, -a.z); }
__host__ __device__ __forceinline__ double dot(d3 a, d3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__host__ __device__ __forceinline__ double sqn(d3 a) { return (a.x * a.x + a.y * a.y) + a.z * a.z; }
__host__ __device__ __forceinline__ double nrm(d3 a) { return sqrt(sqn(a)); }
__host__ __device__ __forceinline__ d3 nrmz(d3 a) {
    double z = sqn(a);
    if (z > 0.0) return dvs(a, sqrt(z));
    return a;
}
__host__ __device__ __forceinline__ d3 crs(d3 a, d3 b) {
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__host__ __device__ __forceinline__ d3 zero3() { return mk3(0.0, 0.0, 0.0); }

// State vectors live in 32-byte aligned slots (w unused) so that one particle field is one aligned
// 32-byte sector, fetched by a single 256-bit load on sm_103a.
typedef double4_32a dbl4;
#ifdef __CUDACC__
// A spring component stored as a float-float pair (hi, lo) in an 8-byte slot.
__device__ __forceinline__ double ffslot_load(const double *p, int64_t idx) {
    const float2 v = reinterpret_cast<const float2 *>(p)[idx];
    return (double)v.x + (double)v.y;
}
__device__ __forceinline__ void ffslot_store(double *p, int64_t idx, double d) {
    const float hi = (float)d;
    reinterpret_cast<float2 *>(p)[idx] = make_float2(hi, (float)(d - (double)hi));
}
// Position of particle i relative to its system's origin as a float-float pair, interleaved (one
// 32-byte sector per particle): x32[2i] receives the FP32 rounding of the FP64 difference,
// x32[2i + 1] the FP32 rounding of what that leaves.
__device__ __forceinline__ void rel_ff(d3 q, double ox, double oy, double oz, const int32_t *agg, const dbl4 *orig,
                                       int64_t i, int64_t n, float4 *__restrict__ x32) {
    if (agg) {
        const dbl4 o = orig[agg[i]];
        ox = o.x;
        oy = o.y;
        oz = o.z;
    }
    const double rx = q.x - ox, ry = q.y - oy, rz = q.z - oz;
    const float hx = (float)rx, hy = (float)ry, hz = (float)rz;
    (void)n;
    x32[2 * i] = make_float4(hx, hy, hz, 0.0f);
    x32[2 * i + 1] = make_float4((float)(rx - (double)hx), (float)(ry - (double)hy), (float)(rz - (double)hz), 0.0f);
}

// Velocity copies of the mixed compacted kernel: v32[i] / v32[n + i] = high / low FP32 parts of v_i,
// v32[2n + i] = FP32 rounding of omega_i.
__device__ __forceinline__ void vel_ff(d3 v, d3 w, int64_t i, int64_t n, float4 *__restrict__ v32) {
    const float hx = (float)v.x, hy = (float)v.y, hz = (float)v.z;
    v32[i] = make_float4(hx, hy, hz, 0.0f);
    v32[n + i] = make_float4((float)(v.x - (double)hx), (float)(v.y - (double)hy), (float)(v.z - (double)hz), 0.0f);
    v32[2 * n + i] = make_float4((float)w.x, (float)w.y, (float)w.z, 0.0f);
}

// The float-float state of particle i after an FP64 update: vel_ff's copies plus, in s32, the low
// FP32 parts of omega_i, and zero for the displacement and rotation accumulated since (s32[n..5n)).
__device__ __forceinline__ void state_ff(d3 v, d3 w, int64_t i, int64_t n, float4 *__restrict__ v32,
                                         float4 *__restrict__ s32) {
    vel_ff(v, w, i, n, v32);
    if (!s32) return;
    s32[i] = make_float4((float)(w.x - (double)(float)w.x), (float)(w.y - (double)(float)w.y),
                         (float)(w.z - (double)(float)w.z), 0.0f);
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int q = 1; q < 5; ++q) s32[q * n + i] = z;
}

// A spring component in either storage form.
__device__ __forceinline__ double spring_load(const double *p, int64_t idx, bool ff) {
    return ff ? ffslot_load(p, idx) : p[idx];
}
__device__ __forceinline__ d3 ld4(const dbl4 *p, int64_t i) {
    dbl4 q = p[i];
    return mk3(q.x, q.y, q.z);
}
__device__ __forceinline__ void st4(dbl4 *p, int64_t i, d3 a) { p[i] = make_double4_32a(a.x, a.y, a.z, 0.0); }
#endif

// ------------------------------------------------------------------------------------------------
// Parameters (one POD block passed by value to every kernel)
// ------------------------------------------------------------------------------------------------
constexpr int kMaxFacets = 4;

struct FacetDev {
    double v[3];
    double area;
    double normal[3];
    int32_t has_contact, has_hamaker;
    lg_contact_params contact;
    lg_hamaker_params hamaker;
};

struct Params {
    int64_t n;
    int32_t binary_model, hamaker_model, neck_mode, pairs;
    lg_contact_params contact;
    lg_sinter_params sinter;
    lg_hamaker_params hamaker;
    double r_verlet;
    int32_t n_facets;
    FacetDev facets[kMaxFacets];
    double contact_skip_d2;  // squared centre distance above which overlap <= 0 is certain
    double hamaker_skip_d2;  // squared centre distance above which the limited Hamaker is zero
    int32_t springs_ff;      // pair and bond springs held as float-float pairs (mixed precision)
    lg_connector_params connector;  // 5-connector sinter model
    const uint8_t *hold;     // [n] LG_HOLD_* bits of the increments the integrator skips; null: none
    const dbl4 *ext_a;       // [n] unary body-force terms (a, alpha) folded after the facets; null: none
    const dbl4 *ext_al;
};

// Internal hold bit of a particle that takes no part in the simulation (an unused particle of a
// serving slot): it is in no cell and no row, and the completion kernels skip it. Callers' hold
// masks may not carry it (LG_HOLD_* are bits 0..3).
constexpr uint32_t kHoldInactive = 16u;
__device__ __forceinline__ bool inactive_of(const uint8_t *hold, int64_t i) {
    return hold && (hold[i] & kHoldInactive);
}

// Kick of one half step, v + h * a, unless a step handler holds that increment.
__device__ __forceinline__ d3 kick_unless(d3 v, double h, d3 a, bool held) { return held ? v : add(v, scl(h, a)); }
__device__ __forceinline__ uint32_t hold_of(const uint8_t *hold, int64_t i) { return hold ? (uint32_t)hold[i] : 0u; }

// Spring component c (0..8: xi_t, xi_r, xi_o) of slot e in a spring array of `stride` slots:
// component-major (c * stride + e, the FP64 kernels' layout: a warp reading slot k of consecutive
// rows coalesces) or, with `aos` (mixed precision, whose kernels reach slots through compacted
// queues in no row order), one record of 9 consecutive 8-byte components per slot (a pair touches 3
// sectors instead of 9).
__host__ __device__ __forceinline__ int64_t spring_at(int32_t aos, int c, int64_t e, int64_t stride) {
    return aos ? e * 9 + c : (int64_t)c * stride + e;
}

// Entry flags of a pair slot (Verlet list slot or implicit all-pairs slot)
constexpr uint32_t kXiLive = 1u;      // contact springs may be nonzero
constexpr uint32_t kBonded = 2u;      // pair is an intact sintered bond; bond slot in bits 8..15
__host__ __device__ __forceinline__ uint32_t bond_slot_of(uint32_t f) { return (f >> 8) & 0xffu; }

// Device-side views of the pair data. Slot e = k * n + i (column-major "ELL" layout: slot k of
// every row is contiguous, so the threads of a warp reading slot k of consecutive rows coalesce).
struct PairView {
    int32_t *nbr;       // [cap * n] neighbour index (Verlet mode)
    int32_t *row_len;   // [n] (Verlet mode)
    uint32_t *flags;    // [cap * n]
    double *xi;         // [9][cap * n] contact springs, component-major (8-byte slots: FP64 values,
                        // or float-float pairs when Params::springs_ff is set)
    int64_t cap;        // slots per row
    // Contact candidates of each row (mixed precision, Verlet mode; null otherwise): the slots whose
    // pair was within the near radius (contact reach + Verlet skin) at the last build, or bonded,
    // in ascending slot order: entry m of row i at m * n + i.
    int32_t *near_j;    // [cap * n] partner
    uint8_t *near_k;    // [cap * n] slot in the row
    int32_t *near_len;  // [n]
    int32_t aos;        // springs as one 9-component record per slot (spring_at)
};

struct BondView {
    int32_t *j;         // [bcap * n] partner of bond slot b of row i (-1 = none)
    int8_t *intact;     // [bcap * n]
    double *strength;   // [bcap * n]
    double *xi;         // [9][bcap * n] bond springs
    int32_t bcap;       // bond slots per row
    // 5-connector model (null otherwise): the five connectors that particle i carries for its bond
    // slot b, component-major (connector k, component c at (3k + c) * bcap * n + b * n + i), and the
    // slot of i in the partner's bond list
    double *cn;         // [15][bcap * n]
    int32_t *rev;       // [bcap * n]
    int32_t aos;        // bond springs as one 9-component record per bond slot (spring_at)
};

struct StateView {
    dbl4 *x, *v, *th, *w;        // positions, velocities (half step inside a step), orientation, spin
    dbl4 *a, *al;                // accelerations of the last force evaluation
    dbl4 *v_out, *w_out;         // full-step velocities written by the force kernel
    double *sxi;                    // [n_facets][9][n] surface contact springs
    double *facet_vert;             // [n_facets * 9] vertices read this step
    double *facet_vert_next;        // [n_facets * 9] vertices after this step's move
    int32_t *err;                   // device error word
};

#ifdef __CUDACC__
// ------------------------------------------------------------------------------------------------
// FP64 functors
// ------------------------------------------------------------------------------------------------
// FAST = true: where libgran divides a vector by a scalar (normalisation, division by a mass or an
// inertia) the vector is multiplied by one reciprocal; every value stays within a few ulp of the
// reference's (per-step forces within
// 1e-12 of it), but not bit-identical. FAST = false is the reference's arithmetic, operation for
// operation. Normals whose overlap 2r - dx.n is a small difference of large numbers (contact, bond)
// keep the reference's division in both forms: with a reciprocal there, a bonded aggregate's forces
// moved by 2.2e-12 of their largest value.
template <bool FAST>
__device__ __forceinline__ d3 dvs_t(d3 a, double s) {
    if (FAST) {
        const double r = 1.0 / s;
        return mk3(a.x * r, a.y * r, a.z * r);
    }
    return dvs(a, s);
}
template <bool FAST>
__device__ __forceinline__ d3 nrmz_t(d3 a) {
    const double z = sqn(a);
    return z > 0.0 ? dvs_t<FAST>(a, sqrt(z)) : a;
}

// contact_force.h:105-147
template <bool FAST = false>
__device__ __forceinline__ d3 shear_coulomb(d3 &xi, d3 n, double stiffness, double damping, double normal_force,
                                            double mu_static, double phi_dynamic, d3 rel, double dt) {
    double mu_dynamic = mu_static * phi_dynamic;
    d3 xi_new = sub(xi, scl(dot(xi, n), n));
    if (nrm(xi_new) > 0.0) {
        double z = sqn(xi_new);
        if (z > 0.0) xi_new = dvs_t<FAST>(xi_new, sqrt(z));
        double old = nrm(xi);
        xi_new = scl(old, xi_new);
    }
    xi = xi_new;
    d3 f0 = sub(scl(-stiffness, xi), scl(damping, rel));
    double static_friction = mu_static * normal_force;
    double dynamic_friction = mu_dynamic * normal_force;
    double f0n = nrm(f0);
    d3 t = (f0n > 0.0) ? (FAST ? dvs_t<true>(f0, f0n) : nrmz(f0)) : zero3();
    double f_selected;
    if (f0n <= static_friction) {
        xi = add(xi, scl(dt, rel));
        f_selected = static_friction;
    } else {
        xi = scl(-1.0 / stiffness, add(scl(dynamic_friction, t), scl(damping, rel)));
        f_selected = dynamic_friction;
    }
    double m = (f0n < f_selected) ? f0n : f_selected;
    return scl(m, t);
}

// alt_sinter_bridge.h:137-156
template <bool FAST = false>
__device__ __forceinline__ d3 shear_bond(d3 &xi, d3 n, double stiffness, double damping, d3 rel, double dt) {
    d3 xi_new = sub(xi, scl(dot(xi, n), n));
    if (nrm(xi_new) > 0.0) {
        double z = sqn(xi_new);
        if (z > 0.0) xi_new = dvs_t<FAST>(xi_new, sqrt(z));
        double old = nrm(xi);
        xi_new = scl(old, xi_new);
    }
    xi = xi_new;
    d3 f0 = sub(scl(-stiffness, xi), scl(damping, rel));
    xi = add(xi, scl(dt, rel));
    return f0;
}

// FP64 overlap of a contact pair exactly as the FP64 path computes it (contact_force.h:65-66:
// n = dx / |dx|, overlap = 2r - dx.n with dx = x_i - x_j), every operation rounded on its own.
__device__ __forceinline__ double overlap_fp64(const dbl4 *x, int64_t i, int64_t j, double r) {
    const dbl4 a = x[i], b = x[j];
    const double dx = __dsub_rn(a.x, b.x), dy = __dsub_rn(a.y, b.y), dz = __dsub_rn(a.z, b.z);
    const double z = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    if (z == 0.0) return __dmul_rn(2.0, r);
    const double s = __dsqrt_rn(z);
    const double nx = __ddiv_rn(dx, s), ny = __ddiv_rn(dy, s), nz = __ddiv_rn(dz, s);
    const double d = __dadd_rn(__dadd_rn(__dmul_rn(dx, nx), __dmul_rn(dy, ny)), __dmul_rn(dz, nz));
    return __dsub_rn(__dmul_rn(2.0, r), d);
}

// contact_force.h:57-96 -- the in-contact branch (caller has established overlap > 0 with the
// reference's own arithmetic, n and overlap are passed in).
template <bool FAST = false>
__device__ __forceinline__ void contact_touching(const lg_contact_params &p, d3 n, double overlap, d3 vi, d3 vj,
                                                 d3 wi, d3 wj, d3 *s, d3 &oa, d3 &oal) {
    double rp = p.r_part - overlap / 2.0;
    double v_n = -dot(sub(vi, vj), n);
    double f_n = p.k * overlap + p.gamma_n * v_n;
    d3 nwi = crs(n, wi), nwj = crs(n, wj);
    d3 v_ij = add(add(sub(vi, vj), scl(rp, nwi)), scl(rp, nwj));
    d3 v_t = sub(v_ij, scl(dot(v_ij, n), n));
    d3 v_r = scl(-rp, sub(nwi, nwj));
    d3 v_o = scl(p.r_part * (dot(n, wi) - dot(n, wj)), n);
    d3 f_t = shear_coulomb<FAST>(s[0], n, p.k_t, p.gamma_t, f_n, p.mu_s, p.phi_d, v_t, p.dt);
    d3 f_r = shear_coulomb<FAST>(s[1], n, p.k_r, p.gamma_r, f_n, p.mu_r, p.phi_r, v_r, p.dt);
    d3 f_o = shear_coulomb<FAST>(s[2], n, p.k_o, p.gamma_o, f_n, p.mu_o, p.phi_o, v_o, p.dt);
    d3 tau_t = scl(rp, crs(n, f_t));
    d3 tau_r = scl(p.r_part, crs(n, f_r));
    d3 tau_o = scl(p.r_part, f_o);
    oa = dvs_t<FAST>(add(scl(f_n, n), f_t), p.mass);
    oal = dvs_t<FAST>(add(add(neg(tau_t), tau_r), tau_o), p.inertia);
}

// alt_sinter_bridge.h:103-128 / alt_breaking_sinter_bridge.h:89-121. Returns true when the
// breaking variant breaks the (i, j) bond (|f_tot| > strength, alt_breaking_sinter_bridge.h:118).
template <bool FAST = false>
__device__ __forceinline__ bool bond_force(const lg_sinter_params &p, d3 dx, d3 vi, d3 vj, d3 wi, d3 wj, d3 *s,
                                           bool breaking, double strength, d3 &oa, d3 &oal) {
    // the normal keeps the reference's division even in FAST: the overlap 2r - dx.n of a bonded pair
    // is a small difference of large numbers, so an ulp of n is a large part of it
    d3 n = nrmz(dx);
    double overlap = 2.0 * p.r_part - dot(dx, n);
    double rp = p.r_part - overlap / 2.0;
    double v_n = -dot(sub(vi, vj), n);
    double f_n = p.k * overlap + p.gamma_n * v_n;
    d3 nwi = crs(n, wi), nwj = crs(n, wj);
    d3 v_ij = add(add(sub(vi, vj), scl(rp, nwi)), scl(rp, nwj));
    d3 v_t = sub(v_ij, scl(dot(v_ij, n), n));
    d3 v_r = scl(-rp, sub(nwi, nwj));
    d3 v_o = scl(p.r_part * (dot(n, wi) - dot(n, wj)), n);
    d3 f_t = shear_bond<FAST>(s[0], n, p.k_t, p.gamma_t, v_t, p.dt);
    d3 f_r = shear_bond<FAST>(s[1], n, p.k_r, p.gamma_r, v_r, p.dt);
    d3 f_o = shear_bond<FAST>(s[2], n, p.k_o, p.gamma_o, v_o, p.dt);
    d3 tau_t = scl(rp, crs(n, f_t));
    d3 tau_r = scl(p.r_part, crs(n, f_r));
    d3 tau_o = scl(p.r_part, f_o);
    d3 f_tot = add(scl(f_n, n), f_t);
    d3 tau_tot = add(add(neg(tau_t), tau_r), tau_o);
    bool brk = breaking && (nrm(f_tot) > strength);
    oa = dvs_t<FAST>(f_tot, p.mass);
    oal = dvs_t<FAST>(tau_tot, p.inertia);
    return brk;
}

// sinter_functor::bonded_contact_accelerations (sinter_bridge.h:238-266): five connector springs
// between the connectors of i (bond slot ei) and those of j (its slot ej for i); rest lengths 2 r
// for the four side springs, 0 for the centre spring (sinter_bridge.h:201-206).
__device__ __forceinline__ void connector_force(const lg_connector_params &cp, double r, double mass, double inertia,
                                                d3 xi, d3 xj, d3 vi, d3 vj, d3 wi, d3 wj, const double *cn,
                                                int64_t bs, int64_t ei, int64_t ej, d3 &oa, d3 &oal) {
    d3 force = zero3(), torque = zero3();
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const d3 ci = mk3(cn[(3 * k) * bs + ei], cn[(3 * k + 1) * bs + ei], cn[(3 * k + 2) * bs + ei]);
        const d3 cj = mk3(cn[(3 * k) * bs + ej], cn[(3 * k + 1) * bs + ej], cn[(3 * k + 2) * bs + ej]);
        const d3 spring = sub(cj, ci);
        const double len = nrm(spring);
        const double eq = k < 4 ? 2.0 * r : 0.0;
        const d3 cvi = add(vi, crs(wi, sub(ci, xi)));
        const d3 cvj = add(vj, crs(wj, sub(cj, xj)));
        const d3 rel = sub(cvj, cvi);
        const d3 df = add(scl(-(eq - len) * cp.k_d, nrmz(spring)), scl(cp.gamma_d, rel));
        force = add(force, df);
        torque = add(torque, crs(sub(ci, xi), df));
    }
    oa = dvs(force, mass);
    oal = dvs(torque, inertia);
}

__device__ __forceinline__ double sq_(double x) { return x * x; }
__device__ __forceinline__ double cb_(double x) { return x * x * x; }

// hamaker_force.h:28-43 / limited_range_hamaker_force.h:33-45 / simplified_hamaker_force.h:23-29.
// r = x_j - x_i. Angular part is zero. The limited variant's cutoff test is done by the caller.
__device__ __forceinline__ d3 hamaker_accel(int mode, const lg_hamaker_params &p, d3 r) {
    double h = nrm(r) - 2.0 * p.r_part;
    if (h < p.h0) h = p.h0;
    double rp = p.r_part;
    double s;
    if (mode == LG_HAMAKER_SIMPLIFIED) {
        s = 2.0 * p.A * rp / sq_(h);
    } else {
        double br = (4.0 * rp + 2.0 * h) / (4.0 * rp + h) / h - 2.0 / (2.0 * rp + h) - 4.0 * sq_(rp) / cb_(2.0 * rp + h) -
                    2.0 * sq_(rp) * (4.0 * rp + 2.0 * h) / sq_(4.0 * rp + h) / sq_(h);
        s = -p.A / 6.0 * br;
    }
    return dvs(scl(s, nrmz(r)), p.mass);
}

// As hamaker_accel, with rn = nrm(r) already computed (the same value nrm() and nrmz() would compute).
// FAST: the bracket over one common denominator, D = (4r + h) h (2r + h), with u = 1 / ((4r + h) h)
// = (2r + h) / D and w = 1 / (2r + h) = (4r + h) h / D:
//   (4r+2h) u - 2 w - 4 r^2 w^3 - 2 r^2 (4r+2h) u^2,
// and the scaling by 1 / (|r| m) as one factor: two divisions per pair instead of twelve.
template <bool FAST = false>
__device__ __forceinline__ d3 hamaker_accel_n(int mode, const lg_hamaker_params &p, d3 r, double rn) {
    double h = rn - 2.0 * p.r_part;
    if (h < p.h0) h = p.h0;
    double rp = p.r_part;
    double s;
    if (FAST && mode != LG_HAMAKER_SIMPLIFIED) {
        const double q = 4.0 * rp + h, w0 = 2.0 * rp + h, a = 4.0 * rp + 2.0 * h;
        const double inv = 1.0 / (q * h * w0);
        const double u = w0 * inv, w = q * h * inv;
        const double br = a * u - 2.0 * w - 4.0 * sq_(rp) * (w * w * w) - 2.0 * sq_(rp) * a * (u * u);
        s = -p.A / 6.0 * br;
        return rn > 0.0 ? scl(s / (rn * p.mass), r) : dvs_t<true>(scl(s, r), p.mass);
    }
    if (mode == LG_HAMAKER_SIMPLIFIED) {
        s = 2.0 * p.A * rp / sq_(h);
    } else {
        double br = (4.0 * rp + 2.0 * h) / (4.0 * rp + h) / h - 2.0 / (2.0 * rp + h) - 4.0 * sq_(rp) / cb_(2.0 * rp + h) -
                    2.0 * sq_(rp) * (4.0 * rp + 2.0 * h) / sq_(4.0 * rp + h) / sq_(h);
        s = -p.A / 6.0 * br;
    }
    if (FAST) return rn > 0.0 ? scl(s / (rn * p.mass), r) : dvs_t<true>(scl(s, r), p.mass);
    d3 u = (rn > 0.0) ? dvs(r, rn) : r;  // nrmz(r)
    return dvs(scl(s, u), p.mass);
}

// triangular_facet.h:73-137
__device__ __forceinline__ d3 closest_point_on_triangle(const double *vt, double area, d3 N, d3 p) {
    d3 v0 = mk3(vt[0], vt[1], vt[2]), v1 = mk3(vt[3], vt[4], vt[5]), v2 = mk3(vt[6], vt[7], vt[8]);
    d3 off = scl(dot(v0, N), N);
    d3 proj = sub(p, scl(dot(p, N), N));
    d3 cp = add(proj, off);
    double s = 0.0;
    d3 pa = sub(v0, cp), pb = sub(v1, cp), pc = sub(v2, cp);
    s += 1.0 / 2.0 * nrm(crs(pa, pb));
    s += 1.0 / 2.0 * nrm(crs(pb, pc));
    s += 1.0 / 2.0 * nrm(crs(pc, pa));
    if (!(s > area)) return cp;
    d3 e[3];
    d3 vv[3] = {v0, v1, v2};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        d3 a = vv[k], b = vv[(k + 1) % 3];
        d3 L = sub(b, a);
        d3 uL = nrmz(L);
        d3 tp = sub(p, a);
        double len = nrm(L);
        double pr = dot(tp, uL);
        if (pr < 0.0)
            e[k] = a;
        else if (pr > len)
            e[k] = b;
        else
            e[k] = add(a, scl(pr, uL));
    }
    double d1 = sqn(sub(p, e[0])), d2 = sqn(sub(p, e[1])), d3_ = sqn(sub(p, e[2]));
    if (d1 < d2) {
        if (d1 < d3_) return e[0];
    } else {
        if (d2 < d3_) return e[1];
    }
    return e[2];
}

// surface_contact_force.h:57-96
__device__ __forceinline__ void surface_contact(const lg_contact_params &p, d3 xf, d3 vf, d3 xi_, d3 vi, d3 wi, d3 *s,
                                                d3 &oa, d3 &oal) {
    d3 dx = sub(xi_, xf);
    d3 n = nrmz(dx);
    double overlap = p.r_part - dot(dx, n);
    if (overlap <= 0) {
        s[0] = s[1] = s[2] = zero3();
        oa = zero3();
        oal = zero3();
        return;
    }
    double rp = p.r_part - overlap;
    double v_n = -dot(sub(vi, vf), n);
    double f_n = p.k * overlap + p.gamma_n * v_n;
    d3 nwi = crs(n, wi);
    d3 v_ij = add(sub(vi, vf), scl(rp, nwi));
    d3 v_t = sub(v_ij, scl(dot(v_ij, n), n));
    d3 v_r = scl(-rp, nwi);
    d3 v_o = scl(p.r_part * dot(n, wi), n);
    d3 f_t = shear_coulomb(s[0], n, p.k_t, p.gamma_t, f_n, p.mu_s, p.phi_d, v_t, p.dt);
    d3 f_r = shear_coulomb(s[1], n, p.k_r, p.gamma_r, f_n, p.mu_r, p.phi_r, v_r, p.dt);
    d3 f_o = shear_coulomb(s[2], n, p.k_o, p.gamma_o, f_n, p.mu_o, p.phi_o, v_o, p.dt);
    d3 tau_t = scl(rp, crs(n, f_t));
    d3 tau_r = scl(p.r_part, crs(n, f_r));
    d3 tau_o = scl(p.r_part, f_o);
    oa = dvs(add(scl(f_n, n), f_t), p.mass);
    oal = dvs(add(add(neg(tau_t), tau_r), tau_o), p.inertia);
}

// surface_hamaker_force.h:18-30
__device__ __forceinline__ d3 surface_hamaker(const lg_hamaker_params &p, d3 xf, d3 xi_) {
    d3 r = sub(xf, xi_);
    double h = nrm(r) - p.r_part;
    if (h < p.h0) h = p.h0;
    double s = 2.0 * p.A / 3.0 * (cb_(p.r_part) / sq_(h) / sq_(h + 2.0 * p.r_part));
    return dvs(scl(s, nrmz(r)), p.mass);
}

__device__ __forceinline__ void set_error(int32_t *err, int32_t bit) {
    if (err) atomicOr(err, bit);
}
#endif  // __CUDACC__

}  // namespace lg
