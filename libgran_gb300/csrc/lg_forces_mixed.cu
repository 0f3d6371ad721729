// lg_forces_mixed.cu -- mixed-precision row-group force kernel (sm_103a; on request or by the
// autotuner: the compacted kernels of lg_forces_compact_mixed.cu are the automatic choice), the
// mixed drift and the float-float copies.
//
// Which steps keep FP64 and why (GB300 issues FP64 at about 1/58 of its FP32 rate, so every FP64
// operation here is spent where cancellation or accumulation needs it):
//   FP64  separation x_i - x_j of every pair that can interact, the squared distance and
//         q = |d|^2 - (2r)^2 (the overlap is -q / (|d| + 2r): its leading digits cancel at
//         nanometre overlaps), the spring vectors xi and their updates (stored, like every mixed
//         kernel's springs, as float-float pairs: ffslot_load / ffslot_store), the per-particle
//         force/torque sums, and the velocity-Verlet integration.
//   FP32  everything else in the pair: unit normal, relative velocities, normal force, Coulomb
//         test, torques, the Hamaker bracket (rewritten with two reciprocals).
// Pairs are culled with the high parts of the float-float positions (relative to a per-system
// origin) against a radius with a 1e-3 margin, so pairs that cannot touch and lie beyond the
// Hamaker cutoff cost no FP64 work. Row groups, slot layout and flags are shared with the FP64 path
// (lg_common.cuh); springs use the mixed path's float-float records (spring_at).
#include "lg_compact.cuh"
#include "lg_kernels.h"

namespace lg {

bool mixed_available() { return true; }

struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 fm(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 fadd(f3 a, f3 b) { return fm(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 fsub(f3 a, f3 b) { return fm(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 fscl(float s, f3 a) { return fm(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float fdot(f3 a, f3 b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)); }
__device__ __forceinline__ f3 fcrs(f3 a, f3 b) {
    return fm(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ f3 tof(d3 a) { return fm((float)a.x, (float)a.y, (float)a.z); }
__device__ __forceinline__ f3 ld4f(const dbl4 *p, int64_t i) {
    dbl4 q = p[i];
    return fm((float)q.x, (float)q.y, (float)q.z);
}
__device__ __forceinline__ void accum(d3 &acc, f3 a) {
    acc.x += (double)a.x;
    acc.y += (double)a.y;
    acc.z += (double)a.z;
}

// Coulomb-capped shear spring (contact_force.h:105-147) with an FP64 spring. The rotation onto the
// tangent plane subtracts (xi.n) n and restores the old magnitude; both are small corrections
// computed in FP32 and applied to the FP64 spring.
__device__ __forceinline__ f3 shear_mixed(d3 &xi, f3 n, float stiffness, float damping, float normal_force,
                                          float mu_static, float phi_dynamic, f3 rel, double dt, bool coulomb) {
    f3 xf = tof(xi);
    float xx = fdot(xf, xf);
    if (xx > 0.0f) {
        float c = fdot(xf, n);
        xi.x -= (double)(c * n.x);
        xi.y -= (double)(c * n.y);
        xi.z -= (double)(c * n.z);
        // |xi_new|^2 = |xi|^2 - c^2 in exact arithmetic: rescale by 1/sqrt(1 - e), e = c^2/|xi|^2
        float e = (c * c) / xx;
        float sm1 = e < 1e-3f ? e * (0.5f + 0.375f * e) : rsqrtf(fmaxf(1.0f - e, 1e-30f)) - 1.0f;
        if (e < 1.0f) {
            double s = (double)sm1;
            xi.x += xi.x * s;
            xi.y += xi.y * s;
            xi.z += xi.z * s;
        }
        xf = tof(xi);
    }
    f3 f0 = fsub(fscl(-stiffness, xf), fscl(damping, rel));
    const float dtf = (float)dt;
    if (!coulomb) {  // bonded spring: uncapped, always stretches (alt_sinter_bridge.h:152-155)
        xi.x += (double)(rel.x * dtf);
        xi.y += (double)(rel.y * dtf);
        xi.z += (double)(rel.z * dtf);
        return f0;
    }
    float fs = mu_static * normal_force;
    float fd = mu_static * phi_dynamic * normal_force;
    float f0n2 = fdot(f0, f0);
    float f0n = sqrtf(f0n2);
    f3 t = f0n > 0.0f ? fscl(1.0f / f0n, f0) : fm(0.f, 0.f, 0.f);
    float sel;
    if (f0n <= fs) {
        xi.x += (double)(rel.x * dtf);
        xi.y += (double)(rel.y * dtf);
        xi.z += (double)(rel.z * dtf);
        sel = fs;
    } else {
        f3 nx = fscl(-1.0f / stiffness, fadd(fscl(fd, t), fscl(damping, rel)));
        xi = mk3((double)nx.x, (double)nx.y, (double)nx.z);
        sel = fd;
    }
    return fscl(fminf(sel, f0n), t);
}

// contact (contact_force.h:73-95) or bond (alt_sinter_bridge.h:106-128) with overlap > 0 known.
// Returns the force (not yet divided by mass) and torque (not yet divided by inertia) in FP32.
__device__ __forceinline__ void contact_mixed(float kn, float gn, float kt, float gt, float mus, float phid, float kr,
                                              float gr, float mur, float phir, float ko, float go, float muo, float phio,
                                              float r_part, double dt, bool coulomb, f3 n, float overlap, f3 vij0,
                                              f3 wi, f3 wj, d3 *s, f3 &force, f3 &torque) {
    float rp = r_part - 0.5f * overlap;
    float v_n = -fdot(vij0, n);
    float f_n = kn * overlap + gn * v_n;
    f3 nwi = fcrs(n, wi), nwj = fcrs(n, wj);
    f3 v_ij = fadd(vij0, fscl(rp, fadd(nwi, nwj)));
    f3 v_t = fsub(v_ij, fscl(fdot(v_ij, n), n));
    f3 v_r = fscl(-rp, fsub(nwi, nwj));
    f3 v_o = fscl(r_part * (fdot(n, wi) - fdot(n, wj)), n);
    f3 f_t = shear_mixed(s[0], n, kt, gt, f_n, mus, phid, v_t, dt, coulomb);
    f3 f_r = shear_mixed(s[1], n, kr, gr, f_n, mur, phir, v_r, dt, coulomb);
    f3 f_o = shear_mixed(s[2], n, ko, go, f_n, muo, phio, v_o, dt, coulomb);
    force = fadd(fscl(f_n, n), f_t);
    torque = fadd(fsub(fscl(r_part, fcrs(n, f_r)), fscl(rp, fcrs(n, f_t))), fscl(r_part, f_o));
}

// Hamaker magnitude factor s(h) of hamaker_force.h:36-40 written with two reciprocals:
// s = -A/6 [ (4r+2h) u - 2 w - 4 r^2 w^3 - 2 r^2 (4r+2h) u^2 ], u = 1/((4r+h) h), w = 1/(2r+h).
__device__ __forceinline__ float hamaker_factor_f(int mode, float A, float r, float h) {
    if (mode == LG_HAMAKER_SIMPLIFIED) return 2.0f * A * r / (h * h);
    float u = 1.0f / ((4.0f * r + h) * h);
    float w = 1.0f / (2.0f * r + h);
    float a = 4.0f * r + 2.0f * h;
    float br = a * u - 2.0f * w - 4.0f * r * r * (w * w * w) - 2.0f * r * r * a * (u * u);
    return -A / 6.0f * br;
}

template <int T>
__device__ __forceinline__ double group_sum_m(double v) {
#pragma unroll
    for (int o = T / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <int T, bool VERLET>
__global__ void __launch_bounds__(256) forces_mixed(Params P, StateView S, PairView PV, BondView BV, double hdt,
                                                    double dt, int move_facets, MixedExtra MX) {
    const int64_t n = P.n;
    const int64_t gid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t i = gid / T;
    const int lane = (int)(gid % T);
    const bool active = i < n;
    const int bm = P.binary_model, hm = P.hamaker_model;
    const bool breaking = bm == LG_BINARY_BREAKING_SINTER;

    if (move_facets && gid == 0) {
        for (int f = 0; f < P.n_facets; ++f)
            for (int q = 0; q < 9; ++q) S.facet_vert_next[9 * f + q] = S.facet_vert[9 * f + q] + P.facets[f].v[q % 3] * dt;
    }
    const lg_contact_params &C = P.contact;
    const lg_sinter_params &B = P.sinter;
    const float rc = (float)C.r_part;
    const double four_r2 = 4.0 * C.r_part * C.r_part;
    const double four_rb2 = 4.0 * B.r_part * B.r_part;
    const float rh = (float)P.hamaker.r_part;
    const double four_rh2 = 4.0 * P.hamaker.r_part * P.hamaker.r_part;
    const float Ah = (float)P.hamaker.A, h0 = (float)P.hamaker.h0;
    const float inv_mh = (float)(1.0 / P.hamaker.mass);

    d3 acc = zero3(), accw = zero3();  // contact/bond force and torque (before / mass, / inertia)
    d3 acch = zero3();                 // Hamaker acceleration
    d3 xi_ = zero3(), vi = zero3(), wi = zero3();
    f3 xfi = fm(0, 0, 0), vfi = fm(0, 0, 0), wfi = fm(0, 0, 0);
    if (active) {
        xi_ = ld4(S.x, i);
        vi = ld4(S.v, i);
        wi = ld4(S.w, i);
        vfi = tof(vi);
        wfi = tof(wi);
        float4 q = MX.x32[2 * i];
        xfi = fm(q.x, q.y, q.z);
        const int64_t len = VERLET ? (int64_t)PV.row_len[i] : n - 1;
        const int64_t xs = PV.cap * n;
        for (int64_t k = lane; k < len; k += T) {
            const int64_t e = k * n + i;
            const int64_t j = VERLET ? (int64_t)PV.nbr[e] : (k < i ? k : k + 1);
            const uint32_t fl = PV.flags[e];
            const float4 qj = MX.x32[2 * j];
            const f3 d32 = fm(xfi.x - qj.x, xfi.y - qj.y, xfi.z - qj.z);
            const float d2f = fdot(d32, d32);
            const bool bonded = (fl & kBonded) && bm != LG_BINARY_NONE;
            if (!bonded && d2f > MX.near2) {
                // cannot touch, beyond the limited Hamaker cutoff
                if (fl & kXiLive) {
#pragma unroll
                    for (int q2 = 0; q2 < 9; ++q2) PV.xi[spring_at(PV.aos, q2, e, xs)] = 0.0;
                    PV.flags[e] = fl & ~kXiLive;
                }
                if (hm == LG_HAMAKER_FULL || hm == LG_HAMAKER_SIMPLIFIED) {
                    float dist = sqrtf(d2f);
                    float h = fmaxf(dist - 2.0f * rh, h0);
                    float sfac = hamaker_factor_f(hm, Ah, rh, h) * inv_mh / dist;  // along r = x_j - x_i
                    f3 a = fscl(-sfac, d32);
                    accum(acch, a);
                }
                continue;
            }
            // near pair: FP64 separation
            const d3 dx = sub(xi_, ld4(S.x, j));
            const double d2 = fma(dx.z, dx.z, fma(dx.y, dx.y, dx.x * dx.x));
            const f3 df = tof(dx);
            const float dist = sqrtf((float)d2);
            const f3 nrm_ij = fscl(rsqrtf((float)d2), df);  // unit vector from j to i
            if (bm != LG_BINARY_NONE) {
                const double q4 = bonded ? four_rb2 : four_r2;
                const float rr = bonded ? (float)B.r_part : rc;
                const float overlap = (float)(q4 - d2) / (dist + 2.0f * rr);  // 2r - |d|
                bool touching = bonded || overlap > 0.0f;
                // at the contact distance to within rounding, the FP64 path's overlap decides
                if (!bonded && fabs(q4 - d2) <= (double)MX.q_marg)
                    touching = overlap_fp64(S.x, i, j, C.r_part) > 0.0;
                if (touching) {
                    const d3 vj = ld4(S.v, j), wj = ld4(S.w, j);
                    const f3 vij0 = tof(sub(vi, vj));
                    d3 s[3];
                    int64_t base, stride;
                    double *store;
                    int32_t aos;
                    if (bonded) {
                        base = (int64_t)bond_slot_of(fl) * n + i;
                        stride = (int64_t)BV.bcap * n;
                        store = BV.xi;
                        aos = BV.aos;
                    } else {
                        base = e;
                        stride = xs;
                        store = PV.xi;
                        aos = PV.aos;
                    }
                    if (bonded || (fl & kXiLive)) {  // springs of a slot that is not live are zero
#pragma unroll
                        for (int q3 = 0; q3 < 3; ++q3)
                            s[q3] = mk3(ffslot_load(store, spring_at(aos, 3 * q3, base, stride)),
                                        ffslot_load(store, spring_at(aos, 3 * q3 + 1, base, stride)),
                                        ffslot_load(store, spring_at(aos, 3 * q3 + 2, base, stride)));
                    } else {
                        s[0] = s[1] = s[2] = zero3();
                    }
                    f3 force, torque;
                    if (bonded)
                        contact_mixed((float)B.k, (float)B.gamma_n, (float)B.k_t, (float)B.gamma_t, 0.f, 0.f,
                                      (float)B.k_r, (float)B.gamma_r, 0.f, 0.f, (float)B.k_o, (float)B.gamma_o, 0.f,
                                      0.f, (float)B.r_part, B.dt, false, nrm_ij, overlap, vij0, tof(wi), tof(wj), s,
                                      force, torque);
                    else
                        contact_mixed((float)C.k, (float)C.gamma_n, (float)C.k_t, (float)C.gamma_t, (float)C.mu_s,
                                      (float)C.phi_d, (float)C.k_r, (float)C.gamma_r, (float)C.mu_r, (float)C.phi_r,
                                      (float)C.k_o, (float)C.gamma_o, (float)C.mu_o, (float)C.phi_o, rc, C.dt, true,
                                      nrm_ij, overlap, vij0, wfi, tof(wj), s, force, torque);
#pragma unroll
                    for (int q3 = 0; q3 < 3; ++q3) {
                        ffslot_store(store, spring_at(aos, 3 * q3, base, stride), s[q3].x);
                        ffslot_store(store, spring_at(aos, 3 * q3 + 1, base, stride), s[q3].y);
                        ffslot_store(store, spring_at(aos, 3 * q3 + 2, base, stride), s[q3].z);
                    }
                    if (bonded) {
                        if (breaking && fdot(force, force) > (float)(BV.strength[base] * BV.strength[base])) {
                            BV.intact[base] = 0;
                            PV.flags[e] = fl & ~(kBonded | (0xffu << 8));
                        }
                    } else if (!(fl & kXiLive)) {
                        PV.flags[e] = fl | kXiLive;
                    }
                    accum(acc, force);
                    accum(accw, torque);
                } else if (fl & kXiLive) {
#pragma unroll
                    for (int q2 = 0; q2 < 9; ++q2) PV.xi[spring_at(PV.aos, q2, e, xs)] = 0.0;
                    PV.flags[e] = fl & ~kXiLive;
                }
            }
            if (hm != LG_HAMAKER_NONE) {
                bool on = true;
                if (hm == LG_HAMAKER_LIMITED) on = !(d2 > MX.rcut2);
                if (on) {
                    float h = (float)(d2 - four_rh2) / (dist + 2.0f * rh);  // |d| - 2r
                    h = fmaxf(h, h0);
                    float sfac = hamaker_factor_f(hm, Ah, rh, h) * inv_mh;
                    f3 a = fscl(-sfac, nrm_ij);  // along r = x_j - x_i = -n
                    accum(acch, a);
                }
            }
        }
    }
    if (T > 1) {
        acc.x = group_sum_m<T>(acc.x);
        acc.y = group_sum_m<T>(acc.y);
        acc.z = group_sum_m<T>(acc.z);
        accw.x = group_sum_m<T>(accw.x);
        accw.y = group_sum_m<T>(accw.y);
        accw.z = group_sum_m<T>(accw.z);
        acch.x = group_sum_m<T>(acch.x);
        acch.y = group_sum_m<T>(acch.y);
        acch.z = group_sum_m<T>(acch.z);
    }
    if (!active || lane != 0) return;
    // masses of the contact and bond functors are the same particle's; both are honoured
    const double m_c = (bm == LG_BINARY_SINTER || bm == LG_BINARY_BREAKING_SINTER) ? B.mass : C.mass;
    const double I_c = (bm == LG_BINARY_SINTER || bm == LG_BINARY_BREAKING_SINTER) ? B.inertia : C.inertia;
    d3 a_tot = add(dvs(acc, m_c), acch);
    d3 al_tot = dvs(accw, I_c);
    compact::finish_row(P, S, i, n, a_tot, al_tot, vi, wi, hdt);
}

// Float-float copies of the positions (relative to the system origin; in a batch every system has
// its own origin) and of the velocities.
// With `uncovered` set, also flags (*uncovered = 1) any position further than four times its system's
// extent (orig.w, or `oext` for a single system) from the origin in some coordinate.
__global__ void mixed_copies(int64_t n, const dbl4 *__restrict__ x, const dbl4 *__restrict__ v,
                             const dbl4 *__restrict__ w, const dbl4 *__restrict__ th, double ox, double oy, double oz,
                             double oext, const int32_t *__restrict__ agg, const dbl4 *__restrict__ orig,
                             float4 *__restrict__ x32, float4 *__restrict__ v32, float4 *__restrict__ s32,
                             int32_t *uncovered) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const d3 xi = ld4(x, i);
    rel_ff(xi, ox, oy, oz, agg, orig, i, n, x32);
    state_ff(ld4(v, i), ld4(w, i), i, n, v32, s32);
    if (uncovered) {
        if (agg) {
            const dbl4 o = orig[agg[i]];
            ox = o.x;
            oy = o.y;
            oz = o.z;
            oext = o.w;
        }
        const double lim = 4.0 * oext;
        if (!(fabs(xi.x - ox) <= lim && fabs(xi.y - oy) <= lim && fabs(xi.z - oz) <= lim)) atomicOr(uncovered, 1);
    }
}

// Kick + drift of the mixed path: FP64 integration, then the float-float position copy.
__global__ void kick_drift_mixed(int64_t n, dbl4 *__restrict__ x, dbl4 *__restrict__ v, dbl4 *__restrict__ th,
                                 dbl4 *__restrict__ w, const dbl4 *__restrict__ a, const dbl4 *__restrict__ al,
                                 double dt, double hdt, double ox, double oy, double oz,
                                 const int32_t *__restrict__ agg, const dbl4 *__restrict__ orig,
                                 float4 *__restrict__ x32, float4 *__restrict__ v32, float4 *__restrict__ s32,
                                 const uint8_t *__restrict__ hold) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t h = hold_of(hold, i);
    d3 vi = kick_unless(ld4(v, i), hdt, ld4(a, i), h & LG_HOLD_V);
    d3 wi = kick_unless(ld4(w, i), hdt, ld4(al, i), h & LG_HOLD_OMEGA);
    st4(v, i, vi);
    st4(w, i, wi);
    d3 xn = ld4(x, i);
    if (!(h & LG_HOLD_X)) {
        xn = add(xn, scl(dt, vi));
        st4(x, i, xn);
    }
    if (!(h & LG_HOLD_THETA)) st4(th, i, add(ld4(th, i), scl(dt, wi)));
    rel_ff(xn, ox, oy, oz, agg, orig, i, n, x32);
    state_ff(vi, wi, i, n, v32, s32);
}

template <int T, bool VERLET>
static void launch_mixed_t(const Params &P, const StateView &S, const PairView &PV, const BondView &BV, double hdt,
                           double dt, int move_facets, const MixedExtra &MX, cudaStream_t st) {
    const int threads = 256;
    const int64_t total = P.n * T;
    const int64_t blocks = (total + threads - 1) / threads;
    forces_mixed<T, VERLET><<<(unsigned)(blocks > 0 ? blocks : 1), threads, 0, st>>>(P, S, PV, BV, hdt, dt, move_facets,
                                                                                   MX);
}

void launch_forces_mixed(int T, const Params &P, const StateView &S, const PairView &PV, const BondView &BV, double hdt,
                         double dt, int move_facets, const MixedExtra &MX, cudaStream_t st) {
    const bool ver = P.pairs == LG_PAIRS_VERLET;
#define LG_CASE(TT)                                                                   \
    case TT:                                                                          \
        if (ver)                                                                      \
            launch_mixed_t<TT, true>(P, S, PV, BV, hdt, dt, move_facets, MX, st);     \
        else                                                                          \
            launch_mixed_t<TT, false>(P, S, PV, BV, hdt, dt, move_facets, MX, st);    \
        break;
    switch (T) {
        LG_CASE(1)
        LG_CASE(2)
        LG_CASE(4)
        LG_CASE(8)
        LG_CASE(16)
        LG_CASE(32)
        default:
            launch_mixed_t<1, false>(P, S, PV, BV, hdt, dt, move_facets, MX, st);
    }
#undef LG_CASE
}

void launch_mixed_copies(int64_t n, const dbl4 *x, const dbl4 *v, const dbl4 *w, const dbl4 *th, const double *origin,
                         const int32_t *agg, const dbl4 *orig, float4 *x32, float4 *v32, float4 *s32, cudaStream_t st,
                         int32_t *uncovered) {
    const int threads = 64;  // small blocks: all SMs get work at moderate n
    int64_t blocks = (n + threads - 1) / threads;
    if (blocks == 0) return;
    mixed_copies<<<(unsigned)blocks, threads, 0, st>>>(n, x, v, w, th, origin[0], origin[1], origin[2], origin[3], agg,
                                                       orig, x32, v32, s32, uncovered);
}

void launch_kick_drift_mixed(int64_t n, dbl4 *x, dbl4 *v, dbl4 *th, dbl4 *w, const dbl4 *a, const dbl4 *al, double dt,
                             double hdt, const double *origin, const int32_t *agg, const dbl4 *orig, float4 *x32,
                             float4 *v32, float4 *s32, const uint8_t *hold, cudaStream_t st) {
    const int threads = 64;  // small blocks: all SMs get work at moderate n
    int64_t blocks = (n + threads - 1) / threads;
    if (blocks == 0) return;
    kick_drift_mixed<<<(unsigned)blocks, threads, 0, st>>>(n, x, v, th, w, a, al, dt, hdt, origin[0], origin[1],
                                                           origin[2], agg, orig, x32, v32, s32, hold);
}

}  // namespace lg
