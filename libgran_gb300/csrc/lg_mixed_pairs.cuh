// lg_mixed_pairs.cuh -- the per-pair and per-row pieces of the mixed-precision force evaluation,
// shared by the kernels of lg_forces_compact_mixed.cu (contacts and Hamaker on two streams, then a
// completion kernel) and the persistent step kernel of lg_step_mixed.cu (the same rows as work items
// of one launch). Inline device code only: each translation unit compiles it with its own flags
// (both with approximate FP32 division and square root in the pair formulas; the float-float steps
// use explicitly rounded intrinsics).
//
// Precision: positions come as interleaved float-float pairs (MixedExtra::x32, hi + lo = x -
// origin) and a pair's separation and q = |d|^2 - (2r)^2 are formed with error-free FP32
// transformations (separation_ff), so the surface gap and the overlap keep FP32 relative precision
// however small they are; velocities come as float-float copies (MixedExtra::v32); springs are
// float-float pairs in 8-byte slots, one 9-component record per slot or bond (spring_at), updated
// by FP32 increments (shear_ff). No pair costs an FP64 operation, except the FP64 overlap of a pair
// at the contact threshold (overlap_fp64). Per-row sums are float-float (compensated) FP32
// accumulations in an order fixed by the row alone.
#pragma once
#include <cstddef>

#include "lg_compact.cuh"
#include "lg_kernels.h"

namespace lg {
namespace mixed {

using compact::kHCap;
using compact::kWin;

// ---- contact / bond items ----
constexpr int kCRound = 32;  // entries per lane classified per round
constexpr int kCQ = 64;      // contact queue capacity (>= 32 + 31)
#ifndef LG_CONTACT_LANES
#define LG_CONTACT_LANES 2   // lanes per row (compile-time override for tuning)
#endif
constexpr int kContactLanes = LG_CONTACT_LANES;
struct ContactSmem {
    float cres[kCQ][6];  // results: linear and angular acceleration
    float4 chj[kCQ];     // partner's position, high part (read while classifying)
    int32_t cj[kCQ];     // partner
    int32_t ck[kCQ];     // slot in the owner's row
    uint32_t cfl[kCQ];   // the slot's flags (read while classifying)
    uint8_t cown[kCQ];   // owner lane
    uint32_t cball[kCRound];
    int32_t cbase[kCRound];
    float4 xh[32], xl[32];  // the rows' own positions (float-float)
    float4 vh[32], vl[32];  // the rows' own velocities (float-float)
    float4 wh[32];          // the rows' own spins (FP32)
};

// ---- Hamaker items ----
struct HamakerSmem {
    float4 hhi[kHCap];     // queued Hamaker partners: high part of the position, w = owner lane
    float4 hlo[kHCap];     // low part of the position
    float hres[kHCap][3];  // their accelerations
    float4 xh[32], xl[32];  // the rows' own positions (float-float)
};
static_assert(sizeof(HamakerSmem::hhi) >= 6 * 32 * sizeof(float), "slice partial sums reuse hhi");

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

// Hamaker factor of hamaker_force.h:36-40 with two reciprocals:
// s = -A/6 [ (4r+2h) u - 2 w - 4 r^2 w^3 - 2 r^2 (4r+2h) u^2 ], u = 1/((4r+h) h), w = 1/(2r+h).
__device__ __forceinline__ float ham_factor(int mode, float A, float r, float h) {
    if (mode == LG_HAMAKER_SIMPLIFIED) return 2.0f * A * r / (h * h);
    float u = 1.0f / ((4.0f * r + h) * h);
    float w = 1.0f / (2.0f * r + h);
    float a = 4.0f * r + 2.0f * h;
    float br = a * u - 2.0f * w - 4.0f * r * r * (w * w * w) - 2.0f * r * r * a * (u * u);
    return -A / 6.0f * br;
}

// Float-float arithmetic (a value is hi + lo with |lo| <= ulp(hi) / 2). The _rn intrinsics keep the
// compiler from contracting or reordering the error-free steps.
struct ff {
    float hi, lo;
};
// TwoSum (Knuth): s + e == a + b exactly, whatever the magnitudes of a and b.
__device__ __forceinline__ ff two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return ff{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
// Compensated accumulation a += b: the rounding error of every addition is kept in a.lo.
__device__ __forceinline__ void ff_acc(ff &a, float b) {
    const ff s = two_sum(a.hi, b);
    a.hi = s.hi;
    a.lo = __fadd_rn(a.lo, s.lo);
}
// a += b for a stored spring component, renormalised so that |lo| <= ulp(hi) / 2 again.
__device__ __forceinline__ void ff_add_norm(ff &a, float b) {
    const ff s = two_sum(a.hi, b);
    const float lo = __fadd_rn(a.lo, s.lo);
    const float hi = __fadd_rn(s.hi, lo);
    a = ff{hi, __fsub_rn(lo, __fsub_rn(hi, s.hi))};
}

// Shear spring (contact_force.h:105-147, Coulomb-capped; alt_sinter_bridge.h:137-156, bond form)
// with the spring vector held as float-float components. Each evaluation computes, in FP32, the
// increment of the spring: the rotation onto the tangent plane, -(xi.n) n, the rescale to the old
// magnitude, (s - 1)(xi - (xi.n) n) with s - 1 evaluated as a series for small tilts, and the
// stretch rel*dt; the increment is small next to xi and is added to the float-float spring, so
// rounding does not accumulate at the spring's own scale. The dynamic (sliding) branch sets the
// spring outright.
__device__ __forceinline__ f3 shear_ff(ff (&xi)[3], f3 n, float stiffness, float damping, float normal_force,
                                       float mu_s, float phi, f3 rel, float dtf, bool coulomb) {
    const f3 xf = fm(xi[0].hi, xi[1].hi, xi[2].hi);  // the FP32 rounding of the spring
    f3 drot = fm(0.f, 0.f, 0.f);
    const float xx = fdot(xf, xf);
    if (xx > 0.0f) {
        const float c = fdot(xf, n);
        const f3 xr = fsub(xf, fscl(c, n));
        const float e = (c * c) / xx;
        float sm1 = 0.0f;
        if (e < 1.0f) sm1 = e < 1e-3f ? e * (0.5f + 0.375f * e) : rsqrtf(1.0f - e) - 1.0f;
        drot = fadd(fscl(-c, n), fscl(sm1, xr));
    }
    const f3 xn = fadd(xf, drot);
    const f3 f0 = fsub(fscl(-stiffness, xn), fscl(damping, rel));
    if (!coulomb) {
        const f3 dxi = fadd(drot, fscl(dtf, rel));
        ff_add_norm(xi[0], dxi.x);
        ff_add_norm(xi[1], dxi.y);
        ff_add_norm(xi[2], dxi.z);
        return f0;
    }
    const float fs = mu_s * normal_force;
    const float fd = mu_s * phi * normal_force;
    const float f0n = sqrtf(fdot(f0, f0));
    const f3 t = f0n > 0.0f ? fscl(1.0f / f0n, f0) : fm(0.f, 0.f, 0.f);
    float sel;
    if (f0n <= fs) {
        const f3 dxi = fadd(drot, fscl(dtf, rel));
        ff_add_norm(xi[0], dxi.x);
        ff_add_norm(xi[1], dxi.y);
        ff_add_norm(xi[2], dxi.z);
        sel = fs;
    } else {
        const f3 nx = fscl(-1.0f / stiffness, fadd(fscl(fd, t), fscl(damping, rel)));
        xi[0] = ff{nx.x, 0.f};
        xi[1] = ff{nx.y, 0.f};
        xi[2] = ff{nx.z, 0.f};
        sel = fd;
    }
    return fscl(fminf(sel, f0n), t);
}

// Separation d = x_i - x_j (FP32) and q = |d|^2 - (2r)^2 from float-float positions. Per component
// the high parts' difference is split exactly (TwoSum) and its error joins the low parts'
// difference, so dh + dl equals the separation to about 2^-48 of the coordinates. Then
// (dh + dl)^2 = dh^2 + dl (2 dh + dl) with dh^2 split exactly by FMA, the three large squares added
// with TwoSum, and -(2r)^2 (fr_hi + fr_lo) subtracted: that subtraction is exact (Sterbenz) whenever
// |d| is within a factor sqrt(2) of 2r, and otherwise |q| >= 2 r^2, so q keeps FP32 relative
// precision however small the surface gap or the overlap is.
struct SepFF {
    f3 d;
    float q;
};
__device__ __forceinline__ SepFF separation_ff(float4 hi, float4 lo, float4 hj, float4 lj, float fr_hi, float fr_lo) {
    const ff tx = two_sum(hi.x, -hj.x), ty = two_sum(hi.y, -hj.y), tz = two_sum(hi.z, -hj.z);
    const float lx = __fadd_rn(tx.lo, __fsub_rn(lo.x, lj.x));
    const float ly = __fadd_rn(ty.lo, __fsub_rn(lo.y, lj.y));
    const float lz = __fadd_rn(tz.lo, __fsub_rn(lo.z, lj.z));
    const float px = __fmul_rn(tx.hi, tx.hi), py = __fmul_rn(ty.hi, ty.hi), pz = __fmul_rn(tz.hi, tz.hi);
    const float ex = __fmaf_rn(tx.hi, tx.hi, -px), ey = __fmaf_rn(ty.hi, ty.hi, -py), ez = __fmaf_rn(tz.hi, tz.hi, -pz);
    const float cx = lx * (2.0f * tx.hi + lx), cy = ly * (2.0f * ty.hi + ly), cz = lz * (2.0f * tz.hi + lz);
    const ff s1 = two_sum(px, py);
    const ff s2 = two_sum(s1.hi, pz);
    const float s3 = __fsub_rn(s2.hi, fr_hi);
    const float rest = (s1.lo + s2.lo) + ((ex + ey) + ez) + ((cx + cy) + cz) - fr_lo;
    return SepFF{fm(tx.hi + lx, ty.hi + ly, tz.hi + lz), s3 + rest};
}

__device__ __forceinline__ void contact_item(const Params &P, const PairView &PV, const BondView &BV,
                                             const MixedExtra &M, ContactSmem &W, int q, int64_t row0, int64_t n,
                                             int64_t xs, int64_t bs) {
    const int own = W.cown[q];
    const int64_t io = row0 + own;
    const int64_t e = (int64_t)W.ck[q] * n + io;
    const int32_t j = W.cj[q];
    const uint32_t fl = W.cfl[q];
    const bool bonded = (fl & kBonded) != 0;
    int64_t base, stride;
    float2 *store;
    int32_t aos;
    if (bonded) {
        base = (int64_t)bond_slot_of(fl) * n + io;
        stride = bs;
        store = reinterpret_cast<float2 *>(BV.xi);
        aos = BV.aos;
    } else {
        base = e;
        stride = xs;
        store = reinterpret_cast<float2 *>(PV.xi);
        aos = PV.aos;
    }
    // every load the pair may need is issued before any arithmetic (one memory round trip): the
    // partner's low position part, velocities and spin, and the springs of a live slot or bond
    const float4 lj = M.x32[2 * j + 1], vhj = M.v32[j], vlj = M.v32[n + j], wj4 = M.v32[2 * n + j];
    ff s[3][3] = {};  // springs of a slot that is not live are zero
    if (bonded || (fl & kXiLive))
#pragma unroll
        for (int c = 0; c < 9; ++c) {
            const float2 v = store[spring_at(aos, c, base, stride)];
            s[c / 3][c % 3] = ff{v.x, v.y};
        }
    const SepFF sp = separation_ff(W.xh[own], W.xl[own], W.chj[q], lj, bonded ? M.b_fr_hi : M.c_fr_hi,
                                   bonded ? M.b_fr_lo : M.c_fr_lo);
    const f3 dxf = sp.d;
    const float d2f = fdot(dxf, dxf);
    const float rr = bonded ? M.b_r : M.c_r;
    const float rsd = rsqrtf(d2f);
    const float overlap = -sp.q / (d2f * rsd + 2.0f * rr);  // 2r - |d|, from |d|^2 - (2r)^2
    bool touching = bonded || overlap > 0.0f;
    // spheres at the contact distance to within rounding (a seeded aggregate places touching
    // monomers there): the FP64 path's overlap decides whether they touch
    if (!bonded && M.x64 && fabsf(sp.q) <= M.q_marg) touching = overlap_fp64(M.x64, io, j, (double)P.contact.r_part) > 0.0;
    f3 force = fm(0.f, 0.f, 0.f), torque = fm(0.f, 0.f, 0.f);
    if (touching) {
        const f3 n3 = fscl(rsd, dxf);
        // relative velocity v_i - v_j from the float-float copies (exact high-part difference)
        const float4 vhi = W.vh[own], vlo = W.vl[own];
        const ff tx = two_sum(vhi.x, -vhj.x), ty = two_sum(vhi.y, -vhj.y), tz = two_sum(vhi.z, -vhj.z);
        const f3 vij0 = fm(tx.hi + (tx.lo + (vlo.x - vlj.x)), ty.hi + (ty.lo + (vlo.y - vlj.y)),
                           tz.hi + (tz.lo + (vlo.z - vlj.z)));
        const float4 wo4 = W.wh[own];
        const f3 wfi = fm(wo4.x, wo4.y, wo4.z), wfj = fm(wj4.x, wj4.y, wj4.z);
        const float kn = bonded ? M.b_k : M.c_k, gn = bonded ? M.b_gn : M.c_gn;
        const float rp = rr - 0.5f * overlap;
        const float v_n = -fdot(vij0, n3);
        const float f_n = kn * overlap + gn * v_n;
        const f3 nwi = fcrs(n3, wfi), nwj = fcrs(n3, wfj);
        const f3 v_ij = fadd(vij0, fscl(rp, fadd(nwi, nwj)));
        const f3 v_t = fsub(v_ij, fscl(fdot(v_ij, n3), n3));
        const f3 v_r = fscl(-rp, fsub(nwi, nwj));
        const f3 v_o = fscl(rr * (fdot(n3, wfi) - fdot(n3, wfj)), n3);
        f3 f_t, f_r, f_o;
        if (bonded) {
            f_t = shear_ff(s[0], n3, M.b_kt, M.b_gt, f_n, 0.f, 0.f, v_t, M.b_dt, false);
            f_r = shear_ff(s[1], n3, M.b_kr, M.b_gr, f_n, 0.f, 0.f, v_r, M.b_dt, false);
            f_o = shear_ff(s[2], n3, M.b_ko, M.b_go, f_n, 0.f, 0.f, v_o, M.b_dt, false);
        } else {
            f_t = shear_ff(s[0], n3, M.c_kt, M.c_gt, f_n, M.c_mus, M.c_phid, v_t, M.c_dt, true);
            f_r = shear_ff(s[1], n3, M.c_kr, M.c_gr, f_n, M.c_mur, M.c_phir, v_r, M.c_dt, true);
            f_o = shear_ff(s[2], n3, M.c_ko, M.c_go, f_n, M.c_muo, M.c_phio, v_o, M.c_dt, true);
        }
#pragma unroll
        for (int c = 0; c < 9; ++c)
            store[spring_at(aos, c, base, stride)] = make_float2(s[c / 3][c % 3].hi, s[c / 3][c % 3].lo);
        force = fadd(fscl(f_n, n3), f_t);
        torque = fadd(fsub(fscl(rr, fcrs(n3, f_r)), fscl(rp, fcrs(n3, f_t))), fscl(rr, f_o));
        if (bonded) {
            if (P.binary_model == LG_BINARY_BREAKING_SINTER) {
                const float st = (float)BV.strength[base];
                if (fdot(force, force) > st * st) {
                    BV.intact[base] = 0;
                    PV.flags[e] = fl & ~(kBonded | (0xffu << 8));
                }
            }
        } else if (!(fl & kXiLive)) {
            PV.flags[e] = fl | kXiLive;
        }
    } else if (fl & kXiLive) {
#pragma unroll
        for (int c = 0; c < 9; ++c) PV.xi[spring_at(PV.aos, c, e, xs)] = 0.0;
        PV.flags[e] = fl & ~kXiLive;
    }
    W.cres[q][0] = force.x * M.bin_im;
    W.cres[q][1] = force.y * M.bin_im;
    W.cres[q][2] = force.z * M.bin_im;
    W.cres[q][3] = torque.x * M.bin_iI;
    W.cres[q][4] = torque.y * M.bin_iI;
    W.cres[q][5] = torque.z * M.bin_iI;
}

// One queued Hamaker pair (hamaker_force.h:28-44; limited form hamaker_force.h:86-93): partner
// position from the queue, owner position from the warp's row data.
__device__ __forceinline__ void hamaker_item(const Params &P, const MixedExtra &M, HamakerSmem &W, int q) {
    const float4 ph = W.hhi[q];
    const int own = __float_as_int(ph.w);
    const SepFF sp = separation_ff(W.xh[own], W.xl[own], ph, W.hlo[q], M.h_fr_hi, M.h_fr_lo);
    f3 a = fm(0.f, 0.f, 0.f);
    if (!(P.hamaker_model == LG_HAMAKER_LIMITED && sp.q > M.h_qcut)) {
        const f3 dxf = sp.d;
        const float d2f = fdot(dxf, dxf);
        const float rsd = rsqrtf(d2f);
        float h = sp.q / (d2f * rsd + 2.0f * M.h_r);  // |d| - 2r to FP32 precision
        h = fmaxf(h, M.h_h0);
        const float sfac = ham_factor(P.hamaker_model, M.h_A, M.h_r, h) * M.inv_mass_h * rsd;
        a = fscl(-sfac, dxf);  // along x_j - x_i
    }
    W.hres[q][0] = a.x;
    W.hres[q][1] = a.y;
    W.hres[q][2] = a.z;
}


// Float-float sum and product (the product's rounding error from an FMA; results renormalised).
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    const ff s = two_sum(a.hi, b.hi);
    return two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const float p = __fmul_rn(a.hi, b.hi);
    const float e = __fmaf_rn(a.hi, b.hi, -p);
    return two_sum(p, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e)));
}
__device__ __forceinline__ double ff_to_d(ff a) { return (double)a.hi + (double)a.lo; }


// Contact and bond pairs of rows row0 .. row0 + 32/T - 1 (one warp): T lanes per row, lane t of a
// row taking its entries t, t + T, ... (so short candidate lists still fill the warp); each lane folds
// its pairs in entry order and the row's T partial sums are combined in lane order. csum receives the
// contact part of the row's accelerations as float-float pairs.
template <bool NEAR, int T>
__device__ __forceinline__ void contact_rows(const Params &P, const PairView &PV, const BondView &BV,
                                             const MixedExtra &MX, ContactSmem &W, int64_t row0, int lane) {
    const int r = lane / T, sub = lane % T;  // local row and sub-lane
    const int64_t n = P.n;
    const int64_t i = row0 + r;
    const bool active = i < n;
    const uint32_t lt = (1u << lane) - 1u;
    int64_t len = 0;
    float4 hi_i = make_float4(0.f, 0.f, 0.f, 0.f);
    if (active) {
        len = NEAR ? (int64_t)PV.near_len[i] : n - 1;
        hi_i = MX.x32[2 * i];
    }
    if (sub == 0) {
        const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
        W.xh[r] = hi_i;
        W.xl[r] = active ? MX.x32[2 * i + 1] : z4;
        W.vh[r] = active ? MX.v32[i] : z4;
        W.vl[r] = active ? MX.v32[n + i] : z4;
        W.wh[r] = active ? MX.v32[2 * n + i] : z4;
    }
    // iterations: the lane's entries sub, sub + T, ... below len
    const int64_t my_it = len > sub ? (len - sub + T - 1) / T : 0;
    const int64_t itmax = (int64_t)__reduce_max_sync(0xffffffffu, (unsigned)my_it);
    const int64_t xs = PV.cap * n;
    const int64_t bs = (int64_t)BV.bcap * n;
    ff acc[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}}, accw[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    __syncwarp();

    // entry of iteration it: partner and slot (-1: none); loaded two iterations ahead, and its flags
    // and partner position one iteration ahead of its classification
    int32_t jn = -1, kn = 0;
    auto load_entry = [&](int64_t it) {
        const int64_t m = it * T + sub;
        jn = -1;
        if (m < len) {
            if (NEAR) {
                jn = PV.near_j[m * n + i];
                kn = PV.near_k[m * n + i];
            } else {
                kn = (int32_t)m;
                jn = (int32_t)(m < i ? m : m + 1);
            }
        }
    };
    int32_t jc = -1, kc = 0;  // the entry being classified, with its flags and partner position
    uint32_t flc = 0;
    float4 pjc = hi_i;
    auto take_entry = [&]() {  // the loaded entry becomes the current one; its data is requested
        jc = jn;
        kc = kn;
        flc = 0;
        pjc = hi_i;
        if (jc >= 0) {
            flc = PV.flags[(int64_t)kc * n + i];
            pjc = MX.x32[2 * jc];
        }
    };
    if (itmax > 0) {
        load_entry(0);
        take_entry();
        if (itmax > 1) load_entry(1);
    }
    for (int64_t it0 = 0; it0 < itmax;) {
        int ccount = 0, cdone = 0;
        int64_t it = it0;
        for (;;) {
            const bool take = it < itmax && it - it0 < kCRound && ccount + 32 <= kCQ;
            if (take) {
                const int32_t j = jc, k = kc;
                const uint32_t fl = flc;
                const float4 pj = pjc;
                if (it + 1 < itmax) {
                    take_entry();
                    if (it + 2 < itmax) load_entry(it + 2);
                }
                bool cb = false;
                if (j >= 0) {
                    const float dx = hi_i.x - pj.x, dy = hi_i.y - pj.y, dz = hi_i.z - pj.z;
                    if ((fl & kBonded) || fmaf(dz, dz, fmaf(dy, dy, dx * dx)) <= MX.contact2f) {
                        cb = true;
                    } else if (fl & kXiLive) {  // reset_springs (contact_force.h:69,99-101)
                        const int64_t e = (int64_t)k * n + i;
#pragma unroll
                        for (int c = 0; c < 9; ++c) PV.xi[spring_at(PV.aos, c, e, xs)] = 0.0;
                        PV.flags[e] = fl & ~kXiLive;
                    }
                }
                const uint32_t bc = __ballot_sync(0xffffffffu, cb);
                if (cb) {
                    const int q = ccount + __popc(bc & lt);
                    W.cj[q] = j;
                    W.ck[q] = k;
                    W.cfl[q] = fl;
                    W.chj[q] = pj;
                    W.cown[q] = (uint8_t)r;
                }
                if (lane == 0) {
                    W.cball[it - it0] = bc;
                    W.cbase[it - it0] = ccount;
                }
                ccount += __popc(bc);
                ++it;
            }
            __syncwarp();
            // full batches of 32 while the round is open, the rest when it closes
            while (ccount - cdone >= 32 || (!take && cdone < ccount)) {
                if (cdone + lane < ccount) contact_item(P, PV, BV, MX, W, cdone + lane, row0, n, xs, bs);
                cdone += 32;
                __syncwarp();
            }
            if (!take) break;
        }
        // the round's pairs, in entry order
        for (int off = 0; off < (int)(it - it0); ++off) {
            const uint32_t bc = W.cball[off];
            if ((bc >> lane) & 1u) {
                const int q = W.cbase[off] + __popc(bc & lt);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    ff_acc(acc[c], W.cres[q][c]);
                    ff_acc(accw[c], W.cres[q][3 + c]);
                }
            }
        }
        __syncwarp();
        it0 = it;
    }
    if (T > 1) {  // the row's partial sums, in lane order, onto its first lane
        const int base = lane - sub;
#pragma unroll
        for (int t = 1; t < T; ++t) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float ah = __shfl_sync(0xffffffffu, acc[c].hi, base + t);
                const float al = __shfl_sync(0xffffffffu, acc[c].lo, base + t);
                const float wh = __shfl_sync(0xffffffffu, accw[c].hi, base + t);
                const float wl = __shfl_sync(0xffffffffu, accw[c].lo, base + t);
                if (sub == 0) {
                    ff_acc(acc[c], ah);
                    ff_acc(acc[c], al);
                    ff_acc(accw[c], wh);
                    ff_acc(accw[c], wl);
                }
            }
        }
    }
    if (!active || sub != 0) return;
    MX.csum[3 * i] = make_float4(acc[0].hi, acc[0].lo, acc[1].hi, acc[1].lo);
    MX.csum[3 * i + 1] = make_float4(acc[2].hi, acc[2].lo, accw[0].hi, accw[0].lo);
    MX.csum[3 * i + 2] = make_float4(accw[1].hi, accw[1].lo, accw[2].hi, accw[2].lo);
}

// Virtual slot v of slice sl of kSlices (its windows sl, sl + kSlices, ...) -> slot of the row; the
// same mapping as compact::slot_of with the slice count known at run time.
__device__ __forceinline__ int64_t slot_at(int64_t v, int sl, int kSlices) {
    return ((v / kWin) * kSlices + sl) * kWin + (v % kWin);
}

// Hamaker pairs of rows row0 .. row0 + 31 (one warp), slice sl of kSlices: the windows sl,
// sl + kSlices, ... of every row. acch receives the lane's row's partial sum (float-float).
template <bool VERLET>
__device__ __forceinline__ void hamaker_rows(const Params &P, const PairView &PV, const MixedExtra &MX,
                                             HamakerSmem &W, int64_t row0, int sl, int kSlices, int lane,
                                             ff (&acch)[3]) {
    const int64_t n = P.n;
    const int64_t i = row0 + lane;
    const bool active = i < n;
    const int hm = P.hamaker_model;
    const uint32_t lt = (1u << lane) - 1u;

    int64_t len = 0;
    float4 hi_i = make_float4(0.f, 0.f, 0.f, 0.f);
    {
        float4 lo_i = hi_i;
        if (active) {
            len = VERLET ? (int64_t)PV.row_len[i] : n - 1;
            hi_i = MX.x32[2 * i];
            lo_i = MX.x32[2 * i + 1];
        }
        W.xh[lane] = hi_i;
        W.xl[lane] = lo_i;
    }
    const int64_t maxlen = (int64_t)__reduce_max_sync(0xffffffffu, (unsigned)len);
    // this warp's windows: sl, sl + kSlices, ...; virtual slot v maps to slot_at(v, sl, kSlices)
    const int64_t nwin = (maxlen + kWin - 1) / kWin;
    const int64_t mywin = nwin > sl ? (nwin - sl + kSlices - 1) / kSlices : 0;
    const int64_t vmax = mywin * kWin;
    acch[0] = acch[1] = acch[2] = ff{0.f, 0.f};
    __syncwarp();

    // partners of the lane's row in the window at virtual slot v (-1: past the row's end)
    int32_t jn[kWin];
    auto load_window = [&](int64_t v) {
        const int64_t k0 = slot_at(v, sl, kSlices);
#pragma unroll
        for (int u = 0; u < kWin; ++u) {
            const int64_t kk = k0 + u;
            jn[u] = -1;
            if (kk < len) jn[u] = VERLET ? PV.nbr[kk * n + i] : (int32_t)(kk < i ? kk : kk + 1);
        }
    };
    if (vmax > 0) load_window(0);

    for (int64_t k = 0; k < vmax; k += kWin) {
        int32_t jg[kWin];
        float4 ph[kWin], pl[kWin];
#pragma unroll
        for (int u = 0; u < kWin; ++u) jg[u] = jn[u];
#pragma unroll
        for (int u = 0; u < kWin; ++u) {
            ph[u] = hi_i;
            pl[u] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (jg[u] >= 0) {
                ph[u] = MX.x32[2 * jg[u]];
                pl[u] = MX.x32[2 * jg[u] + 1];
            }
        }
        if (k + kWin < vmax) load_window(k + kWin);  // next window, in flight during this one
        int hcount = 0;
        uint32_t hbal[kWin];
        int hbas[kWin];
#pragma unroll
        for (int u = 0; u < kWin; ++u) {
            bool hb = false;
            if (jg[u] >= 0) {
                if (hm == LG_HAMAKER_LIMITED) {
                    const float dx = hi_i.x - ph[u].x, dy = hi_i.y - ph[u].y, dz = hi_i.z - ph[u].z;
                    hb = fmaf(dz, dz, fmaf(dy, dy, dx * dx)) <= MX.near2;
                } else {
                    hb = true;
                }
            }
            const uint32_t bh = __ballot_sync(0xffffffffu, hb);
            if (hb) {
                const int q = hcount + __popc(bh & lt);
                W.hhi[q] = make_float4(ph[u].x, ph[u].y, ph[u].z, __int_as_float(lane));
                W.hlo[q] = pl[u];
            }
            hbal[u] = bh;
            hbas[u] = hcount;
            hcount += __popc(bh);
        }
        __syncwarp();
        for (int q = lane; q < hcount; q += 32) hamaker_item(P, MX, W, q);
        __syncwarp();
        {  // the window's (at most four) terms in slot order, then one compensated add
            float wsum[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int u = 0; u < kWin; ++u)
                if ((hbal[u] >> lane) & 1u) {
                    const int q = hbas[u] + __popc(hbal[u] & lt);
#pragma unroll
                    for (int c = 0; c < 3; ++c) wsum[c] += W.hres[q][c];
                }
#pragma unroll
            for (int c = 0; c < 3; ++c) ff_acc(acch[c], wsum[c]);
        }
        __syncwarp();  // the next window reuses the queue
    }

}

// The completion of a step of a run for a particle that no step handler holds (the body of
// forces_finish_ff below): a, al are the row's float-float accelerations (contact + Hamaker). The
// float-float state is read from MX (x32, v32, s32) and the next step's positions and velocities are
// written to x32o / v32o (MX.x32 / MX.v32 themselves, or the other buffers of a double-buffered
// state); every load of the row precedes its stores.
template <bool LAST>
__device__ __forceinline__ void finish_ff_plain(const StateView &S, int64_t i, int64_t n, ff (&a)[3], const ff (&al)[3],
                                                ff hdt, ff dt, const MixedExtra &MX, float4 *x32o, float4 *v32o) {
    const float4 vh = MX.v32[i], vl = MX.v32[n + i], wh = MX.v32[2 * n + i], wl = MX.s32[i];
    const float4 dh = MX.s32[n + i], dl = MX.s32[2 * n + i], rh = MX.s32[3 * n + i], rl = MX.s32[4 * n + i];
    bool finite = true;
#pragma unroll
    for (int c = 0; c < 3; ++c) finite = finite && isfinite(a[c].hi) && isfinite(al[c].hi);
    if (!finite) set_error(S.err, LG_DEVERR_NONFINITE);
    ff v[3] = {{vh.x, vl.x}, {vh.y, vl.y}, {vh.z, vl.z}};
    ff w[3] = {{wh.x, wl.x}, {wh.y, wl.y}, {wh.z, wl.z}};
    ff dx[3] = {{dh.x, dl.x}, {dh.y, dl.y}, {dh.z, dl.z}};
    ff dr[3] = {{rh.x, rl.x}, {rh.y, rl.y}, {rh.z, rl.z}};
    // end-of-step half kick
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        v[c] = ff_add(v[c], ff_mul(hdt, a[c]));
        w[c] = ff_add(w[c], ff_mul(hdt, al[c]));
    }
    if (LAST) {
        const d3 x0 = ld4(S.x, i), t0 = ld4(S.th, i);
        st4(S.a, i, mk3(ff_to_d(a[0]), ff_to_d(a[1]), ff_to_d(a[2])));
        st4(S.al, i, mk3(ff_to_d(al[0]), ff_to_d(al[1]), ff_to_d(al[2])));
        st4(S.v_out, i, mk3(ff_to_d(v[0]), ff_to_d(v[1]), ff_to_d(v[2])));
        st4(S.w_out, i, mk3(ff_to_d(w[0]), ff_to_d(w[1]), ff_to_d(w[2])));
        st4(S.x, i, mk3(x0.x + ff_to_d(dx[0]), x0.y + ff_to_d(dx[1]), x0.z + ff_to_d(dx[2])));
        st4(S.th, i, mk3(t0.x + ff_to_d(dr[0]), t0.y + ff_to_d(dr[1]), t0.z + ff_to_d(dr[2])));
        return;
    }
    // the next step's opening half kick and drift
    const float4 xh = MX.x32[2 * i], xl = MX.x32[2 * i + 1];  // loaded before anything is stored
    ff x[3] = {{xh.x, xl.x}, {xh.y, xl.y}, {xh.z, xl.z}};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        v[c] = ff_add(v[c], ff_mul(hdt, a[c]));
        w[c] = ff_add(w[c], ff_mul(hdt, al[c]));
        const ff step = ff_mul(dt, v[c]);
        x[c] = ff_add(x[c], step);
        dx[c] = ff_add(dx[c], step);
        dr[c] = ff_add(dr[c], ff_mul(dt, w[c]));
    }
    x32o[2 * i] = make_float4(x[0].hi, x[1].hi, x[2].hi, 0.f);
    x32o[2 * i + 1] = make_float4(x[0].lo, x[1].lo, x[2].lo, 0.f);
    v32o[i] = make_float4(v[0].hi, v[1].hi, v[2].hi, 0.f);
    v32o[n + i] = make_float4(v[0].lo, v[1].lo, v[2].lo, 0.f);
    v32o[2 * n + i] = make_float4(w[0].hi, w[1].hi, w[2].hi, 0.f);
    MX.s32[i] = make_float4(w[0].lo, w[1].lo, w[2].lo, 0.f);
    MX.s32[n + i] = make_float4(dx[0].hi, dx[1].hi, dx[2].hi, 0.f);
    MX.s32[2 * n + i] = make_float4(dx[0].lo, dx[1].lo, dx[2].lo, 0.f);
    MX.s32[3 * n + i] = make_float4(dr[0].hi, dr[1].hi, dr[2].hi, 0.f);
    MX.s32[4 * n + i] = make_float4(dr[0].lo, dr[1].lo, dr[2].lo, 0.f);
}

}  // namespace mixed
}  // namespace lg
