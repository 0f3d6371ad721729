// lg_forces_compact.cu -- warp-compacted force kernel (sm_103a), FP64 and mixed precision.
//
// On GB300 a warp instruction on the FP64 pipe costs the same issue time whether 1 or 32 lanes are
// active, so a kernel whose lanes each walk their own row and branch on "is this pair in Hamaker
// range / in contact" wastes most of its FP64 issue slots. This kernel gives each lane one row (one
// particle i) and processes the rows of a warp in rounds of up to kRound slots:
//   A. classify  -- every lane tests its slot k (separation against the cutoffs); the warp appends
//                   contact/bond candidates to a shared-memory queue in a fixed order (slot-major,
//                   lane-minor, via ballots) and records which slots need a Hamaker evaluation.
//                   As soon as 32 contact items are pending, all 32 lanes evaluate them, one pair
//                   per lane (springs read and written in global memory: each slot belongs to
//                   exactly one item), so the expensive contact code runs with full warps;
//   B. Hamaker   -- per window of kWin slots, the warp queues that window's Hamaker pairs and all
//                   32 lanes evaluate them, one pair per lane;
//      fold      -- each lane adds its row's results in ascending slot order, exactly as the
//                   reference's loop adds (contact + Hamaker) pair by pair.
// Per-pair results live only in shared memory, so the per-particle sums come out in a fixed order
// with no floating-point atomics. In FP64 (this file compiled with --fmad=false) every pair value
// is computed by the same functions as the sequential kernel and the fold adds in the same order,
// so the result is bit-identical to the sequential evaluation.
//
// Compiled twice: LG_COMPACT_MIXED=0 (FP64) and LG_COMPACT_MIXED=1. The mixed build keeps the FP64
// pipe for the contact/bond items only (FP64 separation, overlap and springs, as in
// lg_forces_mixed.cu): every Hamaker pair takes its separation and |d|^2 - (2r)^2 from float-float
// positions with error-free FP32 transformations, and the per-row sums are float-float
// (compensated) FP32 accumulations, converted to FP64 once per row.
#include "lg_common.cuh"
#include "lg_kernels.h"

#ifndef LG_COMPACT_MIXED
#define LG_COMPACT_MIXED 0
#endif

namespace lg {

namespace {

constexpr int kWin = 4;            // Hamaker window (slots)
constexpr int kGroup = 4;          // slots classified per memory round trip
constexpr int kHCap = 32 * kWin;   // Hamaker queue capacity per window
// Slicing: the slots of a 32-row group may be split over SL warps (window w of a row goes to warp
// w % SL), which gives the GPU SL times as many warps to hide latency with when a launch has few
// rows; each warp's per-row partial sums are then combined in warp order at the end. The FP64
// kernel always uses SL = 1, so every row is added in ascending slot order.
template <int SL>
struct Shape {
    static constexpr int kSlices = SL;
    static constexpr int kRowWarps = SL == 1 ? 2 : 1;
    static constexpr int kRound = SL == 1 ? 128 : 64;  // slots classified per round (per warp)
    static constexpr int kCCap = SL == 1 ? 256 : 160;  // contact queue capacity per round
    static constexpr int kWarps = kSlices * kRowWarps;
};
#if LG_COMPACT_MIXED
typedef float rt;
#else
typedef double rt;
#endif

// Virtual slot v of slice sl (its windows sl, sl + SL, ...) -> slot of the row.
template <int SL>
__device__ __forceinline__ int64_t slot_of(int64_t v, int sl) {
    return ((v / kWin) * SL + sl) * kWin + (v % kWin);
}

template <int SL>
struct WarpSmem {
    static constexpr int kCCap = Shape<SL>::kCCap, kRound = Shape<SL>::kRound;
    rt hres[kHCap][3];
    rt cres[kCCap][6];
    int32_t hj[kHCap], cj[kCCap];
    uint16_t hown[kHCap], cown[kCCap];  // (owner lane << 8) | slot offset within the round
    uint32_t cball[kRound], hballA[kRound];
    int32_t cbase[kRound];
    uint32_t hball[kWin];
    int32_t hbase[kWin];
    d3 xo[32], vo[32], wo[32];
#if LG_COMPACT_MIXED
    float4 xh[32], xl[32];  // own position as float-float (high, low parts)
#endif
};

#if LG_COMPACT_MIXED
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

// Shear spring (contact_force.h:105-147, Coulomb-capped; alt_sinter_bridge.h:137-156, bond form)
// with the spring vector held in FP64. Each evaluation computes, in FP32, the increment of the
// spring: the rotation onto the tangent plane, -(xi.n) n, the rescale to the old magnitude,
// (s - 1)(xi - (xi.n) n) with s - 1 evaluated as a series for small tilts, and the stretch rel*dt;
// the increment is small next to xi and is added to the FP64 spring, so rounding does not
// accumulate at the spring's own scale. The dynamic (sliding) branch sets the spring outright.
__device__ __forceinline__ f3 shear_mx(d3 &xi, f3 n, float stiffness, float damping, float normal_force, float mu_s,
                                       float phi, f3 rel, float dtf, bool coulomb) {
    f3 xf = tof(xi);
    f3 drot = fm(0.f, 0.f, 0.f);
    float xx = fdot(xf, xf);
    if (xx > 0.0f) {
        float c = fdot(xf, n);
        f3 xr = fsub(xf, fscl(c, n));
        float e = (c * c) / xx;
        float sm1 = 0.0f;
        if (e < 1.0f) sm1 = e < 1e-3f ? e * (0.5f + 0.375f * e) : rsqrtf(1.0f - e) - 1.0f;
        drot = fadd(fscl(-c, n), fscl(sm1, xr));
    }
    const f3 xn = fadd(xf, drot);
    const f3 f0 = fsub(fscl(-stiffness, xn), fscl(damping, rel));
    if (!coulomb) {
        const f3 dxi = fadd(drot, fscl(dtf, rel));
        xi.x += (double)dxi.x;
        xi.y += (double)dxi.y;
        xi.z += (double)dxi.z;
        return f0;
    }
    const float fs = mu_s * normal_force;
    const float fd = mu_s * phi * normal_force;
    const float f0n = sqrtf(fdot(f0, f0));
    const f3 t = f0n > 0.0f ? fscl(1.0f / f0n, f0) : fm(0.f, 0.f, 0.f);
    float sel;
    if (f0n <= fs) {
        const f3 dxi = fadd(drot, fscl(dtf, rel));
        xi.x += (double)dxi.x;
        xi.y += (double)dxi.y;
        xi.z += (double)dxi.z;
        sel = fs;
    } else {
        const f3 nx = fscl(-1.0f / stiffness, fadd(fscl(fd, t), fscl(damping, rel)));
        xi = mk3((double)nx.x, (double)nx.y, (double)nx.z);
        sel = fd;
    }
    return fscl(fminf(sel, f0n), t);
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
__device__ __forceinline__ void ff_acc(ff &a, ff b) {
    const ff s = two_sum(a.hi, b.hi);
    a.hi = s.hi;
    a.lo = __fadd_rn(a.lo, __fadd_rn(s.lo, b.lo));
}
__device__ __forceinline__ double ff_to_d(ff a) { return (double)a.hi + (double)a.lo; }

// Separation d = x_i - x_j (FP32) and q = |d|^2 - (2r)^2 from float-float positions. Per component
// the high parts' difference is split exactly (TwoSum) and its error joins the low parts'
// difference, so dh + dl equals the separation to about 2^-48 of the coordinates. Then
// (dh + dl)^2 = dh^2 + dl (2 dh + dl), with dh^2 split exactly by FMA; the three large squares and
// -(2r)^2 (given as fr_hi + fr_lo) are added with TwoSum, so q comes out with FP32 relative
// precision however close |d| is to 2r.
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
    const ff s3 = two_sum(s2.hi, -fr_hi);
    const float rest = ((s1.lo + s2.lo) + s3.lo) + ((ex + ey) + ez) + ((cx + cy) + cz) - fr_lo;
    return SepFF{fm(tx.hi + lx, ty.hi + ly, tz.hi + lz), s3.hi + rest};
}
#endif

// One queued contact / bond pair: owner row io (lane own of the warp), slot e, partner j.
#if LG_COMPACT_MIXED
template <int SL>
__device__ __forceinline__ void contact_item(const Params &P, const StateView &S, const PairView &PV,
                                             const BondView &BV, const MixedExtra &M, WarpSmem<SL> &W, int q,
                                             int64_t row0, int64_t kstart, int sl, int64_t n, int64_t xs, int64_t bs) {
    const int own = W.cown[q] >> 8;
    const int64_t io = row0 + own;
    const int64_t e = slot_of<SL>(kstart + (W.cown[q] & 0xff), sl) * n + io;
    const int32_t j = W.cj[q];
    const uint32_t fl = PV.flags[e];
    const bool bonded = (fl & kBonded) != 0;
    const d3 vo = W.vo[own], wo = W.wo[own];
    const SepFF sp = separation_ff(W.xh[own], W.xl[own], M.x32[j], M.x32lo[j], bonded ? M.b_fr_hi : M.c_fr_hi,
                                   bonded ? M.b_fr_lo : M.c_fr_lo);
    const f3 dxf = sp.d;
    const float d2f = fdot(dxf, dxf);
    const float rr = bonded ? M.b_r : M.c_r;
    const float rsd = rsqrtf(d2f);
    const float overlap = -sp.q / (d2f * rsd + 2.0f * rr);  // 2r - |d|, from |d|^2 - (2r)^2
    f3 force = fm(0.f, 0.f, 0.f), torque = fm(0.f, 0.f, 0.f);
    if (bonded || overlap > 0.0f) {
        const f3 n3 = fscl(rsd, dxf);
        const d3 vj = ld4(S.v, j), wj = ld4(S.w, j);
        const f3 vij0 = tof(sub(vo, vj));
        const f3 wfi = tof(wo), wfj = tof(wj);
        int64_t base, stride;
        double *store;
        if (bonded) {
            base = (int64_t)bond_slot_of(fl) * n + io;
            stride = bs;
            store = BV.xi;
        } else {
            base = e;
            stride = xs;
            store = PV.xi;
        }
        d3 s[3] = {zero3(), zero3(), zero3()};  // springs of a slot that is not live are zero
        if (bonded || (fl & kXiLive))
#pragma unroll
            for (int c = 0; c < 3; ++c)
                s[c] = mk3(store[(3 * c) * stride + base], store[(3 * c + 1) * stride + base], store[(3 * c + 2) * stride + base]);
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
            f_t = shear_mx(s[0], n3, M.b_kt, M.b_gt, f_n, 0.f, 0.f, v_t, M.b_dt, false);
            f_r = shear_mx(s[1], n3, M.b_kr, M.b_gr, f_n, 0.f, 0.f, v_r, M.b_dt, false);
            f_o = shear_mx(s[2], n3, M.b_ko, M.b_go, f_n, 0.f, 0.f, v_o, M.b_dt, false);
        } else {
            f_t = shear_mx(s[0], n3, M.c_kt, M.c_gt, f_n, M.c_mus, M.c_phid, v_t, M.c_dt, true);
            f_r = shear_mx(s[1], n3, M.c_kr, M.c_gr, f_n, M.c_mur, M.c_phir, v_r, M.c_dt, true);
            f_o = shear_mx(s[2], n3, M.c_ko, M.c_go, f_n, M.c_muo, M.c_phio, v_o, M.c_dt, true);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            store[(3 * c) * stride + base] = s[c].x;
            store[(3 * c + 1) * stride + base] = s[c].y;
            store[(3 * c + 2) * stride + base] = s[c].z;
        }
        force = fadd(fscl(f_n, n3), f_t);
        torque = fadd(fsub(fscl(rr, fcrs(n3, f_r)), fscl(rp, fcrs(n3, f_t))), fscl(rr, f_o));
        if (bonded) {
            if (P.binary_model == LG_BINARY_BREAKING_SINTER) {
                const double st = BV.strength[base];
                if ((double)fdot(force, force) > st * st) {
                    BV.intact[base] = 0;
                    PV.flags[e] = fl & ~(kBonded | (0xffu << 8));
                }
            }
        } else if (!(fl & kXiLive)) {
            PV.flags[e] = fl | kXiLive;
        }
    } else if (fl & kXiLive) {
#pragma unroll
        for (int c = 0; c < 9; ++c) PV.xi[c * xs + e] = 0.0;
        PV.flags[e] = fl & ~kXiLive;
    }
    // accelerations: the binary functor's force and torque over its mass and moment of inertia
    W.cres[q][0] = force.x * M.bin_im;
    W.cres[q][1] = force.y * M.bin_im;
    W.cres[q][2] = force.z * M.bin_im;
    W.cres[q][3] = torque.x * M.bin_iI;
    W.cres[q][4] = torque.y * M.bin_iI;
    W.cres[q][5] = torque.z * M.bin_iI;
}

template <int SL>
__device__ __forceinline__ void hamaker_item(const Params &P, const StateView &S, const MixedExtra &M,
                                             WarpSmem<SL> &W, int q) {
    (void)S;
    const int own = W.hown[q] >> 8;
    const int32_t j = W.hj[q];
    const SepFF sp = separation_ff(W.xh[own], W.xl[own], M.x32[j], M.x32lo[j], M.h_fr_hi, M.h_fr_lo);
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
#else
template <int SL>
__device__ __forceinline__ void contact_item(const Params &P, const StateView &S, const PairView &PV,
                                             const BondView &BV, WarpSmem<SL> &W, int q, int64_t row0, int64_t kstart,
                                             int sl, int64_t n, int64_t xs, int64_t bs) {
    const int own = W.cown[q] >> 8;
    const int64_t io = row0 + own;
    const int64_t e = slot_of<SL>(kstart + (W.cown[q] & 0xff), sl) * n + io;
    const int32_t j = W.cj[q];
    const uint32_t fl = PV.flags[e];
    const d3 xo = W.xo[own], vo = W.vo[own], wo = W.wo[own];
    const d3 dx = sub(xo, ld4(S.x, j));
    d3 pa = zero3(), pal = zero3();
    if (fl & kBonded) {
        const bool breaking = P.binary_model == LG_BINARY_BREAKING_SINTER;
        const int64_t be = (int64_t)bond_slot_of(fl) * n + io;
        d3 s[3];
#pragma unroll
        for (int c = 0; c < 3; ++c)
            s[c] = mk3(BV.xi[(3 * c) * bs + be], BV.xi[(3 * c + 1) * bs + be], BV.xi[(3 * c + 2) * bs + be]);
        const d3 vj = ld4(S.v, j), wj = ld4(S.w, j);
        const bool brk = bond_force(P.sinter, dx, vo, vj, wo, wj, s, breaking, breaking ? BV.strength[be] : 0.0, pa, pal);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            BV.xi[(3 * c) * bs + be] = s[c].x;
            BV.xi[(3 * c + 1) * bs + be] = s[c].y;
            BV.xi[(3 * c + 2) * bs + be] = s[c].z;
        }
        if (brk) {
            BV.intact[be] = 0;
            PV.flags[e] = fl & ~(kBonded | (0xffu << 8));
        }
    } else {
        const d3 nn = nrmz(dx);
        const double overlap = 2.0 * P.contact.r_part - dot(dx, nn);
        if (!(overlap <= 0)) {
            d3 s[3] = {zero3(), zero3(), zero3()};  // springs of a slot that is not live are zero
            if (fl & kXiLive)
#pragma unroll
                for (int c = 0; c < 3; ++c)
                    s[c] = mk3(PV.xi[(3 * c) * xs + e], PV.xi[(3 * c + 1) * xs + e], PV.xi[(3 * c + 2) * xs + e]);
            const d3 vj = ld4(S.v, j), wj = ld4(S.w, j);
            contact_touching(P.contact, nn, overlap, vo, vj, wo, wj, s, pa, pal);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                PV.xi[(3 * c) * xs + e] = s[c].x;
                PV.xi[(3 * c + 1) * xs + e] = s[c].y;
                PV.xi[(3 * c + 2) * xs + e] = s[c].z;
            }
            if (!(fl & kXiLive)) PV.flags[e] = fl | kXiLive;
        } else if (fl & kXiLive) {  // reset_springs (contact_force.h:69,99-101)
#pragma unroll
            for (int c = 0; c < 9; ++c) PV.xi[c * xs + e] = 0.0;
            PV.flags[e] = fl & ~kXiLive;
        }
    }
    W.cres[q][0] = pa.x;
    W.cres[q][1] = pa.y;
    W.cres[q][2] = pa.z;
    W.cres[q][3] = pal.x;
    W.cres[q][4] = pal.y;
    W.cres[q][5] = pal.z;
}

template <int SL>
__device__ __forceinline__ void hamaker_item(const Params &P, const StateView &S, WarpSmem<SL> &W, int q) {
    const int own = W.hown[q] >> 8;
    const d3 xo = W.xo[own];
    const d3 xj = ld4(S.x, W.hj[q]);
    d3 ha = zero3();
    // |x_i - x_j| and |x_j - x_i| are the same value (the squares of negated differences are
    // identical), so one square root serves the cutoff test, h and the unit vector
    const d3 r = sub(xj, xo);
    const double rn = nrm(r);
    bool on = true;
    if (P.hamaker_model == LG_HAMAKER_LIMITED) on = !(rn > P.hamaker.r_cutoff);
    if (on) ha = hamaker_accel_n(P.hamaker_model, P.hamaker, r, rn);
    W.hres[q][0] = ha.x;
    W.hres[q][1] = ha.y;
    W.hres[q][2] = ha.z;
}
#endif

}  // namespace

template <bool VERLET, int SL>
__global__ void __launch_bounds__(Shape<SL>::kWarps * 32)
#if LG_COMPACT_MIXED
    forces_compact_mixed(Params P, StateView S, PairView PV, BondView BV, double hdt, double dt, int move_facets,
                         MixedExtra MX)
#else
    forces_compact_fp64(Params P, StateView S, PairView PV, BondView BV, double hdt, double dt, int move_facets)
#endif
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int kSlices = Shape<SL>::kSlices, kRowWarps = Shape<SL>::kRowWarps, kWarps = Shape<SL>::kWarps;
    constexpr int kRound = Shape<SL>::kRound, kCCap = Shape<SL>::kCCap;
    WarpSmem<SL> &W = reinterpret_cast<WarpSmem<SL> *>(smem_raw)[warp];
    const int rw = warp / kSlices, sl = warp % kSlices;  // row group of the block, slice of it
    const int64_t n = P.n;
    const int64_t row0 = ((int64_t)blockIdx.x * kRowWarps + rw) * 32;
    const int64_t i = row0 + lane;
    const bool active = i < n;
    const int bm = P.binary_model, hm = P.hamaker_model;
    const uint32_t lt = (1u << lane) - 1u;

    if (move_facets && blockIdx.x == 0 && threadIdx.x == 0) {
        for (int f = 0; f < P.n_facets; ++f)
            for (int q = 0; q < 9; ++q) S.facet_vert_next[9 * f + q] = S.facet_vert[9 * f + q] + P.facets[f].v[q % 3] * dt;
    }

    d3 xi_ = zero3(), vi = zero3(), wi = zero3();
    int64_t len = 0;
    if (active) {
        xi_ = ld4(S.x, i);
        vi = ld4(S.v, i);
        wi = ld4(S.w, i);
        len = VERLET ? (int64_t)PV.row_len[i] : n - 1;
    }
#if LG_COMPACT_MIXED
    const float4 q4i = active ? MX.x32[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    W.xh[lane] = q4i;
    W.xl[lane] = active ? MX.x32lo[i] : make_float4(0.f, 0.f, 0.f, 0.f);
#else
    W.xo[lane] = xi_;
#endif
    W.vo[lane] = vi;
    W.wo[lane] = wi;
    const int64_t maxlen = (int64_t)__reduce_max_sync(0xffffffffu, (unsigned)len);
    // this warp's slots: windows sl, sl + kSlices, ...; virtual slot v maps to slot_of(v)
    const int64_t nwin = (maxlen + kWin - 1) / kWin;
    const int64_t mywin = nwin > sl ? (nwin - sl + kSlices - 1) / kSlices : 0;
    const int64_t vmax = mywin * kWin;
    auto slot = [sl](int64_t v) -> int64_t { return slot_of<SL>(v, sl); };
    const int64_t xs = PV.cap * n;
    const int64_t bs = (int64_t)BV.bcap * n;
#if LG_COMPACT_MIXED
    ff acc[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}}, accw[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
#else
    d3 acc = zero3(), accw = zero3();
#endif
    __syncwarp();

    for (int64_t kstart = 0; kstart < vmax;) {
        // ---------------- pass A: classify, queue contacts, evaluate them in full warps ----------------
        int ccount = 0, cdone = 0;
        int64_t k = kstart;  // virtual slot index (the actual slot is slot_of(k))
        // slots are taken four at a time: their indices and neighbour positions are loaded together
        // (one memory round trip per group), then classified and queued slot by slot
        for (; k < vmax && k - kstart + kGroup <= kRound && ccount + 32 * kGroup <= kCCap; k += kGroup) {
            int32_t jg[kGroup];
            uint32_t fg[kGroup];
            const int64_t k0 = slot(k);  // kGroup == kWin: a group is one window of consecutive slots
#pragma unroll
            for (int u = 0; u < kGroup; ++u) {
                const int64_t kk = k0 + u;
                jg[u] = 0;
                fg[u] = 0;
                if (kk < len) {
                    const int64_t e = kk * n + i;
                    jg[u] = VERLET ? PV.nbr[e] : (int32_t)(kk < i ? kk : kk + 1);
                    fg[u] = PV.flags[e];
                }
            }
#if LG_COMPACT_MIXED
            float4 pg[kGroup];
#pragma unroll
            for (int u = 0; u < kGroup; ++u) pg[u] = (k0 + u < len) ? MX.x32[jg[u]] : q4i;
#else
            d3 pg[kGroup];
#pragma unroll
            for (int u = 0; u < kGroup; ++u) pg[u] = (k0 + u < len) ? ld4(S.x, jg[u]) : xi_;
#endif
#pragma unroll
            for (int u = 0; u < kGroup; ++u) {
                const int64_t kk = k0 + u;
                const int64_t vv = k + u;
                bool hb = false, cb = false;
                const int32_t j = jg[u];
                if (kk < len) {
                    const int64_t e = kk * n + i;
                    const uint32_t fl = fg[u];
                    const bool bonded = (fl & kBonded) && bm != LG_BINARY_NONE;
#if LG_COMPACT_MIXED
                    const float dxf = q4i.x - pg[u].x, dyf = q4i.y - pg[u].y, dzf = q4i.z - pg[u].z;
                    const float d2f = fmaf(dzf, dzf, fmaf(dyf, dyf, dxf * dxf));
                    const bool ccand = d2f <= MX.contact2f;
                    if (hm == LG_HAMAKER_LIMITED)
                        hb = d2f <= MX.near2;
                    else if (hm != LG_HAMAKER_NONE)
                        hb = true;
#else
                    const double d2 = sqn(sub(xi_, pg[u]));
                    const bool ccand = !(d2 > P.contact_skip_d2);
                    if (hm == LG_HAMAKER_LIMITED)
                        hb = !(d2 > P.hamaker_skip_d2);
                    else if (hm != LG_HAMAKER_NONE)
                        hb = true;
#endif
                    if (bm != LG_BINARY_NONE) {
                        if (bonded || ccand)
                            cb = true;
                        else if (fl & kXiLive) {  // reset_springs (contact_force.h:69,99-101)
#pragma unroll
                            for (int c = 0; c < 9; ++c) PV.xi[c * xs + e] = 0.0;
                            PV.flags[e] = fl & ~kXiLive;
                        }
                    }
                }
                const uint32_t bc = __ballot_sync(0xffffffffu, cb);
                const uint32_t bh = __ballot_sync(0xffffffffu, hb);
                if (cb) {
                    const int q = ccount + __popc(bc & lt);
                    W.cj[q] = j;
                    W.cown[q] = (uint16_t)((lane << 8) | (int)(vv - kstart));
                }
                if (lane == 0) {
                    W.cball[vv - kstart] = bc;
                    W.cbase[vv - kstart] = ccount;
                    W.hballA[vv - kstart] = bh;
                }
                ccount += __popc(bc);
            }
            __syncwarp();
            while (ccount - cdone >= 32) {
#if LG_COMPACT_MIXED
                contact_item<SL>(P, S, PV, BV, MX, W, cdone + lane, row0, kstart, sl, n, xs, bs);
#else
                contact_item<SL>(P, S, PV, BV, W, cdone + lane, row0, kstart, sl, n, xs, bs);
#endif
                cdone += 32;
                __syncwarp();
            }
        }
        const int64_t kend = k;
        if (cdone < ccount) {
            if (cdone + lane < ccount)
#if LG_COMPACT_MIXED
                contact_item<SL>(P, S, PV, BV, MX, W, cdone + lane, row0, kstart, sl, n, xs, bs);
#else
                contact_item<SL>(P, S, PV, BV, W, cdone + lane, row0, kstart, sl, n, xs, bs);
#endif
            cdone = ccount;
        }
        __syncwarp();

        // ---------------- pass B: Hamaker windows and the ordered fold ----------------
        for (int64_t vw = kstart; vw < kend; vw += kWin) {
            int hcount = 0;
            const int64_t kw = slot(vw);  // first slot of the window
#pragma unroll
            for (int t = 0; t < kWin; ++t) {
                const int64_t kk = kw + t;
                const uint32_t bh = vw + t < kend ? W.hballA[vw + t - kstart] : 0u;
                if ((bh >> lane) & 1u) {
                    const int q = hcount + __popc(bh & lt);
                    W.hj[q] = VERLET ? PV.nbr[kk * n + i] : (int32_t)(kk < i ? kk : kk + 1);
                    W.hown[q] = (uint16_t)((lane << 8) | t);
                }
                if (lane == 0) {
                    W.hball[t] = bh;
                    W.hbase[t] = hcount;
                }
                hcount += __popc(bh);
            }
            __syncwarp();
            for (int q = lane; q < hcount; q += 32)
#if LG_COMPACT_MIXED
                hamaker_item<SL>(P, S, MX, W, q);
#else
                hamaker_item<SL>(P, S, W, q);
#endif
            __syncwarp();
#pragma unroll
            for (int t = 0; t < kWin; ++t) {
                const int64_t kk = kw + t;
                if (vw + t < kend && kk < len) {
                    const uint32_t bh = W.hball[t], bc = W.cball[vw + t - kstart];
                    const bool hb = (bh >> lane) & 1u, cb = (bc >> lane) & 1u;
#if LG_COMPACT_MIXED
                    if (cb) {
                        const int q = W.cbase[vw + t - kstart] + __popc(bc & lt);
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            ff_acc(acc[c], W.cres[q][c]);
                            ff_acc(accw[c], W.cres[q][3 + c]);
                        }
                    }
                    if (hb) {
                        const int q = W.hbase[t] + __popc(bh & lt);
#pragma unroll
                        for (int c = 0; c < 3; ++c) ff_acc(acc[c], W.hres[q][c]);
                    }
#else
                    // the reference's fold: pa = binary(i, j) [+ hamaker(i, j)]; acc += pa. Pairs with no
                    // queued item contribute exact zeros, which leave the sums unchanged.
                    if (cb || hb) {
                        d3 pa = zero3(), pal = zero3();
                        bool have = false;
                        if (bm != LG_BINARY_NONE) {
                            have = true;
                            if (cb) {
                                const int q = W.cbase[vw + t - kstart] + __popc(bc & lt);
                                pa = mk3(W.cres[q][0], W.cres[q][1], W.cres[q][2]);
                                pal = mk3(W.cres[q][3], W.cres[q][4], W.cres[q][5]);
                            }
                        }
                        if (hm != LG_HAMAKER_NONE) {
                            d3 ha = zero3();
                            if (hb) {
                                const int q = W.hbase[t] + __popc(bh & lt);
                                ha = mk3(W.hres[q][0], W.hres[q][1], W.hres[q][2]);
                            }
                            if (have) {
                                pa = add(pa, ha);
                                pal = add(pal, zero3());
                            } else {
                                pa = ha;
                                pal = zero3();
                            }
                        }
                        acc = add(acc, pa);
                        accw = add(accw, pal);
                    }
#endif
                }
            }
            __syncwarp();
        }
        kstart = kend;
    }
#if LG_COMPACT_MIXED
    // combine the slices' partial sums of each row in slice order (fixed, deterministic)
    if (kSlices > 1) {
        ff *part = reinterpret_cast<ff *>(smem_raw + sizeof(WarpSmem<SL>) * kWarps);
        ff *mine = part + ((int64_t)(rw * kSlices + sl) * 32 + lane) * 6;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            mine[c] = acc[c];
            mine[3 + c] = accw[c];
        }
        __syncthreads();
        if (sl != 0) return;
        for (int q = 1; q < kSlices; ++q) {
            const ff *o = part + ((int64_t)(rw * kSlices + q) * 32 + lane) * 6;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                ff_acc(acc[c], o[c]);
                ff_acc(accw[c], o[3 + c]);
            }
        }
    }
#endif
    if (!active) return;

#if LG_COMPACT_MIXED
    d3 a_tot = mk3(ff_to_d(acc[0]), ff_to_d(acc[1]), ff_to_d(acc[2]));
    d3 al_tot = mk3(ff_to_d(accw[0]), ff_to_d(accw[1]), ff_to_d(accw[2]));
    d3 &accA = a_tot;
    d3 &accW = al_tot;
#else
    d3 &accA = acc;
    d3 &accW = accw;
#endif
    if (P.n_facets > 0) {
        d3 ua = zero3(), ual = zero3();
        for (int f = 0; f < P.n_facets; ++f) {
            const FacetDev &fd = P.facets[f];
            d3 N = mk3(fd.normal[0], fd.normal[1], fd.normal[2]);
            d3 xf = closest_point_on_triangle(S.facet_vert + 9 * f, fd.area, N, xi_);
            d3 vf = mk3(fd.v[0], fd.v[1], fd.v[2]);
            d3 fa = zero3(), fal = zero3();
            bool hv = false;
            if (fd.has_contact) {
                const int64_t base = (int64_t)f * 9 * n;
                d3 s[3];
#pragma unroll
                for (int q = 0; q < 3; ++q)
                    s[q] = mk3(S.sxi[base + (3 * q) * n + i], S.sxi[base + (3 * q + 1) * n + i], S.sxi[base + (3 * q + 2) * n + i]);
                surface_contact(fd.contact, xf, vf, xi_, vi, wi, s, fa, fal);
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    S.sxi[base + (3 * q) * n + i] = s[q].x;
                    S.sxi[base + (3 * q + 1) * n + i] = s[q].y;
                    S.sxi[base + (3 * q + 2) * n + i] = s[q].z;
                }
                hv = true;
            }
            if (fd.has_hamaker) {
                d3 ha = surface_hamaker(fd.hamaker, xf, xi_);
                if (hv) {
                    fa = add(fa, ha);
                    fal = add(fal, zero3());
                } else {
                    fa = ha;
                    fal = zero3();
                }
            }
            if (f == 0) {
                ua = fa;
                ual = fal;
            } else {
                ua = add(ua, fa);
                ual = add(ual, fal);
            }
        }
        accA = add(accA, ua);
        accW = add(accW, ual);
    }
    st4(S.a, i, accA);
    st4(S.al, i, accW);
    st4(S.v_out, i, add(vi, scl(hdt, accA)));
    st4(S.w_out, i, add(wi, scl(hdt, accW)));
    if (!isfinite(accA.x) || !isfinite(accA.y) || !isfinite(accA.z) || !isfinite(accW.x) || !isfinite(accW.y) ||
        !isfinite(accW.z))
        set_error(S.err, LG_DEVERR_NONFINITE);
}

template <bool VERLET, int SL>
static void launch_compact(const Params &P, const StateView &S, const PairView &PV, const BondView &BV, double hdt,
                           double dt, int move_facets, const MixedExtra *MX, cudaStream_t st) {
    using Sh = Shape<SL>;
    const size_t smem = sizeof(WarpSmem<SL>) * Sh::kWarps + (SL > 1 ? sizeof(float) * 12 * 32 * Sh::kWarps : 0);
    const int64_t rows_per_block = Sh::kRowWarps * 32;
    const unsigned blocks = (unsigned)((P.n + rows_per_block - 1) / rows_per_block);
    static thread_local int attr_device = -1;  // the attribute is per device; set once per thread and device
    int dev = 0;
    cudaGetDevice(&dev);
#if LG_COMPACT_MIXED
    auto kern = forces_compact_mixed<VERLET, SL>;
#else
    auto kern = forces_compact_fp64<VERLET, SL>;
#endif
    if (attr_device != dev) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr_device = dev;
    }
#if LG_COMPACT_MIXED
    kern<<<blocks, Sh::kWarps * 32, smem, st>>>(P, S, PV, BV, hdt, dt, move_facets, *MX);
#else
    (void)MX;
    kern<<<blocks, Sh::kWarps * 32, smem, st>>>(P, S, PV, BV, hdt, dt, move_facets);
#endif
}

#if LG_COMPACT_MIXED
void launch_forces_compact_mixed(const Params &P, const StateView &S, const PairView &PV, const BondView &BV, double hdt,
                                 double dt, int move_facets, const MixedExtra &MX, cudaStream_t st) {
    // slice rows over four warps when the launch has too few rows to fill the GPU with warps
    const bool slice = P.n < 152 * 32 * 12;
    const bool ver = P.pairs == LG_PAIRS_VERLET;
    if (ver && slice) launch_compact<true, 4>(P, S, PV, BV, hdt, dt, move_facets, &MX, st);
    else if (ver) launch_compact<true, 1>(P, S, PV, BV, hdt, dt, move_facets, &MX, st);
    else if (slice) launch_compact<false, 4>(P, S, PV, BV, hdt, dt, move_facets, &MX, st);
    else launch_compact<false, 1>(P, S, PV, BV, hdt, dt, move_facets, &MX, st);
}
#else
void launch_forces_compact_fp64(const Params &P, const StateView &S, const PairView &PV, const BondView &BV, double hdt,
                                double dt, int move_facets, cudaStream_t st) {
    if (P.pairs == LG_PAIRS_VERLET)
        launch_compact<true, 1>(P, S, PV, BV, hdt, dt, move_facets, nullptr, st);
    else
        launch_compact<false, 1>(P, S, PV, BV, hdt, dt, move_facets, nullptr, st);
}
#endif

}  // namespace lg
