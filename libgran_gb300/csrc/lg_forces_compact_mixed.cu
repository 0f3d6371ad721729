// lg_forces_compact_mixed.cu -- force evaluation of the mixed-precision path (sm_103a): two
// warp-compacted kernels, one lane per row (particle i), slot layout and flags shared with the FP64
// path.
//
//   forces_contacts_mixed  contact and bond pairs. Verlet mode walks each row's contact candidates
//                          (PairView::near_*, listed by the list build: the slots within contact
//                          reach plus the Verlet skin, and bonded slots); all-pairs mode walks every
//                          slot. Candidates are queued per warp (ballot order) and evaluated 32 at a
//                          time; the pair's linear and angular accelerations are folded per row in
//                          slot order into float-float sums (MixedExtra::csum).
//   forces_hamaker_mixed   Hamaker pairs over all slots, in windows of four slots: the owner lane
//                          gathers its partners' float-float positions, the window's Hamaker pairs
//                          are evaluated one per lane from those shared-memory copies, the next
//                          window's partners are loaded meanwhile. For launches with few rows a
//                          row's windows are sliced over SL warps, whose partial sums are combined
//                          in slice order. Runs beside forces_contacts_mixed (two streams).
//   forces_finish_ff       completion inside a run of steps (no facets, no body term): the sums, the
//                          end-of-step half kick, the next step's half kick and drift, all in
//                          float-float on the FP32 pipes; the run's last step writes the FP64 state.
//   forces_finish_mixed    the FP64 completion (facets, body terms, single steps): contact part +
//                          Hamaker part to FP64, unary terms, stores, half kick (+ next kick and
//                          drift).
//
// Precision: positions come as interleaved float-float pairs (MixedExtra::x32, hi + lo = x -
// origin) and a pair's separation and q = |d|^2 - (2r)^2 are formed with error-free FP32
// transformations (separation_ff), so the surface gap and the overlap keep FP32 relative precision
// however small they are; velocities come as float-float copies (MixedExtra::v32); springs are
// float-float pairs in 8-byte slots, one 9-component record per slot or bond (spring_at), updated
// by FP32 increments (shear_ff). No pair costs an FP64 operation. Per-row sums are float-float (compensated) FP32 accumulations in an order fixed by
// the row alone, so a system gives the same bits alone and inside a batch (with the same slicing).
#include <cstddef>

#include "lg_compact.cuh"
#include "lg_kernels.h"

// Slices per row group of the Hamaker kernel: 0 chooses from the launch size (compile-time
// override for tuning).
#ifndef LG_MIXED_SLICES
#define LG_MIXED_SLICES 0
#endif

namespace lg {

namespace {

using compact::kHCap;
using compact::kWin;
using compact::slot_of;

// ---- contact / bond kernel ----
constexpr int kCRound = 32;  // entries per lane classified per round
constexpr int kCQ = 64;      // contact queue capacity (>= 32 + 31)
constexpr int kCWarps = 2;   // warps per block
#ifndef LG_HAMAKER_REGS
#define LG_HAMAKER_REGS 96  // register budget of the Hamaker kernel (compile-time override for tuning)
#endif
// Resident blocks per SM the contact kernel is compiled for (its register budget): beside the Hamaker
// kernel (two streams) a tighter budget lets more of both kernels' warps share an SM; alone, the
// looser one avoids spills. Measured on the 32768-particle workload (graph-replayed steps): 12 blocks
// beside the Hamaker kernel, 9.3e8 against 8.2e8 particle-steps/s with 8; contacts alone, 8 blocks,
// 30 against 36 us per step with 12.
#ifndef LG_CONTACT_MIN_BLOCKS
#define LG_CONTACT_MIN_BLOCKS 12
#endif
#ifndef LG_CONTACT_MIN_BLOCKS_ALONE
#define LG_CONTACT_MIN_BLOCKS_ALONE 8
#endif
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

// ---- Hamaker kernel ----
template <int SL>
struct ShapeH {
    static constexpr int kSlices = SL;
    static constexpr int kRowWarps = SL == 1 ? 2 : 1;  // 32-row groups per block
    static constexpr int kWarps = kSlices * kRowWarps;
    // blocks per SM that the register budget allows (shared memory allows as many)
    static constexpr int kMinBlocks = 65536 / (kWarps * 32 * LG_HAMAKER_REGS);
};
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


}  // namespace

// Contact and bond pairs of rows row0 .. row0 + 32/T - 1: T lanes per row, lane t of a row taking
// its entries t, t + T, ... (so short candidate lists still fill the warp); each lane folds its
// pairs in entry order and the row's T partial sums are combined in lane order. csum receives the
// contact part of the row's accelerations as float-float pairs.
template <bool NEAR, int T, int MINB>
__global__ void __launch_bounds__(kCWarps * 32, MINB)
    forces_contacts_mixed(Params P, StateView S, PairView PV, BondView BV, MixedExtra MX) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int kRows = 32 / T;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int r = lane / T, sub = lane % T;  // local row and sub-lane
    ContactSmem &W = reinterpret_cast<ContactSmem *>(smem_raw)[warp];
    const int64_t n = P.n;
    const int64_t row0 = ((int64_t)blockIdx.x * kCWarps + warp) * kRows;
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

// Hamaker pairs of rows row0 .. row0 + 31; hsum receives the Hamaker part of the row's acceleration
// as float-float pairs.
template <bool VERLET, int SL>
__global__ void __launch_bounds__(ShapeH<SL>::kWarps * 32, ShapeH<SL>::kMinBlocks)
    forces_hamaker_mixed(Params P, PairView PV, MixedExtra MX) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int kSlices = ShapeH<SL>::kSlices, kRowWarps = ShapeH<SL>::kRowWarps;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    HamakerSmem *Wall = reinterpret_cast<HamakerSmem *>(smem_raw);
    HamakerSmem &W = Wall[warp];
    const int rw = warp / kSlices, sl = warp % kSlices;  // row group of the block, slice of it
    const int64_t n = P.n;
    const int64_t row0 = ((int64_t)blockIdx.x * kRowWarps + rw) * 32;
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
    // this warp's windows: sl, sl + kSlices, ...; virtual slot v maps to slot_of<SL>(v, sl)
    const int64_t nwin = (maxlen + kWin - 1) / kWin;
    const int64_t mywin = nwin > sl ? (nwin - sl + kSlices - 1) / kSlices : 0;
    const int64_t vmax = mywin * kWin;
    ff acch[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    __syncwarp();

    // partners of the lane's row in the window at virtual slot v (-1: past the row's end)
    int32_t jn[kWin];
    auto load_window = [&](int64_t v) {
        const int64_t k0 = slot_of<SL>(v, sl);
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

    if (kSlices > 1) {
        // combine the slices' partial sums of each row in slice order (fixed, deterministic); each
        // warp parks its partials in its own queue, which is no longer in use
        float *mine = reinterpret_cast<float *>(W.hhi);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            mine[(2 * c) * 32 + lane] = acch[c].hi;
            mine[(2 * c + 1) * 32 + lane] = acch[c].lo;
        }
        __syncthreads();
        if (sl != 0) return;
        for (int q = 1; q < kSlices; ++q) {
            const float *o = reinterpret_cast<const float *>(Wall[rw * kSlices + q].hhi);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                ff_acc(acch[c], o[(2 * c) * 32 + lane]);
                ff_acc(acch[c], o[(2 * c + 1) * 32 + lane]);
            }
        }
    }
    if (!active) return;
    MX.hsum[2 * i] = make_float4(acch[0].hi, acch[0].lo, acch[1].hi, acch[1].lo);
    MX.hsum[2 * i + 1] = make_float4(acch[2].hi, acch[2].lo, 0.f, 0.f);
}

// Completion of row i in FP64: contact part (csum when `contacts`) plus the Hamaker part (hsum when
// `hamaker`), both converted to FP64, then the unary terms, stores and half kick; with `kick` also
// the next step's opening half kick and drift, and the float-float copies of the new state.
template <bool FACETS>
__device__ __forceinline__ void finish_fp64_row(const Params &P, const StateView &S, int64_t i, double hdt, double dt,
                                                int contacts, int hamaker, int kick, const MixedExtra &MX) {
    // every input is loaded before anything is stored (the buffers are distinct)
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 c0 = contacts ? MX.csum[3 * i] : z4, c1 = contacts ? MX.csum[3 * i + 1] : z4,
                 c2 = contacts ? MX.csum[3 * i + 2] : z4;
    const float4 h0 = hamaker ? MX.hsum[2 * i] : z4, h1 = hamaker ? MX.hsum[2 * i + 1] : z4;
    const d3 vi = ld4(S.v, i), wi = ld4(S.w, i);
    d3 xo = zero3(), tho = zero3();
    if (kick) {
        xo = ld4(S.x, i);
        tho = ld4(S.th, i);
    }
    // contact part (float-float pairs hi, lo), then the Hamaker part
    d3 a_tot = mk3((double)c0.x + (double)c0.y, (double)c0.z + (double)c0.w, (double)c1.x + (double)c1.y);
    d3 al_tot = mk3((double)c1.z + (double)c1.w, (double)c2.x + (double)c2.y, (double)c2.z + (double)c2.w);
    if (hamaker) {
        const d3 ah = mk3((double)h0.x + (double)h0.y, (double)h0.z + (double)h0.w, (double)h1.x + (double)h1.y);
        a_tot = contacts ? add(a_tot, ah) : ah;
    }
    compact::finish_row<FACETS>(P, S, i, P.n, a_tot, al_tot, vi, wi, hdt);
    if (kick) {  // the next step's opening half kick and drift (the end-of-step velocities are not kept)
        const uint32_t h = hold_of(P.hold, i);
        const bool hv = h & LG_HOLD_V, hw = h & LG_HOLD_OMEGA;
        const d3 vh = kick_unless(kick_unless(vi, hdt, a_tot, hv), hdt, a_tot, hv);
        const d3 wh = kick_unless(kick_unless(wi, hdt, al_tot, hw), hdt, al_tot, hw);
        st4(S.v_out, i, vh);
        st4(S.w_out, i, wh);
        const d3 xn = (h & LG_HOLD_X) ? xo : add(xo, scl(dt, vh));
        const d3 thn = (h & LG_HOLD_THETA) ? tho : add(tho, scl(dt, wh));
        if (!(h & LG_HOLD_X)) st4(S.x, i, xn);
        if (!(h & LG_HOLD_THETA)) st4(S.th, i, thn);
        rel_ff(xn, MX.ox, MX.oy, MX.oz, MX.agg, MX.orig, i, P.n, MX.x32);
        state_ff(vh, wh, i, P.n, MX.v32, MX.s32);
    }
}

template <bool FACETS>
__global__ void __launch_bounds__(64) forces_finish_mixed(Params P, StateView S, double hdt, double dt,
                                                          int move_facets, int contacts, int hamaker, int kick,
                                                          MixedExtra MX) {
    if (move_facets && blockIdx.x == 0 && threadIdx.x == 0) compact::move_facets(P, S, dt);
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    finish_fp64_row<FACETS>(P, S, i, hdt, dt, contacts, hamaker, kick, MX);
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

// Completion of a step of a run (no facets, no body term), integrating in float-float on the FP32
// pipes: between the first and the last step of a run the state lives in x32 / v32 / s32 (the FP64
// x and theta keep the values of the run's first step, v and omega are left behind) and the last
// step writes the FP64 state. Velocities and spins are float-float values (about 2^-46 of their
// magnitude). Positions are carried twice: x32 (relative to the system origin) advances for the
// force kernels, and the displacement since the run's first step accumulates from zero in s32, so
// that the last step's FP64 position x_first + displacement is not limited by the float-float
// resolution of x32 (a step moves a particle by about 1e-9 of its distance from the origin); the
// rotation theta accumulates the same way.
//   LAST = false: the end-of-step half kick, the next step's opening half kick and drift;
//   LAST = true:  the end-of-step half kick, then a, alpha, v, omega, x and theta in FP64.
// s32: [i] low parts of omega; [n + i] / [2n + i] displacement hi / lo; [3n + i] / [4n + i]
// rotation hi / lo.
template <bool LAST>
__global__ void __launch_bounds__(64) forces_finish_ff(Params P, StateView S, int contacts, int hamaker, ff hdt, ff dt,
                                                       double hdt_d, double dt_d, MixedExtra MX) {
    const int64_t n = P.n;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t h = hold_of(P.hold, i);
    if (h) {  // a held particle keeps its FP64 state current (a held value stays exactly as it was)
        finish_fp64_row<false>(P, S, i, hdt_d, dt_d, contacts, hamaker, LAST ? 0 : 1, MX);
        return;
    }
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 c0 = contacts ? MX.csum[3 * i] : z4, c1 = contacts ? MX.csum[3 * i + 1] : z4,
                 c2 = contacts ? MX.csum[3 * i + 2] : z4;
    const float4 h0 = hamaker ? MX.hsum[2 * i] : z4, h1 = hamaker ? MX.hsum[2 * i + 1] : z4;
    const float4 vh = MX.v32[i], vl = MX.v32[n + i], wh = MX.v32[2 * n + i], wl = MX.s32[i];
    const float4 dh = MX.s32[n + i], dl = MX.s32[2 * n + i], rh = MX.s32[3 * n + i], rl = MX.s32[4 * n + i];
    ff a[3] = {{c0.x, c0.y}, {c0.z, c0.w}, {c1.x, c1.y}};
    const ff al[3] = {{c1.z, c1.w}, {c2.x, c2.y}, {c2.z, c2.w}};
    if (hamaker) {
        const ff ah[3] = {{h0.x, h0.y}, {h0.z, h0.w}, {h1.x, h1.y}};
#pragma unroll
        for (int c = 0; c < 3; ++c) a[c] = contacts ? ff_add(a[c], ah[c]) : ah[c];
    }
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
    const float4 xh = MX.x32[2 * i], xl = MX.x32[2 * i + 1];
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
    MX.x32[2 * i] = make_float4(x[0].hi, x[1].hi, x[2].hi, 0.f);
    MX.x32[2 * i + 1] = make_float4(x[0].lo, x[1].lo, x[2].lo, 0.f);
    MX.v32[i] = make_float4(v[0].hi, v[1].hi, v[2].hi, 0.f);
    MX.v32[n + i] = make_float4(v[0].lo, v[1].lo, v[2].lo, 0.f);
    MX.v32[2 * n + i] = make_float4(w[0].hi, w[1].hi, w[2].hi, 0.f);
    MX.s32[i] = make_float4(w[0].lo, w[1].lo, w[2].lo, 0.f);
    MX.s32[n + i] = make_float4(dx[0].hi, dx[1].hi, dx[2].hi, 0.f);
    MX.s32[2 * n + i] = make_float4(dx[0].lo, dx[1].lo, dx[2].lo, 0.f);
    MX.s32[3 * n + i] = make_float4(dr[0].hi, dr[1].hi, dr[2].hi, 0.f);
    MX.s32[4 * n + i] = make_float4(dr[0].lo, dr[1].lo, dr[2].lo, 0.f);
}

namespace {

template <bool NEAR>
void launch_contacts(const Params &P, const StateView &S, const PairView &PV, const BondView &BV, const MixedExtra &MX,
                     cudaStream_t st, bool beside_hamaker) {
    constexpr int T = kContactLanes;
    const size_t smem = sizeof(ContactSmem) * kCWarps;
    const int64_t rows_per_block = (32 / T) * kCWarps;
    const unsigned blocks = (unsigned)((P.n + rows_per_block - 1) / rows_per_block);
    if (beside_hamaker)
        forces_contacts_mixed<NEAR, T, LG_CONTACT_MIN_BLOCKS><<<blocks, kCWarps * 32, smem, st>>>(P, S, PV, BV, MX);
    else
        forces_contacts_mixed<NEAR, T, LG_CONTACT_MIN_BLOCKS_ALONE><<<blocks, kCWarps * 32, smem, st>>>(P, S, PV, BV, MX);
}

template <bool VERLET, int SL>
void launch_hamaker(const Params &P, const PairView &PV, const MixedExtra &MX, cudaStream_t st) {
    using Sh = ShapeH<SL>;
    const size_t smem = sizeof(HamakerSmem) * Sh::kWarps;
    const int64_t rows_per_block = Sh::kRowWarps * 32;
    const unsigned blocks = (unsigned)((P.n + rows_per_block - 1) / rows_per_block);
    if (smem > 48 * 1024) {  // above the default dynamic shared-memory limit: opt in, once per device
        static thread_local int attr_device = -1;
        int dev = 0;
        cudaGetDevice(&dev);
        if (attr_device != dev) {
            cudaFuncSetAttribute(forces_hamaker_mixed<VERLET, SL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            attr_device = dev;
        }
    }
    forces_hamaker_mixed<VERLET, SL><<<blocks, Sh::kWarps * 32, smem, st>>>(P, PV, MX);
}

// Slices per 32-row group of the Hamaker kernel: the most slices that keep the launch within about
// two waves of resident warps (152 SMs x 20); rows of long launches are not sliced.
int hamaker_slices(int64_t n) {
    if (LG_MIXED_SLICES == 1 || LG_MIXED_SLICES == 2 || LG_MIXED_SLICES == 4 || LG_MIXED_SLICES == 8)
        return LG_MIXED_SLICES;
    const int64_t two_waves = 2 * 152 * 20;
    const int64_t groups = (n + 31) / 32;
    if (groups * 4 <= two_waves) return 4;
    if (groups * 2 <= two_waves) return 2;
    return 1;
}

}  // namespace

int launch_forces_compact_mixed(const Params &P, const StateView &S, const PairView &PV, const BondView &BV, double hdt,
                                double dt, int move_facets, bool kick, bool prev_fused, const MixedExtra &MX,
                                cudaStream_t st, cudaStream_t side, cudaEvent_t fork, cudaEvent_t join) {
    const bool ver = P.pairs == LG_PAIRS_VERLET;
    const int contacts = P.binary_model != LG_BINARY_NONE ? 1 : 0;
    const int hamaker = P.hamaker_model != LG_HAMAKER_NONE ? 1 : 0;
    int kernels = 1;
    if (contacts) {  // the contact branch runs beside the Hamaker kernel
        cudaEventRecord(fork, st);
        cudaStreamWaitEvent(side, fork, 0);
        // the FP64 positions are current unless the step before integrated in float-float
        MixedExtra MC = MX;
        MC.x64 = prev_fused ? nullptr : S.x;
        if (ver && PV.near_len)
            launch_contacts<true>(P, S, PV, BV, MC, side, hamaker != 0);
        else
            launch_contacts<false>(P, S, PV, BV, MC, side, hamaker != 0);
        ++kernels;
    }
    if (hamaker) {
        switch (hamaker_slices(P.n)) {
            case 8:
                if (ver) launch_hamaker<true, 8>(P, PV, MX, st);
                else launch_hamaker<false, 8>(P, PV, MX, st);
                break;
            case 4:
                if (ver) launch_hamaker<true, 4>(P, PV, MX, st);
                else launch_hamaker<false, 4>(P, PV, MX, st);
                break;
            case 2:
                if (ver) launch_hamaker<true, 2>(P, PV, MX, st);
                else launch_hamaker<false, 2>(P, PV, MX, st);
                break;
            default:
                if (ver) launch_hamaker<true, 1>(P, PV, MX, st);
                else launch_hamaker<false, 1>(P, PV, MX, st);
        }
        ++kernels;
    }
    if (contacts) {
        cudaEventRecord(join, side);
        cudaStreamWaitEvent(st, join, 0);
    }
    const unsigned blocks = (unsigned)((P.n + 63) / 64);
    // without facets or a body term the completion of a run's steps integrates in float-float; the
    // FP64 completion serves the rest (and a run's last step when the step before was not fused)
    const bool plain = P.n_facets == 0 && !P.ext_a && MX.s32;
    auto split = [](double d) { const float hi = (float)d; return ff{hi, (float)(d - (double)hi)}; };
    if (plain && kick) {
        forces_finish_ff<false><<<blocks, 64, 0, st>>>(P, S, contacts, hamaker, split(hdt), split(dt), hdt, dt, MX);
        return kernels;
    }
    if (plain && prev_fused) {
        forces_finish_ff<true><<<blocks, 64, 0, st>>>(P, S, contacts, hamaker, split(hdt), split(dt), hdt, dt, MX);
        return kernels;
    }
    if (P.n_facets > 0 || P.ext_a)
        forces_finish_mixed<true><<<blocks, 64, 0, st>>>(P, S, hdt, dt, move_facets, contacts, hamaker, kick ? 1 : 0, MX);
    else
        forces_finish_mixed<false><<<blocks, 64, 0, st>>>(P, S, hdt, dt, 0, contacts, hamaker, kick ? 1 : 0, MX);
    return kernels;
}

}  // namespace lg
