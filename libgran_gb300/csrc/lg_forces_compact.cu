// lg_forces_compact.cu -- warp-compacted force kernel (sm_103a), FP64; compiled with --fmad=false.
// Two instances: the reference's arithmetic operation for operation (bit-identical to the sequential
// evaluation), and FAST (LG_FORCE_KERNEL_FP64_FAST), which multiplies by one reciprocal where libgran
// divides a vector by a scalar and evaluates the Hamaker bracket over one common denominator
// (per-step forces within 1e-12 of the reference's); both decide
// contact with the reference's exact overlap.
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
// with no floating-point atomics. Every pair value is computed by the same functions as the
// sequential kernel and the fold adds in the same order, so the result is bit-identical to the
// sequential evaluation. The mixed-precision counterpart is lg_forces_compact_mixed.cu.
#include "lg_compact.cuh"
#include "lg_kernels.h"

namespace lg {

namespace {

using compact::kHCap;
using compact::kWin;
using compact::slot_of;
constexpr int kGroup = kWin;  // slots classified per memory round trip: one window
// The FP64 kernel runs with SL = 1 (no slicing), so every row is added in ascending slot order.
template <int SL>
struct Shape {
    static constexpr int kSlices = SL;
    static constexpr int kRowWarps = SL == 1 ? 2 : 1;
    static constexpr int kRound = SL == 1 ? 128 : 64;  // slots classified per round (per warp)
    static constexpr int kCCap = SL == 1 ? 256 : 160;  // contact queue capacity per round
    static constexpr int kWarps = kSlices * kRowWarps;
};
typedef double rt;

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
};

// One queued contact / bond pair: owner row io (lane own of the warp), slot e, partner j.
template <int SL, bool FAST>
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
    if ((fl & kBonded) && BV.cn) {  // 5-connector model
        const int64_t be = (int64_t)bond_slot_of(fl) * n + io;
        const d3 xj = ld4(S.x, j), vj = ld4(S.v, j), wj = ld4(S.w, j);
        connector_force(P.connector, P.contact.r_part, P.contact.mass, P.contact.inertia, xo, xj, vo, vj, wo, wj, BV.cn,
                        bs, be, (int64_t)BV.rev[be] * n + j, pa, pal);
    } else if (fl & kBonded) {
        const bool breaking = P.binary_model == LG_BINARY_BREAKING_SINTER;
        const int64_t be = (int64_t)bond_slot_of(fl) * n + io;
        d3 s[3];
#pragma unroll
        for (int c = 0; c < 3; ++c)
            s[c] = mk3(BV.xi[(3 * c) * bs + be], BV.xi[(3 * c + 1) * bs + be], BV.xi[(3 * c + 2) * bs + be]);
        const d3 vj = ld4(S.v, j), wj = ld4(S.w, j);
        const bool brk =
            bond_force<FAST>(P.sinter, dx, vo, vj, wo, wj, s, breaking, breaking ? BV.strength[be] : 0.0, pa, pal);
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
            contact_touching<FAST>(P.contact, nn, overlap, vo, vj, wo, wj, s, pa, pal);
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

template <int SL, bool FAST>
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
    if (on) ha = hamaker_accel_n<FAST>(P.hamaker_model, P.hamaker, r, rn);
    W.hres[q][0] = ha.x;
    W.hres[q][1] = ha.y;
    W.hres[q][2] = ha.z;
}

}  // namespace

template <bool VERLET, int SL, bool FAST>
__global__ void __launch_bounds__(Shape<SL>::kWarps * 32)
    forces_compact_fp64(Params P, StateView S, PairView PV, BondView BV, double hdt, double dt, int move_facets)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int kSlices = Shape<SL>::kSlices, kRowWarps = Shape<SL>::kRowWarps;
    constexpr int kRound = Shape<SL>::kRound, kCCap = Shape<SL>::kCCap;
    WarpSmem<SL> &W = reinterpret_cast<WarpSmem<SL> *>(smem_raw)[warp];
    const int rw = warp / kSlices, sl = warp % kSlices;  // row group of the block, slice of it
    const int64_t n = P.n;
    const int64_t row0 = ((int64_t)blockIdx.x * kRowWarps + rw) * 32;
    const int64_t i = row0 + lane;
    const bool active = i < n;
    const int bm = P.binary_model, hm = P.hamaker_model;
    const uint32_t lt = (1u << lane) - 1u;

    if (move_facets && blockIdx.x == 0 && threadIdx.x == 0) compact::move_facets(P, S, dt);

    d3 xi_ = zero3(), vi = zero3(), wi = zero3();
    int64_t len = 0;
    if (active) {
        xi_ = ld4(S.x, i);
        vi = ld4(S.v, i);
        wi = ld4(S.w, i);
        len = VERLET ? (int64_t)PV.row_len[i] : n - 1;
    }
    W.xo[lane] = xi_;
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
    d3 acc = zero3(), accw = zero3();
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
            d3 pg[kGroup];
#pragma unroll
            for (int u = 0; u < kGroup; ++u) pg[u] = (k0 + u < len) ? ld4(S.x, jg[u]) : xi_;
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
                    const double d2 = sqn(sub(xi_, pg[u]));
                    const bool ccand = !(d2 > P.contact_skip_d2);
                    if (hm == LG_HAMAKER_LIMITED)
                        hb = !(d2 > P.hamaker_skip_d2);
                    else if (hm != LG_HAMAKER_NONE)
                        hb = true;
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
                contact_item<SL, FAST>(P, S, PV, BV, W, cdone + lane, row0, kstart, sl, n, xs, bs);
                cdone += 32;
                __syncwarp();
            }
        }
        const int64_t kend = k;
        if (cdone < ccount) {
            if (cdone + lane < ccount)
                contact_item<SL, FAST>(P, S, PV, BV, W, cdone + lane, row0, kstart, sl, n, xs, bs);
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
                hamaker_item<SL, FAST>(P, S, W, q);
            __syncwarp();
#pragma unroll
            for (int t = 0; t < kWin; ++t) {
                const int64_t kk = kw + t;
                if (vw + t < kend && kk < len) {
                    const uint32_t bh = W.hball[t], bc = W.cball[vw + t - kstart];
                    const bool hb = (bh >> lane) & 1u, cb = (bc >> lane) & 1u;
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
                }
            }
            __syncwarp();
        }
        kstart = kend;
    }
    if (!active) return;

    compact::finish_row(P, S, i, n, acc, accw, vi, wi, hdt);
}

template <bool VERLET, int SL, bool FAST>
static void launch_compact(const Params &P, const StateView &S, const PairView &PV, const BondView &BV, double hdt,
                           double dt, int move_facets, cudaStream_t st) {
    using Sh = Shape<SL>;
    const size_t smem = sizeof(WarpSmem<SL>) * Sh::kWarps;
    const int64_t rows_per_block = Sh::kRowWarps * 32;
    const unsigned blocks = (unsigned)((P.n + rows_per_block - 1) / rows_per_block);
    static thread_local int attr_device = -1;  // the attribute is per device; set once per thread and device
    int dev = 0;
    cudaGetDevice(&dev);
    auto kern = forces_compact_fp64<VERLET, SL, FAST>;
    if (attr_device != dev) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr_device = dev;
    }
    kern<<<blocks, Sh::kWarps * 32, smem, st>>>(P, S, PV, BV, hdt, dt, move_facets);
}

void launch_forces_compact_fp64(const Params &P, const StateView &S, const PairView &PV, const BondView &BV, double hdt,
                                double dt, int move_facets, cudaStream_t st, bool fast) {
    const bool ver = P.pairs == LG_PAIRS_VERLET;
    if (fast) {
        if (ver) launch_compact<true, 1, true>(P, S, PV, BV, hdt, dt, move_facets, st);
        else launch_compact<false, 1, true>(P, S, PV, BV, hdt, dt, move_facets, st);
    } else {
        if (ver) launch_compact<true, 1, false>(P, S, PV, BV, hdt, dt, move_facets, st);
        else launch_compact<false, 1, false>(P, S, PV, BV, hdt, dt, move_facets, st);
    }
}

}  // namespace lg
