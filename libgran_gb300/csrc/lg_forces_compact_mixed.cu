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
// The per-pair and per-row pieces (and the precision scheme) are in lg_mixed_pairs.cuh, shared with
// the persistent step kernel (lg_step_mixed.cu). Per-row sums are in an order fixed by the row
// alone, so a system gives the same bits alone and inside a batch (with the same slicing).
#include <cstddef>

#include "lg_mixed_pairs.cuh"

namespace lg {

using namespace mixed;

namespace {

// ---- launch shapes of the two-stream kernels ----
// Slices per row group of the Hamaker kernel: 0 chooses from the launch size (compile-time
// override for tuning).
#ifndef LG_MIXED_SLICES
#define LG_MIXED_SLICES 0
#endif
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
template <int SL>
struct ShapeH {
    static constexpr int kSlices = SL;
    static constexpr int kRowWarps = SL == 1 ? 2 : 1;  // 32-row groups per block
    static constexpr int kWarps = kSlices * kRowWarps;
    // blocks per SM that the register budget allows (shared memory allows as many)
    static constexpr int kMinBlocks = 65536 / (kWarps * 32 * LG_HAMAKER_REGS);
};
}  // namespace

// Contact and bond pairs of rows row0 .. row0 + 32/T - 1 per warp (contact_rows), csum receives the
// contact part of the row's accelerations.
template <bool NEAR, int T, int MINB>
__global__ void __launch_bounds__(kCWarps * 32, MINB)
    forces_contacts_mixed(Params P, StateView S, PairView PV, BondView BV, MixedExtra MX) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int kRows = 32 / T;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    ContactSmem &W = reinterpret_cast<ContactSmem *>(smem_raw)[warp];
    contact_rows<NEAR, T>(P, PV, BV, MX, W, ((int64_t)blockIdx.x * kCWarps + warp) * kRows, lane);
}

// Hamaker pairs of rows row0 .. row0 + 31; hsum receives the Hamaker part of the row's acceleration
// as float-float pairs. With SL > 1 slices the row group's windows are spread over SL warps of the
// block, whose partial sums are combined in slice order.
template <bool VERLET, int SL>
__global__ void __launch_bounds__(ShapeH<SL>::kWarps * 32, ShapeH<SL>::kMinBlocks)
    forces_hamaker_mixed(Params P, PairView PV, MixedExtra MX) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int kSlices = ShapeH<SL>::kSlices, kRowWarps = ShapeH<SL>::kRowWarps;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    HamakerSmem *Wall = reinterpret_cast<HamakerSmem *>(smem_raw);
    HamakerSmem &W = Wall[warp];
    const int rw = warp / kSlices, sl = warp % kSlices;  // row group of the block, slice of it
    const int64_t row0 = ((int64_t)blockIdx.x * kRowWarps + rw) * 32;
    const int64_t i = row0 + lane;
    const bool active = i < P.n;
    ff acch[3];
    hamaker_rows<VERLET>(P, PV, MX, W, row0, sl, kSlices, lane, acch);
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
    if (i >= P.n || inactive_of(P.hold, i)) return;
    finish_fp64_row<FACETS>(P, S, i, hdt, dt, contacts, hamaker, kick, MX);
}

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
    if (h & kHoldInactive) return;  // takes no part
    if (h) {  // a held particle keeps its FP64 state current (a held value stays exactly as it was)
        finish_fp64_row<false>(P, S, i, hdt_d, dt_d, contacts, hamaker, LAST ? 0 : 1, MX);
        return;
    }
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 c0 = contacts ? MX.csum[3 * i] : z4, c1 = contacts ? MX.csum[3 * i + 1] : z4,
                 c2 = contacts ? MX.csum[3 * i + 2] : z4;
    const float4 h0 = hamaker ? MX.hsum[2 * i] : z4, h1 = hamaker ? MX.hsum[2 * i + 1] : z4;
    ff a[3] = {{c0.x, c0.y}, {c0.z, c0.w}, {c1.x, c1.y}};
    const ff al[3] = {{c1.z, c1.w}, {c2.x, c2.y}, {c2.z, c2.w}};
    if (hamaker) {
        const ff ah[3] = {{h0.x, h0.y}, {h0.z, h0.w}, {h1.x, h1.y}};
#pragma unroll
        for (int c = 0; c < 3; ++c) a[c] = contacts ? ff_add(a[c], ah[c]) : ah[c];
    }
    finish_ff_plain<LAST>(S, i, n, a, al, hdt, dt, MX, MX.x32, MX.v32);
}

namespace {

// Lanes per row of the contact kernel: T = 2 (or 1, a tuning choice that suits large batches) for
// candidate lists (a few entries per row); a whole warp per row for all pairs (n - 1 candidates per
// row: the lanes share them, and the row count no longer bounds the warps a small system can use).
template <bool NEAR, int T>
void launch_contacts(const Params &P, const StateView &S, const PairView &PV, const BondView &BV, const MixedExtra &MX,
                     cudaStream_t st, bool beside_hamaker) {
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

}  // namespace

// Slices per 32-row group of the Hamaker kernel: the most slices that keep the launch within about
// two waves of resident warps (152 SMs x 20); rows of long launches are not sliced.
int mixed_hamaker_slices(int64_t n) {
    if (LG_MIXED_SLICES == 1 || LG_MIXED_SLICES == 2 || LG_MIXED_SLICES == 4 || LG_MIXED_SLICES == 8)
        return LG_MIXED_SLICES;
    const int64_t two_waves = 2 * 152 * 20;
    const int64_t groups = (n + 31) / 32;
    if (groups * 4 <= two_waves) return 4;
    if (groups * 2 <= two_waves) return 2;
    return 1;
}

// All pairs: every row holds n - 1 partners, so small systems slice their rows further (up to 16
// warps per 32-row group) under the same two-wave bound.
static int mixed_hamaker_slices_all_pairs(int64_t n) {
    const int64_t two_waves = 2 * 152 * 20;
    const int64_t groups = (n + 31) / 32;
    for (int sl = 16; sl > 1; sl /= 2)
        if (groups * sl <= two_waves && (n - 1) >= 4 * kWin * sl) return sl;
    return 1;
}

int launch_forces_compact_mixed(const Params &P, const StateView &S, const PairView &PV, const BondView &BV, double hdt,
                                double dt, int move_facets, bool kick, bool prev_fused, const MixedExtra &MX,
                                cudaStream_t st, cudaStream_t side, cudaEvent_t fork, cudaEvent_t join, int slices,
                                int contact_lanes) {
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
        if (ver && PV.near_len && contact_lanes == 1)
            launch_contacts<true, 1>(P, S, PV, BV, MC, side, hamaker != 0);
        else if (ver && PV.near_len)
            launch_contacts<true, kContactLanes>(P, S, PV, BV, MC, side, hamaker != 0);
        else
            launch_contacts<false, 32>(P, S, PV, BV, MC, side, hamaker != 0);
        ++kernels;
    }
    if (hamaker) {
        switch (slices > 0 ? slices : ver ? mixed_hamaker_slices(P.n) : mixed_hamaker_slices_all_pairs(P.n)) {
            case 16:
                if (ver) launch_hamaker<true, 16>(P, PV, MX, st);
                else launch_hamaker<false, 16>(P, PV, MX, st);
                break;
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
