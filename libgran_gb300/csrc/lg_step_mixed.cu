// lg_step_mixed.cu -- the mixed-precision force evaluation and completion of one velocity-Verlet
// step inside a run of steps as ONE persistent launch (sm_103a).
//
// The work of a step is a list of items, each a warp's worth: for every group of 32 rows, two
// contact items (16 rows each, two lanes per row: contact_rows) and `slices` Hamaker items (the
// group's windows sl, sl + slices, ...: hamaker_rows). A launch has as many blocks as fit on the
// GPU at once; each warp pulls item indices from a device counter until the list is exhausted, so
// contact and Hamaker work share every SM and uneven rows (or uneven systems of a batch) balance
// themselves. A Hamaker item writes its rows' partial sums to hpart[slice]; the contact items write
// csum. When an item finishes it counts itself in its group's arrival counter; the warp that brings
// the count to the group's item total completes the group's 32 rows in the same launch: it combines
// the Hamaker partials in slice order, adds the contact sums, and integrates in float-float
// (finish_ff_plain). No warp ever waits for another.
//
// The completion writes the next step's float-float positions and velocities to the other buffers
// of the double-buffered state (x32n / v32n), because other warps of the same launch may still
// gather this step's values of the same particles as partners. Each row's arithmetic, its order of
// terms and its combination of slices are those of the two-stream kernels (lg_forces_compact_mixed.cu)
// with the same slice count, so both give the same bits; which warp runs which item does not
// change any result.
//
// The step may also run as two launches side by side (ROLE 1: the contact items, on a second
// stream; ROLE 2: the Hamaker items): each is compiled with only its own item code, so each has its
// own register budget, and they count arrivals in the same group counters, so whichever warp of either
// launch finishes a group's last item completes the group. No completion kernel follows.
//
// Counters: ctr[0] and ctr[1] are the item counters of alternate steps for the one-launch form and
// for ROLE 2, ctr[2] and ctr[3] those of ROLE 1 (a launch uses its pair's [par] and sets its [1 - par]
// to zero for the next step: no warp of the previous step can still touch it); ctr[6 + g] counts the
// finished items of group g and is set back to zero by the warp that completes the group.
#include <algorithm>

#include "lg_mixed_pairs.cuh"

namespace lg {

using namespace mixed;

namespace {

constexpr int kStepWarps = 4;  // warps per block; each takes its own items
// Register budgets the kernel is compiled for, as resident blocks per SM: 4 (127 registers), 5 (96
// registers) and 6 (80 registers) trade spills for resident warps; the autotuner (or
// lg_set_step_shape) picks one. In the two-launch form the budget applies to the contact launch; the
// Hamaker launch always takes 6, which its code alone fits without spills.

// per-warp shared memory: the contact queue or the Hamaker window queue
union StepSmem {
    ContactSmem c;
    HamakerSmem h;
};

// Completion of row i of a group: contact sums (csum), then the Hamaker partials of the group's
// slices in slice order, then the float-float half kicks and drift (or, at a run's last step, the
// FP64 state). The sums were written by other warps of this launch: they are read through L2.
__device__ __forceinline__ void complete_row(const StepArgs &A, const StateView &S, const MixedExtra &MX, int64_t i,
                                             int64_t n) {
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 c0 = A.contacts ? __ldcg(MX.csum + 3 * i) : z4, c1 = A.contacts ? __ldcg(MX.csum + 3 * i + 1) : z4,
                 c2 = A.contacts ? __ldcg(MX.csum + 3 * i + 2) : z4;
    ff a[3] = {{c0.x, c0.y}, {c0.z, c0.w}, {c1.x, c1.y}};
    const ff al[3] = {{c1.z, c1.w}, {c2.x, c2.y}, {c2.z, c2.w}};
    if (A.hamaker) {
        const float4 p0 = __ldcg(A.hpart + 2 * i), p1 = __ldcg(A.hpart + 2 * i + 1);
        ff ah[3] = {{p0.x, p0.y}, {p0.z, p0.w}, {p1.x, p1.y}};
        for (int s = 1; s < A.slices; ++s) {
            const float4 q0 = __ldcg(A.hpart + 2 * ((int64_t)s * n + i)), q1 = __ldcg(A.hpart + 2 * ((int64_t)s * n + i) + 1);
            ff_acc(ah[0], q0.x);
            ff_acc(ah[0], q0.y);
            ff_acc(ah[1], q0.z);
            ff_acc(ah[1], q0.w);
            ff_acc(ah[2], q1.x);
            ff_acc(ah[2], q1.y);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) a[c] = A.contacts ? ff_add(a[c], ah[c]) : ah[c];
    }
    const ff hdt{A.hdt_hi, A.hdt_lo}, dt{A.dt_hi, A.dt_lo};
    if (A.last)
        finish_ff_plain<true>(S, i, n, a, al, hdt, dt, MX, A.x32n, A.v32n);
    else
        finish_ff_plain<false>(S, i, n, a, al, hdt, dt, MX, A.x32n, A.v32n);
}

}  // namespace

template <bool NEAR, bool VERLET, int MINB, int ROLE>
__global__ void __launch_bounds__(kStepWarps * 32, MINB)
    forces_step_mixed(Params P, StateView S, PairView PV, BondView BV, MixedExtra MX, StepArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    StepSmem &W = reinterpret_cast<StepSmem *>(smem_raw)[warp];
    unsigned *const cnt = A.ctr + (ROLE == 1 ? 2 : 0);  // this launch's pair of item counters
    if (blockIdx.x == 0 && threadIdx.x == 0) cnt[1 - A.par] = 0u;  // the next step's counter
    const int nc = A.contacts ? 2 : 0;
    const int per = nc + (A.hamaker ? A.slices : 0);  // items (arrivals) per group
    const int mine = ROLE == 0 ? per : ROLE == 1 ? nc : per - nc;  // of which this launch's
    unsigned *const arrive = A.ctr + 6;
    const int64_t n = P.n;
    // items in turn: pulled from the counter (assign 0 and 2), or every W-th item from the warp's
    // global index on (assign 1, W warps in the launch)
    const int64_t gw = (int64_t)blockIdx.x * kStepWarps + warp, W_all = (int64_t)gridDim.x * kStepWarps;
    for (int64_t next = gw;; next += W_all) {
        unsigned t = (unsigned)next;
        if (A.assign != 1) {
            if (lane == 0) t = atomicAdd(cnt + A.par, 1u);
            t = __shfl_sync(0xffffffffu, t, 0);
        }
        if ((int64_t)t >= A.items) break;
        const int64_t g = (int64_t)t / mine;
        const int k = (int)((int64_t)t - g * mine) + (ROLE == 2 ? nc : 0);
        const int64_t row0 = g * 32;
        bool contact_item_kind;
        if constexpr (ROLE == 1)
            contact_item_kind = true;
        else if constexpr (ROLE == 2)
            contact_item_kind = false;
        else
            contact_item_kind = k < nc;
        if (contact_item_kind) {
            if constexpr (ROLE != 2) contact_rows<NEAR, 2>(P, PV, BV, MX, W.c, row0 + 16 * k, lane);
        } else {
            if constexpr (ROLE != 1) {
                const int sl = k - nc;
                ff acch[3];
                hamaker_rows<VERLET>(P, PV, MX, W.h, row0, sl, A.slices, lane, acch);
                const int64_t i = row0 + lane;
                if (i < n) {
                    float4 *hp = A.hpart + 2 * ((int64_t)sl * n + i);
                    hp[0] = make_float4(acch[0].hi, acch[0].lo, acch[1].hi, acch[1].lo);
                    hp[1] = make_float4(acch[2].hi, acch[2].lo, 0.f, 0.f);
                }
            }
        }
        __syncwarp();
        __threadfence();  // this item's sums are visible device-wide before its arrival is counted
        __syncwarp();
        unsigned old = 0;
        if (lane == 0) old = atomicAdd(arrive + g, 1u);
        old = __shfl_sync(0xffffffffu, old, 0);
        if ((int)old == per - 1) {  // the group's last item: complete its rows
            if (lane == 0) arrive[g] = 0u;
            __threadfence();
            const int64_t i = row0 + lane;
            if (i < n) complete_row(A, S, MX, i, n);
        }
        __syncwarp();
    }
}

namespace {

// blocks of one instantiation that fit on the GPU at once, looked up once per device
template <bool NEAR, bool VERLET, int MINB, int ROLE>
int resident_blocks(size_t smem) {
    static thread_local int cached_device = -1, cached_blocks = 0;
    int dev = 0;
    cudaGetDevice(&dev);
    if (cached_device != dev) {
        int per_sm = 0, sms = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, forces_step_mixed<NEAR, VERLET, MINB, ROLE>,
                                                      kStepWarps * 32, smem);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cached_blocks = std::max(1, per_sm) * std::max(1, sms);
        cached_device = dev;
    }
    return cached_blocks;
}

template <bool NEAR, bool VERLET, int MINB, int ROLE>
void launch_role(const Params &P, const StateView &S, const PairView &PV, const BondView &BV, const MixedExtra &MX,
                 const StepArgs &A, cudaStream_t st) {
    const size_t smem = sizeof(StepSmem) * kStepWarps;
    const int64_t want = (A.items + kStepWarps - 1) / kStepWarps;
    const unsigned blocks =
        (unsigned)std::max<int64_t>(1, std::min<int64_t>(resident_blocks<NEAR, VERLET, MINB, ROLE>(smem), want));
    forces_step_mixed<NEAR, VERLET, MINB, ROLE><<<blocks, kStepWarps * 32, smem, st>>>(P, S, PV, BV, MX, A);
}

template <bool NEAR, bool VERLET, int MINB>
int launch_step(const Params &P, const StateView &S, const PairView &PV, const BondView &BV, const MixedExtra &MX,
                const StepArgs &A, cudaStream_t st, cudaStream_t side, cudaEvent_t fork, cudaEvent_t join) {
    if constexpr (NEAR && VERLET) {  // the two-launch form exists for Verlet rows with contact candidates
        if (A.assign == 2 && A.contacts && A.hamaker && side) {
            // contact items on the side stream beside the Hamaker items on st
            const int64_t groups = (P.n + 31) / 32;
            StepArgs C = A, H = A;
            C.items = groups * 2;
            H.items = groups * A.slices;
            cudaEventRecord(fork, st);
            cudaStreamWaitEvent(side, fork, 0);
            launch_role<NEAR, VERLET, MINB, 1>(P, S, PV, BV, MX, C, side);
            // the Hamaker items need fewer registers: they always run with the smallest budget, which
            // they fit without spills (80 registers, 6 resident blocks per SM)
            launch_role<NEAR, VERLET, 6, 2>(P, S, PV, BV, MX, H, st);
            cudaEventRecord(join, side);
            cudaStreamWaitEvent(st, join, 0);
            return 2;
        }
    }
    launch_role<NEAR, VERLET, MINB, 0>(P, S, PV, BV, MX, A, st);
    return 1;
}

}  // namespace

int launch_step_mixed(const Params &P, const StateView &S, const PairView &PV, const BondView &BV,
                      const MixedExtra &MX, const StepArgs &A, cudaStream_t st, cudaStream_t side, cudaEvent_t fork,
                      cudaEvent_t join) {
    const bool ver = P.pairs == LG_PAIRS_VERLET;
    if (ver && PV.near_len) {  // the common case (Verlet rows with contact candidates): every budget
        if (A.min_blocks == 6) return launch_step<true, true, 6>(P, S, PV, BV, MX, A, st, side, fork, join);
        if (A.min_blocks == 5) return launch_step<true, true, 5>(P, S, PV, BV, MX, A, st, side, fork, join);
        return launch_step<true, true, 4>(P, S, PV, BV, MX, A, st, side, fork, join);
    }
    if (ver) return launch_step<false, true, 4>(P, S, PV, BV, MX, A, st, side, fork, join);
    return launch_step<false, false, 4>(P, S, PV, BV, MX, A, st, side, fork, join);
}

}  // namespace lg
