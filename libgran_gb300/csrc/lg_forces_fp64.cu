// lg_forces_fp64.cu -- FP64 force evaluation, integration and Verlet-list kernels (sm_103a).
//
// Compiled with --fmad=false: a thread that walks its row in ascending j evaluates every pair with
// the same operations, in the same order, as libgran's functors evaluated sequentially on a CPU
// (see lg_common.cuh). One "row group" of T consecutive lanes (T in {1, 2, 4, 8, 16, 32}) owns one
// particle i: lane l handles slots k = l, l + T, ... of row i, and the group then combines its T
// partial sums with a fixed xor-butterfly. T = 1 reproduces the sequential sum bit for bit; larger
// T spreads short, FP64-heavy rows (all-pairs mode on a few hundred particles) over more of the
// GPU's FP64 units. No floating-point atomics are used anywhere: every per-particle sum is owned
// by one row group, so results are deterministic run to run.
#include "lg_compact.cuh"
#include "lg_kernels.h"

namespace lg {

// ------------------------------------------------------------------------------------------------
// Kick + drift (first half of the rotational velocity-Verlet step):
//   v += a*(dt/2); w += al*(dt/2); x += v*dt; th += w*dt
// ------------------------------------------------------------------------------------------------
// With connectors (BV.cn): the drift is sinter_step_handler's increment_x then increment_theta
// (sinter_bridge.h:24-42, 55-75): the particle's connectors move with it by dx, then turn by
// dtheta about its moved centre.
// Drift of particle i with kicked velocities vi, wi (stored by the caller).
// A held increment (LG_HOLD_X, LG_HOLD_THETA in `h`) is skipped together with its connector update.
__device__ __forceinline__ void drift_one(int64_t n, int64_t i, dbl4 *__restrict__ x, dbl4 *__restrict__ th, d3 vi,
                                          d3 wi, double dt, const BondView &BV, uint32_t h) {
    const bool hx = h & LG_HOLD_X, hth = h & LG_HOLD_THETA;
    const d3 dx = scl(dt, vi);
    const d3 xn = hx ? ld4(x, i) : add(ld4(x, i), dx);
    if (!hx) st4(x, i, xn);
    const d3 dth = scl(dt, wi);
    if (!hth) st4(th, i, add(ld4(th, i), dth));
    if (BV.cn && !(hx && hth)) {
        const int64_t bs = (int64_t)BV.bcap * n;
        for (int b = 0; b < BV.bcap; ++b) {
            const int64_t e = (int64_t)b * n + i;
            if (BV.j[e] < 0) continue;
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                double *cx = BV.cn + (3 * k) * bs + e, *cy = BV.cn + (3 * k + 1) * bs + e, *cz = BV.cn + (3 * k + 2) * bs + e;
                d3 c = mk3(*cx, *cy, *cz);
                if (!hx) c = add(c, dx);
                if (!hth) c = add(c, crs(dth, sub(c, xn)));
                *cx = c.x;
                *cy = c.y;
                *cz = c.z;
            }
        }
    }
}

__global__ void kick_drift_fp64(int64_t n, dbl4 *__restrict__ x, dbl4 *__restrict__ v,
                                dbl4 *__restrict__ th, dbl4 *__restrict__ w, const dbl4 *__restrict__ a,
                                const dbl4 *__restrict__ al, double dt, double hdt, BondView BV,
                                const uint8_t *__restrict__ hold) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t h = hold_of(hold, i);
    d3 vi = kick_unless(ld4(v, i), hdt, ld4(a, i), h & LG_HOLD_V);
    d3 wi = kick_unless(ld4(w, i), hdt, ld4(al, i), h & LG_HOLD_OMEGA);
    st4(v, i, vi);
    st4(w, i, wi);
    drift_one(n, i, x, th, vi, wi, dt, BV, h);
}

// Body force LG_BODY_CENTRAL (central_attraction_functor, Custom-unary-force-model.md:108-118):
// a = k_a / mass * (centre - x_i), alpha = 0; kam = k_a / mass (formed on the host, as the
// functor forms it); one centre per system.
__global__ void body_central(int64_t n, const dbl4 *__restrict__ x, const int32_t *__restrict__ agg,
                             const double *__restrict__ centre, double kam, dbl4 *__restrict__ ea,
                             dbl4 *__restrict__ eal) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t q = agg ? (int64_t)agg[i] : 0;
    const d3 c = mk3(centre[3 * q], centre[3 * q + 1], centre[3 * q + 2]);
    st4(ea, i, scl(kam, sub(c, ld4(x, i))));
    st4(eal, i, zero3());
}

// ------------------------------------------------------------------------------------------------
// Pair force kernel
// ------------------------------------------------------------------------------------------------
template <int T>
__device__ __forceinline__ double group_sum(double v) {
#pragma unroll
    for (int o = T / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// The binary functor's value for slot e of row i (P.binary_model != LG_BINARY_NONE); pair state
// (springs, bond state, flags) of slot e is read and written here and nowhere else.
__device__ __forceinline__ void slot_binary_fp64(const Params &P, const StateView &S, const PairView &PV,
                                                 const BondView &BV, int64_t n, int64_t i, int64_t e, int64_t j,
                                                 const d3 xi_, const d3 vi, const d3 wi, d3 &pa, d3 &pal) {
    const int bm = P.binary_model;
    const bool breaking = bm == LG_BINARY_BREAKING_SINTER;
    const uint32_t fl = PV.flags[e];
    const d3 xj = ld4(S.x, j);
    const d3 dx = sub(xi_, xj);
    pa = zero3();
    pal = zero3();
    {
        if ((fl & kBonded) && BV.cn) {  // 5-connector model
            const int64_t be = (int64_t)bond_slot_of(fl) * n + i;
            const d3 vj = ld4(S.v, j), wj = ld4(S.w, j);
            connector_force(P.connector, P.contact.r_part, P.contact.mass, P.contact.inertia, xi_, xj, vi, vj,
                            wi, wj, BV.cn, (int64_t)BV.bcap * n, be, (int64_t)BV.rev[be] * n + j, pa, pal);
        } else if (fl & kBonded) {
            const int b = (int)bond_slot_of(fl);
            const int64_t be = (int64_t)b * n + i;
            const int64_t bs = (int64_t)BV.bcap * n;
            d3 s[3];
#pragma unroll
            for (int q = 0; q < 3; ++q)
                s[q] = mk3(BV.xi[(3 * q) * bs + be], BV.xi[(3 * q + 1) * bs + be], BV.xi[(3 * q + 2) * bs + be]);
            const d3 vj = ld4(S.v, j), wj = ld4(S.w, j);
            bool brk = bond_force(P.sinter, dx, vi, vj, wi, wj, s, breaking, breaking ? BV.strength[be] : 0.0, pa,
                                  pal);
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                BV.xi[(3 * q) * bs + be] = s[q].x;
                BV.xi[(3 * q + 1) * bs + be] = s[q].y;
                BV.xi[(3 * q + 2) * bs + be] = s[q].z;
            }
            if (brk) {
                BV.intact[be] = 0;
                PV.flags[e] = fl & ~(kBonded | (0xffu << 8));
            }
        } else {
            const int64_t xs = PV.cap * n;
            bool touching = false;
            d3 nn = zero3();
            double overlap = 0.0;
            if (!(sqn(dx) > P.contact_skip_d2)) {
                nn = nrmz(dx);
                overlap = 2.0 * P.contact.r_part - dot(dx, nn);
                touching = !(overlap <= 0);
            }
            if (touching) {
                d3 s[3] = {zero3(), zero3(), zero3()};  // springs of a slot that is not live are zero
                if (fl & kXiLive)
#pragma unroll
                    for (int q = 0; q < 3; ++q)
                        s[q] = mk3(PV.xi[(3 * q) * xs + e], PV.xi[(3 * q + 1) * xs + e], PV.xi[(3 * q + 2) * xs + e]);
                const d3 vj = ld4(S.v, j), wj = ld4(S.w, j);
                contact_touching(P.contact, nn, overlap, vi, vj, wi, wj, s, pa, pal);
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    PV.xi[(3 * q) * xs + e] = s[q].x;
                    PV.xi[(3 * q + 1) * xs + e] = s[q].y;
                    PV.xi[(3 * q + 2) * xs + e] = s[q].z;
                }
                if (!(fl & kXiLive)) PV.flags[e] = fl | kXiLive;
            } else if (fl & kXiLive) {  // reset_springs (contact_force.h:69,99-101)
#pragma unroll
                for (int q = 0; q < 9; ++q) PV.xi[q * xs + e] = 0.0;
                PV.flags[e] = fl & ~kXiLive;
            }
        }
    }
}

// The Hamaker term of the pair (i, j) (P.hamaker_model != LG_HAMAKER_NONE).
__device__ __forceinline__ d3 slot_hamaker_fp64(const Params &P, const StateView &S, int64_t j, const d3 xi_) {
    const int hm = P.hamaker_model;
    const d3 xj = ld4(S.x, j);
    const d3 dx = sub(xi_, xj);
    d3 ha = zero3();
    bool on = true;
    if (hm == LG_HAMAKER_LIMITED) on = !(sqn(dx) > P.hamaker_skip_d2) && !(nrm(dx) > P.hamaker.r_cutoff);
    if (on) ha = hamaker_accel(hm, P.hamaker, sub(xj, xi_));
    return ha;
}

// The pair value of a slot: binary + Hamaker as the reference's container adds them.
__device__ __forceinline__ void combine_pair_fp64(bool have_binary, bool have_hamaker, const d3 &pb, const d3 &pbl,
                                                  const d3 &ha, d3 &pa, d3 &pal) {
    pa = pb;
    pal = pbl;
    if (have_hamaker) {
        if (have_binary) {
            pa = add(pa, ha);
            pal = add(pal, zero3());
        } else {
            pa = ha;
            pal = zero3();
        }
    }
}

// One slot of row i: the binary functor's pair value plus the Hamaker term, in that order (the
// reference's container returns binary + hamaker for each pair, operator_overloads.h:16-20).
__device__ __forceinline__ void slot_pair_fp64(const Params &P, const StateView &S, const PairView &PV,
                                               const BondView &BV, int64_t n, int64_t i, int64_t e, int64_t j,
                                               const d3 xi_, const d3 vi, const d3 wi, d3 &pa_out, d3 &pal_out) {
    const bool hb = P.binary_model != LG_BINARY_NONE, hh = P.hamaker_model != LG_HAMAKER_NONE;
    d3 pb = zero3(), pbl = zero3(), ha = zero3();
    if (hb) slot_binary_fp64(P, S, PV, BV, n, i, e, j, xi_, vi, wi, pb, pbl);
    if (hh) ha = slot_hamaker_fp64(P, S, j, xi_);
    combine_pair_fp64(hb, hh, pb, pbl, ha, pa_out, pal_out);
}

template <int T, bool VERLET>
__global__ void __launch_bounds__(256) forces_fp64(Params P, StateView S, PairView PV, BondView BV, double hdt,
                                                   double dt, int move_facets) {
    const int64_t n = P.n;
    const int64_t gid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t i = gid / T;
    const int lane = (int)(gid % T);
    const bool active = i < n;

    if (move_facets && gid == 0) {
        for (int f = 0; f < P.n_facets; ++f)
            for (int q = 0; q < 9; ++q) S.facet_vert_next[9 * f + q] = S.facet_vert[9 * f + q] + P.facets[f].v[q % 3] * dt;
    }

    d3 acc = zero3(), accw = zero3();
    d3 xi_ = zero3(), vi = zero3(), wi = zero3();
    if (active) {
        xi_ = ld4(S.x, i);
        vi = ld4(S.v, i);
        wi = ld4(S.w, i);
        const int64_t len = VERLET ? (int64_t)PV.row_len[i] : n - 1;
        const int64_t stride = n;  // slot k of row i lives at k * n + i
        for (int64_t k = lane; k < len; k += T) {
            const int64_t e = k * stride + i;
            const int64_t j = VERLET ? (int64_t)PV.nbr[e] : (k < i ? k : k + 1);
            d3 pa, pal;
            slot_pair_fp64(P, S, PV, BV, n, i, e, j, xi_, vi, wi, pa, pal);
            acc = add(acc, pa);
            accw = add(accw, pal);
        }
    }
    if (T > 1) {
        acc.x = group_sum<T>(acc.x);
        acc.y = group_sum<T>(acc.y);
        acc.z = group_sum<T>(acc.z);
        accw.x = group_sum<T>(accw.x);
        accw.y = group_sum<T>(accw.y);
        accw.z = group_sum<T>(accw.z);
    }
    if (!active || lane != 0) return;
    compact::finish_row(P, S, i, n, acc, accw, vi, wi, hdt);
}

// ------------------------------------------------------------------------------------------------
// Pair-parallel evaluation for small systems (latency path)
// ------------------------------------------------------------------------------------------------
// A GB300 SM retires few FP64 instructions per clock, so a small system whose rows all sit on one
// or two SMs spends its step waiting on those SMs' FP64 pipes while the rest of the GPU idles. Here
// every slot (i, k) gets its own thread, in one-warp blocks that the block scheduler spreads over
// all SMs; each thread writes its pair value (a, alpha: 6 doubles) to a slot-major scratch array.
// A second kernel then adds each row's values in ascending slot order, exactly as the sequential
// row loop adds them (so results match the T = 1 row kernel bit for bit), runs the facet terms
// and the closing half kick and, when another step follows, the next step's kick and drift.
constexpr int kPairBlock = 32;
constexpr int kFoldBlock = 32;
constexpr int kFoldRows = 5;    // rows per warp of the fold (six lanes each)
constexpr int kFoldAhead = 8;   // slots whose pair terms a lane of the fold loads at once

template <bool VERLET>
__global__ void __launch_bounds__(kPairBlock) forces_pairs_fp64(Params P, StateView S, PairView PV, BondView BV,
                                                                double *__restrict__ pres, int64_t ps, int64_t total) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int64_t n = P.n;
    const int64_t k = t / n, i = t - k * n;  // slot t = k * n + i
    if (VERLET && k >= (int64_t)PV.row_len[i]) return;
    const int64_t j = VERLET ? (int64_t)PV.nbr[t] : (k < i ? k : k + 1);
    d3 pa, pal;
    slot_pair_fp64(P, S, PV, BV, n, i, t, j, ld4(S.x, i), ld4(S.v, i), ld4(S.w, i), pa, pal);
    pres[t] = pa.x;
    pres[ps + t] = pa.y;
    pres[2 * ps + t] = pa.z;
    pres[3 * ps + t] = pal.x;
    pres[4 * ps + t] = pal.y;
    pres[5 * ps + t] = pal.z;
}

// The same slots with the binary functor and the Hamaker term in two warps of one block (warp 0:
// binary, warp 1: Hamaker, 32 slots each): each warp issues only its own part's FP64 instructions,
// which halves the longest instruction sequence a small system waits for. Warp 1 then adds the two
// parts exactly as slot_pair_fp64 does.
template <bool VERLET>
__global__ void __launch_bounds__(2 * kPairBlock) forces_pairs_split_fp64(Params P, StateView S, PairView PV,
                                                                          BondView BV, double *__restrict__ pres,
                                                                          int64_t ps, int64_t total) {
    __shared__ double part[6][kPairBlock];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t t = blockIdx.x * (int64_t)kPairBlock + lane;
    const int64_t n = P.n;
    const int64_t k = t / n, i = t - k * n;  // slot t = k * n + i
    const bool live = t < total && (!VERLET || k < (int64_t)PV.row_len[i]);
    const int64_t j = !live ? 0 : VERLET ? (int64_t)PV.nbr[t] : (k < i ? k : k + 1);
    d3 pb = zero3(), pbl = zero3();
    if (warp == 0) {
        if (live) slot_binary_fp64(P, S, PV, BV, n, i, t, j, ld4(S.x, i), ld4(S.v, i), ld4(S.w, i), pb, pbl);
        part[0][lane] = pb.x;
        part[1][lane] = pb.y;
        part[2][lane] = pb.z;
        part[3][lane] = pbl.x;
        part[4][lane] = pbl.y;
        part[5][lane] = pbl.z;
    }
    d3 ha = zero3();
    if (warp == 1 && live) ha = slot_hamaker_fp64(P, S, j, ld4(S.x, i));
    __syncthreads();
    if (warp != 1 || !live) return;
    pb = mk3(part[0][lane], part[1][lane], part[2][lane]);
    pbl = mk3(part[3][lane], part[4][lane], part[5][lane]);
    d3 pa, pal;
    combine_pair_fp64(true, true, pb, pbl, ha, pa, pal);
    pres[t] = pa.x;
    pres[ps + t] = pa.y;
    pres[2 * ps + t] = pa.z;
    pres[3 * ps + t] = pal.x;
    pres[4 * ps + t] = pal.y;
    pres[5 * ps + t] = pal.z;
}

template <bool VERLET, bool FACETS>
__global__ void __launch_bounds__(kFoldBlock) fold_pairs_fp64(Params P, StateView S, PairView PV, BondView BV,
                                                              const double *__restrict__ pres, int64_t ps, double hdt,
                                                              double dt, int move_facets, int kick) {
    const int64_t n = P.n;
    if (move_facets && blockIdx.x == 0 && threadIdx.x == 0) compact::move_facets(P, S, dt);
    // lane 6 r + c of a warp sums component c (force x, y, z, torque x, y, z) of the warp's row r:
    // each component's terms in slot order, as one dependent chain per lane, so that a warp's FP64
    // instructions each advance six chains of a row instead of one (FP64 issues slowly on this GPU).
    // The loads of kFoldAhead slots are issued before their additions.
    const int lane = threadIdx.x & 31;
    const int64_t wg = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int r = lane / 6, c = lane % 6;
    const int64_t i = wg * kFoldRows + r;
    const bool mine = r < kFoldRows && i < n;
    double sum = 0.0;
    if (mine) {
        const int64_t len = VERLET ? (int64_t)PV.row_len[i] : n - 1;
        const double *col = pres + (int64_t)c * ps + i;
        for (int64_t k = 0; k < len; k += kFoldAhead) {
            double t[kFoldAhead];
#pragma unroll
            for (int u = 0; u < kFoldAhead; ++u) t[u] = k + u < len ? col[(k + u) * n] : 0.0;
#pragma unroll
            for (int u = 0; u < kFoldAhead; ++u)
                if (k + u < len) sum += t[u];  // (adding a padding zero could turn -0 into +0)
        }
    }
    double f[6];
    const int src = r < kFoldRows ? 6 * r : 0;
#pragma unroll
    for (int q = 0; q < 6; ++q) f[q] = __shfl_sync(0xffffffffu, sum, src + q);
    if (!mine || c != 0) return;
    d3 acc = mk3(f[0], f[1], f[2]), accw = mk3(f[3], f[4], f[5]);
    const d3 vi = ld4(S.v, i), wi = ld4(S.w, i);
    compact::finish_row<FACETS>(P, S, i, n, acc, accw, vi, wi, hdt);
    if (kick) {  // the next step's opening half kick and drift, as kick_drift_fp64
        const uint32_t h = hold_of(P.hold, i);
        const d3 v2 = kick_unless(kick_unless(vi, hdt, acc, h & LG_HOLD_V), hdt, acc, h & LG_HOLD_V);
        const d3 w2 = kick_unless(kick_unless(wi, hdt, accw, h & LG_HOLD_OMEGA), hdt, accw, h & LG_HOLD_OMEGA);
        st4(S.v_out, i, v2);
        st4(S.w_out, i, w2);
        drift_one(n, i, S.x, S.th, v2, w2, dt, BV, h);
    }
}

// ------------------------------------------------------------------------------------------------
// Verlet list: bounding box, cell grid, counting sort, row build with spring carry
// ------------------------------------------------------------------------------------------------
// Position used for cell hashing: the particle's own coordinates plus, in a batch, the spatial
// offset of its system (systems of a batch keep their own coordinates; the offsets only keep
// their cells apart).
__device__ __forceinline__ dbl4 hash_pos(const dbl4 *__restrict__ x, BatchView B, int64_t i) {
    dbl4 q = x[i];
    if (B.agg) {
        const dbl4 o = B.hoff[B.agg[i]];
        q.x += o.x;
        q.y += o.y;
        q.z += o.z;
    }
    return q;
}

__global__ void bbox_partial(int64_t n, const dbl4 *__restrict__ x, BatchView B, double *__restrict__ part) {
    __shared__ double s[6][256];
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        dbl4 q = hash_pos(x, B, i);
        lo[0] = fmin(lo[0], q.x); lo[1] = fmin(lo[1], q.y); lo[2] = fmin(lo[2], q.z);
        hi[0] = fmax(hi[0], q.x); hi[1] = fmax(hi[1], q.y); hi[2] = fmax(hi[2], q.z);
    }
    for (int c = 0; c < 3; ++c) {
        s[c][threadIdx.x] = lo[c];
        s[3 + c][threadIdx.x] = hi[c];
    }
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int c = 0; c < 3; ++c) {
                s[c][threadIdx.x] = fmin(s[c][threadIdx.x], s[c][threadIdx.x + o]);
                s[3 + c][threadIdx.x] = fmax(s[3 + c][threadIdx.x], s[3 + c][threadIdx.x + o]);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int c = 0; c < 6; ++c) part[6 * blockIdx.x + c] = s[c][0];
}

// One block: combine the block partials and size the grid (cells of edge >= r_verlet; the edge
// grows by 1.25 until the grid has at most max_cells cells). Also fixes the FP32 accept / reject
// bounds of the squared list radius for positions stored relative to the grid origin.
__global__ void __launch_bounds__(256) grid_setup(int nparts, const double *__restrict__ part, double rv, double rnear,
                                                  int64_t max_cells, GridDev *g) {
    __shared__ double s[6][256];
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int b = threadIdx.x; b < nparts; b += blockDim.x)
        for (int c = 0; c < 3; ++c) {
            lo[c] = fmin(lo[c], part[6 * b + c]);
            hi[c] = fmax(hi[c], part[6 * b + 3 + c]);
        }
    for (int c = 0; c < 3; ++c) {
        s[c][threadIdx.x] = lo[c];
        s[3 + c][threadIdx.x] = hi[c];
    }
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
            for (int c = 0; c < 3; ++c) {
                s[c][threadIdx.x] = fmin(s[c][threadIdx.x], s[c][threadIdx.x + o]);
                s[3 + c][threadIdx.x] = fmax(s[3 + c][threadIdx.x], s[3 + c][threadIdx.x + o]);
            }
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    for (int c = 0; c < 3; ++c) {
        lo[c] = s[c][0];
        hi[c] = s[3 + c][0];
    }
    double edge = rv;
    int64_t dim[3];
    for (int it = 0; it < 4096; ++it) {
        for (int c = 0; c < 3; ++c) {
            double m = floor((hi[c] - lo[c]) / edge) + 1.0;
            dim[c] = m < 1.0 ? 1 : (int64_t)m;
        }
        double cells = (double)dim[0] * (double)dim[1] * (double)dim[2];
        if (cells <= (double)max_cells) break;
        edge *= 1.25;
    }
    double cells = (double)dim[0] * (double)dim[1] * (double)dim[2];
    if (!(cells <= (double)max_cells) || !(edge < 1e300)) {  // non-finite positions: one cell
        dim[0] = dim[1] = dim[2] = 1;
        edge = 1e300;
    }
    double span = 0.0;
    for (int c = 0; c < 3; ++c) {
        g->lo[c] = lo[c];
        g->dim[c] = dim[c];
        span = fmax(span, hi[c] - lo[c]);
    }
    g->edge = edge;
    g->ncell = dim[0] * dim[1] * dim[2];
    // FP32 coordinates relative to lo carry an error below span * 2^-24 each; bound |d| by 2 such
    // errors per component and the squared radius by a further relative 1e-6
    const double del = 4.0 * span * 5.9604644775390625e-8 + 1e-300;
    const double lo_r = rv - 2.0 * del, hi_r = rv + 2.0 * del;
    g->rv2_lo = lo_r > 0 ? (float)(lo_r * lo_r * (1.0 - 1e-6)) : 0.0f;
    g->rv2_hi = (float)(hi_r * hi_r * (1.0 + 1e-6));
    g->rn2_hi = rnear > 0 ? (float)((rnear + 2.0 * del) * (rnear + 2.0 * del) * (1.0 + 1e-6)) : -1.0f;
}

__device__ __forceinline__ int64_t cell_coord(double q, double lo, double edge, int64_t dim) {
    int64_t k = (int64_t)floor((q - lo) / edge);
    return k < 0 ? 0 : (k >= dim ? dim - 1 : k);
}

__global__ void cell_count(int64_t n, const dbl4 *__restrict__ x, BatchView B, const GridDev *__restrict__ g,
                           int32_t *__restrict__ cell_of, int32_t *__restrict__ count, float4 *__restrict__ x32) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (inactive_of(B.hold, i)) {  // in no cell: never a candidate of any row
        cell_of[i] = -1;
        return;
    }
    dbl4 q = hash_pos(x, B, i);
    int64_t cx = cell_coord(q.x, g->lo[0], g->edge, g->dim[0]);
    int64_t cy = cell_coord(q.y, g->lo[1], g->edge, g->dim[1]);
    int64_t cz = cell_coord(q.z, g->lo[2], g->edge, g->dim[2]);
    int32_t c = (int32_t)((cz * g->dim[1] + cy) * g->dim[0] + cx);
    cell_of[i] = c;
    x32[i] = make_float4((float)(q.x - g->lo[0]), (float)(q.y - g->lo[1]), (float)(q.z - g->lo[2]), 0.0f);
    atomicAdd(&count[c], 1);
}

// Exclusive scan of the cell counts (start of every cell in the sorted list), in three passes over
// tiles of kScanTile cells: the tiles' totals, an exclusive scan of the totals (one block), and each
// tile's own scan plus its offset. Loads and stores go through shared memory so that they coalesce.
constexpr int kScanThreads = 256;
constexpr int kScanPer = 16;
constexpr int kScanTile = kScanThreads * kScanPer;  // 4096 cells

__global__ void __launch_bounds__(kScanThreads) scan_tile_sums(const GridDev *__restrict__ g,
                                                                const int32_t *__restrict__ count,
                                                                int32_t *__restrict__ tile_sum) {
    const int64_t nc = g->ncell, base = (int64_t)blockIdx.x * kScanTile;
    if (base >= nc) return;
    __shared__ int32_t red[kScanThreads];
    int32_t v = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
        const int64_t c = base + (int64_t)k * kScanThreads + threadIdx.x;
        if (c < nc) v += count[c];
    }
    red[threadIdx.x] = v;
    __syncthreads();
    for (int o = kScanThreads / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = red[0];
}

// Exclusive scan of the tile totals in place (one block of 1024 threads, any number of tiles).
__global__ void __launch_bounds__(1024) scan_tile_offsets(const GridDev *__restrict__ g, int32_t *__restrict__ tile_sum) {
    __shared__ int32_t part[1024];
    const int64_t tiles = (g->ncell + kScanTile - 1) / kScanTile;
    const int t = threadIdx.x;
    const int64_t per = (tiles + 1023) / 1024;
    const int64_t b = (int64_t)t * per, e = b + per < tiles ? b + per : tiles;
    int32_t sum = 0;
    for (int64_t q = b; q < e; ++q) sum += tile_sum[q];
    part[t] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const int32_t v = t >= o ? part[t - o] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int32_t run = part[t] - sum;
    for (int64_t q = b; q < e; ++q) {
        const int32_t c = tile_sum[q];
        tile_sum[q] = run;
        run += c;
    }
}

__global__ void __launch_bounds__(kScanThreads) scan_tiles(const GridDev *__restrict__ g, const int32_t *__restrict__ count,
                                                            const int32_t *__restrict__ tile_off,
                                                            int32_t *__restrict__ start) {
    const int64_t nc = g->ncell, base = (int64_t)blockIdx.x * kScanTile;
    if (base >= nc) return;
    __shared__ int32_t cell[kScanTile];
    __shared__ int32_t part[kScanThreads];
    const int t = threadIdx.x;
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {  // coalesced load of the tile
        const int64_t c = base + (int64_t)k * kScanThreads + t;
        cell[k * kScanThreads + t] = c < nc ? count[c] : 0;
    }
    __syncthreads();
    int32_t sum = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) sum += cell[t * kScanPer + k];
    part[t] = sum;
    __syncthreads();
    for (int o = 1; o < kScanThreads; o <<= 1) {
        const int32_t v = t >= o ? part[t - o] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int32_t run = tile_off[blockIdx.x] + part[t] - sum;
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {  // exclusive starts of this thread's cells, in place
        const int32_t c = cell[t * kScanPer + k];
        cell[t * kScanPer + k] = run;
        run += c;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {  // coalesced store
        const int64_t c = base + (int64_t)k * kScanThreads + t;
        if (c < nc) start[c] = cell[k * kScanThreads + t];
    }
}

__global__ void cell_scatter(int64_t n, const int32_t *__restrict__ cell_of, const int32_t *__restrict__ start,
                             int32_t *__restrict__ fill, int32_t *__restrict__ sorted) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t c = cell_of[i];
    if (c < 0) return;  // inactive
    int32_t p = atomicAdd(&fill[c], 1);
    sorted[start[c] + p] = (int32_t)i;
}

constexpr int kBuildRows = 32;   // rows per block
constexpr int kBuildWarps = 16;  // warps per block; warp w builds rows w, w + 16
constexpr int kBuildBatches = 3; // candidate batches of 32 whose loads are in flight together
constexpr uint32_t kNearBit = 0x80000000u;  // a listed partner within the contact-candidate radius

// Shared-memory layout of build_rows for row capacity cap and bond capacity bcap: four 32-row
// tiles (partner, flags, old slot, near partner) with an odd row stride, then per warp the unsorted
// candidates, the old row, the old row's flags and the row's bond partners, then the near-slot tile
// (bytes).
__host__ __device__ inline int64_t build_tile_stride(int64_t cap) { return cap | 1; }
__host__ __device__ inline int64_t build_warp_ints(int64_t cap, int64_t bcap) { return 3 * cap + bcap; }
__host__ __device__ inline size_t build_smem_bytes(int64_t cap, int64_t bcap) {
    return sizeof(int32_t) * (size_t)(4 * kBuildRows * build_tile_stride(cap) + kBuildWarps * build_warp_ints(cap, bcap)) +
           (size_t)(kBuildRows * build_tile_stride(cap));
}

// Build rows row0 .. row0 + 31: every j != i with squared centre distance < r_verlet^2 (the FP64
// test; an FP32 filter accepts or rejects the clear cases), ascending j, carrying the springs (and
// live flag) of pairs that were already listed, and marking intact bonds.
// One warp per row: the 27 neighbour cells are 9 runs of consecutive cells (x fastest), i.e. 9
// contiguous ranges of the cell-sorted particle list, walked as one list; the lanes take
// kBuildBatches x 32 candidates at a time (all their index and position loads issued before the
// first test, so that one round trip serves them all) and append the accepted ones (ballot +
// popc), each with its contact-candidate test in bit 31. The old row (partners and flags) and the
// row's bonds are requested before the candidate loop, so their round trip overlaps it. The row is
// then ordered by partner (j is unique, so the append order does not matter), the old row is
// searched by bisection for spring carry-over, and the finished rows of the block are written
// slot-major so that the 32 rows' slot k go out as one coalesced store.
__global__ void __launch_bounds__(kBuildRows * kBuildWarps, 2) build_rows(
    int64_t n, const dbl4 *__restrict__ x, BatchView B, const float4 *__restrict__ x32, const GridDev *__restrict__ g,
    const int32_t *__restrict__ cstart, const int32_t *__restrict__ ccount, const int32_t *__restrict__ sorted,
    const int32_t *__restrict__ cell_of, double rv2, PairView oldv, PairView newv, BondView BV, int32_t *err,
    int32_t *max_row) {
    extern __shared__ int32_t sm[];
    __shared__ int32_t rlen[kBuildRows];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    const int64_t cap = newv.cap, ts = build_tile_stride(cap);
    const int bcap = BV.bcap;
    int32_t *tj = sm;
    uint32_t *tf = reinterpret_cast<uint32_t *>(tj + kBuildRows * ts);
    int32_t *tp = reinterpret_cast<int32_t *>(tf + kBuildRows * ts);
    int32_t *tnj = tp + kBuildRows * ts;
    int32_t *wraw = tnj + kBuildRows * ts + (int64_t)warp * build_warp_ints(cap, bcap);
    int32_t *wold = wraw + cap;
    uint32_t *wofl = reinterpret_cast<uint32_t *>(wold + cap);
    int32_t *wbond = reinterpret_cast<int32_t *>(wofl + cap);
    uint8_t *tnk = reinterpret_cast<uint8_t *>(tnj + kBuildRows * ts + kBuildWarps * build_warp_ints(cap, bcap));
    __shared__ int32_t rnear[kBuildRows];
    const bool near_lists = newv.near_len != nullptr;
    const float rn2 = g->rn2_hi;
    const int64_t row0 = (int64_t)blockIdx.x * kBuildRows;
    const float rlo = g->rv2_lo, rhi = g->rv2_hi;
    const int64_t dim0 = g->dim[0], dim1 = g->dim[1], dim2 = g->dim[2];

    for (int r = warp; r < kBuildRows; r += kBuildWarps) {
        const int64_t i = row0 + r;
        if (i >= n || inactive_of(B.hold, i)) {  // an inactive particle's row is empty
            if (lane == 0) rlen[r] = rnear[r] = 0;
            continue;
        }
        // requested now, used after the candidate loop: the first 32 slots of the old row (partner
        // and flags; every slot below the capacity is allocated, so the loads need not wait for the
        // old length) and the first 32 bond slots
        const bool have_old = oldv.row_len != nullptr;
        const int32_t olen_raw = have_old ? oldv.row_len[i] : 0;
        int32_t onb0 = -1, bj0 = -1;
        uint32_t ofl0 = 0;
        uint8_t bok0 = 0;
        if (have_old && lane < oldv.cap) {
            onb0 = oldv.nbr[(int64_t)lane * n + i];
            ofl0 = oldv.flags[(int64_t)lane * n + i];
        }
        if (lane < bcap) {
            bj0 = BV.j[(int64_t)lane * n + i];
            bok0 = BV.intact[(int64_t)lane * n + i];
        }
        const float4 fi = x32[i];
        const dbl4 xd = x[i];
        const d3 xi_ = mk3(xd.x, xd.y, xd.z);
        const int32_t ai = B.agg ? B.agg[i] : 0;
        // the row's cell as cell_count placed it (integer decode: an FP64 division here would be a
        // full-warp FP64 instruction per row)
        const int32_t ci = cell_of[i];
        const int32_t d0 = (int32_t)dim0, d1 = (int32_t)dim1;
        const int64_t cx = ci % d0, cy = (ci / d0) % d1, cz = ci / (d0 * d1);
        const int64_t x0 = cx > 0 ? cx - 1 : 0, x1 = cx + 1 < dim0 ? cx + 1 : dim0 - 1;
        // the 9 runs of cells (z, y fixed; x0..x1) are 9 contiguous ranges of the sorted list; lane
        // r < 9 looks up range r, and the ranges are walked as one virtual list of `total`
        // candidates, kBuildBatches x 32 per iteration
        int32_t rb = 0, rl = 0;
        if (lane < 9) {
            const int64_t z = cz - 1 + lane / 3, y = cy - 1 + lane % 3;
            if (z >= 0 && z < dim2 && y >= 0 && y < dim1) {
                const int64_t c0 = (z * dim1 + y) * dim0 + x0, c1 = (z * dim1 + y) * dim0 + x1;
                rb = cstart[c0];
                rl = cstart[c1] + ccount[c1] - rb;
            }
        }
        int32_t incl = rl;  // inclusive prefix sum of the range lengths over lanes 0..8
#pragma unroll
        for (int o = 1; o < 16; o <<= 1) {
            const int32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int32_t total = __shfl_sync(0xffffffffu, incl, 8);
        // the non-empty ranges, compacted: lane c < m holds the c-th one's begin in the sorted list
        // (rbc) and its first virtual index (exc), which increase strictly with c
        const uint32_t nem = __ballot_sync(0xffffffffu, lane < 9 && rl > 0);
        const int m = __popc(nem);
        int src = 0;  // the range whose rank among the non-empty ones is this lane
#pragma unroll
        for (int r = 0; r < 9; ++r)
            if (((nem >> r) & 1u) && __popc(nem & ((1u << r) - 1u)) == lane) src = r;
        const int32_t rbc = __shfl_sync(0xffffffffu, rb, src), exc = __shfl_sync(0xffffffffu, incl - rl, src);
        const uint32_t upto = lane == 31 ? 0xffffffffu : ((2u << lane) - 1u);
        // candidate of virtual index tb + lane (-1 past the end): the lane's range is the last one
        // starting at or before its index; ranges starting inside the batch are found with one OR
        // over the lanes that hold them
        auto fetch_batch = [&](int32_t tb) -> int32_t {
            const int32_t L = exc - tb;  // lane of the batch at which range `lane` starts
            const uint32_t starts = __reduce_or_sync(0xffffffffu, (lane < m && L > 0 && L < 32) ? (1u << L) : 0u);
            const int before = __popc(__ballot_sync(0xffffffffu, lane < m && L <= 0));
            const int q = before - 1 + __popc(starts & upto);
            const int qs = q < 0 ? 0 : q;
            const int32_t rbq = __shfl_sync(0xffffffffu, rbc, qs), exq = __shfl_sync(0xffffffffu, exc, qs);
            const int32_t t = tb + lane;
            return t < total ? sorted[rbq + (t - exq)] : -1;
        };
        int32_t cnt = 0;
        for (int32_t t0 = 0; t0 < total; t0 += 32 * kBuildBatches) {
            int32_t jb[kBuildBatches];
            float4 fb[kBuildBatches];
            bool same[kBuildBatches];
#pragma unroll
            for (int u = 0; u < kBuildBatches; ++u) jb[u] = fetch_batch(t0 + 32 * u);
#pragma unroll
            for (int u = 0; u < kBuildBatches; ++u) {
                fb[u] = fi;
                same[u] = true;
                if (jb[u] >= 0) {
                    fb[u] = x32[jb[u]];
                    if (B.agg) same[u] = B.agg[jb[u]] == ai;  // pairs never cross systems
                }
            }
#pragma unroll
            for (int u = 0; u < kBuildBatches; ++u) {
                const int32_t j = jb[u];
                bool in = false, near_c = false;
                if (j >= 0 && j != (int32_t)i && same[u]) {
                    const float ex = fi.x - fb[u].x, ey = fi.y - fb[u].y, ez = fi.z - fb[u].z;
                    const float d2f = fmaf(ez, ez, fmaf(ey, ey, ex * ex));
                    near_c = d2f <= rn2;
                    if (d2f < rlo)
                        in = true;
                    else if (!(d2f > rhi))
                        in = sqn(sub(xi_, ld4(x, j))) < rv2;
                }
                const uint32_t bal = __ballot_sync(0xffffffffu, in);
                if (in) {  // the partner, with its contact-candidate test in bit 31
                    const int32_t pos = cnt + __popc(bal & lt);
                    if (pos < cap) wraw[pos] = (int32_t)((uint32_t)j | (near_c ? kNearBit : 0u));
                }
                cnt += __popc(bal);
            }
        }
        if (lane == 0) atomicMax(max_row, cnt);
        if (cnt > cap) {
            if (lane == 0) set_error(err, LG_DEVERR_LIST_OVERFLOW);
            cnt = (int32_t)cap;
        }
        int32_t olen = olen_raw;
        if (olen > oldv.cap) olen = (int32_t)oldv.cap;  // both buffers share one capacity
        if (lane < olen) {
            wold[lane] = onb0;
            wofl[lane] = ofl0;
        }
        for (int32_t p = lane + 32; p < olen; p += 32) {
            wold[p] = oldv.nbr[(int64_t)p * n + i];
            wofl[p] = oldv.flags[(int64_t)p * n + i];
        }
        int32_t intact = 0;
        for (int b = lane; b < bcap; b += 32) {
            int32_t bj = bj0;
            bool ok = bj0 >= 0 && bok0;
            if (b >= 32) {
                const int64_t be = (int64_t)b * n + i;
                bj = BV.j[be];
                ok = bj >= 0 && BV.intact[be];
            }
            wbond[b] = ok ? bj : -1;
            intact += ok ? 1 : 0;
        }
        __syncwarp();
        // order the row by partner (compared without the candidate bit, which travels to tf until
        // the slot's flags replace it): up to 32 partners by a bitonic network across the lanes (15
        // compare-exchange steps, padding sorts last), more by a rank sort (the partners are distinct,
        // so each one's rank is its slot)
        if (cnt <= 32) {
            uint32_t w = lane < cnt ? (uint32_t)wraw[lane] : 0xffffffffu;
#pragma unroll
            for (int kk = 2; kk <= 32; kk <<= 1)
#pragma unroll
                for (int jj = kk >> 1; jj > 0; jj >>= 1) {
                    const uint32_t o = __shfl_xor_sync(0xffffffffu, w, jj);
                    const bool keep_min = ((lane & jj) == 0) == ((lane & kk) == 0);
                    const bool w_less = (w & ~kNearBit) < (o & ~kNearBit);
                    w = keep_min == w_less ? w : o;
                }
            if (lane < cnt) {
                tj[r * ts + lane] = (int32_t)(w & ~kNearBit);
                tf[r * ts + lane] = w & kNearBit;
            }
        } else {
            for (int32_t a = lane; a < cnt; a += 32) {
                const uint32_t w = (uint32_t)wraw[a];
                const int32_t v = (int32_t)(w & ~kNearBit);
                int32_t rank = 0;
                for (int32_t t = 0; t < cnt; ++t) rank += (wraw[t] & (int32_t)~kNearBit) < v ? 1 : 0;
                tj[r * ts + rank] = v;
                tf[r * ts + rank] = w & kNearBit;
            }
        }
        __syncwarp();
        int32_t found = 0, nnear = 0;
        for (int32_t kb = 0; kb < cnt; kb += 32) {  // warp-uniform trip count (ballots inside)
            const int32_t k = kb + lane;
            const bool slot_ok = k < cnt;
            const int32_t j = slot_ok ? tj[r * ts + k] : 0;
            const bool near_c = slot_ok && tf[r * ts + k] != 0u;
            int32_t lo = 0, hi = olen;
            while (lo < hi) {
                const int32_t mid = (lo + hi) >> 1;
                if (wold[mid] < j)
                    lo = mid + 1;
                else
                    hi = mid;
            }
            uint32_t fl = 0;
            int32_t po = -1;
            if (slot_ok && lo < olen && wold[lo] == j && (wofl[lo] & kXiLive)) {
                fl |= kXiLive;
                po = lo;
            }
            if (slot_ok)
                for (int b = 0; b < bcap; ++b)
                    if (wbond[b] == j) {
                        fl |= kBonded | ((uint32_t)b << 8);
                        ++found;
                        break;
                    }
            bool is_near = false;
            if (near_lists && slot_ok) {
                is_near = (fl & kBonded) || near_c;
                if (!is_near) {  // apart: its springs reset, so they are not carried
                    fl &= ~kXiLive;
                    po = -1;
                }
            }
            if (near_lists) {
                const uint32_t bal = __ballot_sync(0xffffffffu, is_near);
                if (is_near) {
                    const int32_t m = nnear + __popc(bal & lt);
                    tnj[r * ts + m] = j;
                    tnk[r * ts + m] = (uint8_t)k;
                }
                nnear += __popc(bal);
            }
            if (slot_ok) {
                tf[r * ts + k] = fl;
                tp[r * ts + k] = po;
            }
        }
        found = __reduce_add_sync(0xffffffffu, found);
        intact = __reduce_add_sync(0xffffffffu, intact);
        if (lane == 0) {
            if (intact != found) set_error(err, LG_DEVERR_BOND_LOST);
            rlen[r] = cnt;
            rnear[r] = nnear;
        }
        __syncwarp();
    }
    __syncthreads();

    // slot-major write-out: lane l owns row row0 + l, warp w writes slots w, w + 8, ...
    const int64_t il = row0 + lane;
    const int32_t len = il < n ? rlen[lane] : 0;
    if (warp == 0 && il < n) newv.row_len[il] = len;
    const int32_t kmax = (int32_t)__reduce_max_sync(0xffffffffu, (unsigned)len);
    const int64_t oxs = oldv.cap * n, nxs = newv.cap * n;
    if (near_lists) {
        const int32_t nl = il < n ? rnear[lane] : 0;
        if (warp == 0 && il < n) newv.near_len[il] = nl;
        const int32_t mmax = (int32_t)__reduce_max_sync(0xffffffffu, (unsigned)nl);
        for (int32_t m = warp; m < mmax; m += kBuildWarps) {
            if (m >= nl) continue;
            newv.near_j[(int64_t)m * n + il] = tnj[lane * ts + m];
            newv.near_k[(int64_t)m * n + il] = tnk[lane * ts + m];
        }
    }
    for (int32_t k = warp; k < kmax; k += kBuildWarps) {
        if (k >= len) continue;
        const int64_t e = (int64_t)k * n + il;
        newv.nbr[e] = tj[lane * ts + k];
        newv.flags[e] = tf[lane * ts + k];
        const int32_t po = tp[lane * ts + k];
        if (po >= 0) {
            const int64_t oe = (int64_t)po * n + il;
#pragma unroll
            for (int q = 0; q < 9; ++q) newv.xi[spring_at(newv.aos, q, e, nxs)] = oldv.xi[spring_at(oldv.aos, q, oe, oxs)];
        }
    }
}

// ------------------------------------------------------------------------------------------------
// Host-side launchers
// ------------------------------------------------------------------------------------------------
template <int T, bool VERLET>
static void launch_forces_t(const Params &P, const StateView &S, const PairView &PV, const BondView &BV, double hdt,
                            double dt, int move_facets, cudaStream_t st) {
    const int threads = 256;
    const int64_t total = P.n * T;
    const int64_t blocks = (total + threads - 1) / threads;
    forces_fp64<T, VERLET><<<(unsigned)(blocks > 0 ? blocks : 1), threads, 0, st>>>(P, S, PV, BV, hdt, dt, move_facets);
}

void launch_forces_fp64(int T, const Params &P, const StateView &S, const PairView &PV, const BondView &BV, double hdt,
                        double dt, int move_facets, cudaStream_t st) {
    const bool ver = P.pairs == LG_PAIRS_VERLET;
#define LG_CASE(TT)                                                                \
    case TT:                                                                       \
        if (ver)                                                                   \
            launch_forces_t<TT, true>(P, S, PV, BV, hdt, dt, move_facets, st);     \
        else                                                                       \
            launch_forces_t<TT, false>(P, S, PV, BV, hdt, dt, move_facets, st);    \
        break;
    switch (T) {
        LG_CASE(1)
        LG_CASE(2)
        LG_CASE(4)
        LG_CASE(8)
        LG_CASE(16)
        LG_CASE(32)
        default:
            launch_forces_t<1, false>(P, S, PV, BV, hdt, dt, move_facets, st);
    }
#undef LG_CASE
}

int launch_forces_pairs_fp64(const Params &P, const StateView &S, const PairView &PV, const BondView &BV,
                             double *pres, double hdt, double dt, int move_facets, bool kick, cudaStream_t st) {
    const int64_t n = P.n;
    const bool verlet = P.pairs == LG_PAIRS_VERLET;
    const int64_t ps = (int64_t)PV.cap * n;
    const int64_t total = (verlet ? (int64_t)PV.cap : n - 1) * n;
    if (total > 0) {
        const int64_t blocks = (total + kPairBlock - 1) / kPairBlock;
        const bool split = P.binary_model != LG_BINARY_NONE && P.hamaker_model != LG_HAMAKER_NONE;
        if (split && verlet)
            forces_pairs_split_fp64<true><<<(unsigned)blocks, 2 * kPairBlock, 0, st>>>(P, S, PV, BV, pres, ps, total);
        else if (split)
            forces_pairs_split_fp64<false><<<(unsigned)blocks, 2 * kPairBlock, 0, st>>>(P, S, PV, BV, pres, ps, total);
        else if (verlet)
            forces_pairs_fp64<true><<<(unsigned)blocks, kPairBlock, 0, st>>>(P, S, PV, BV, pres, ps, total);
        else
            forces_pairs_fp64<false><<<(unsigned)blocks, kPairBlock, 0, st>>>(P, S, PV, BV, pres, ps, total);
    }
    const unsigned fb = (unsigned)((n + kFoldRows - 1) / kFoldRows);  // one warp per kFoldRows rows
    const int kk = kick ? 1 : 0;
    const bool unary = P.n_facets > 0 || P.ext_a;
    if (verlet) {
        if (unary)
            fold_pairs_fp64<true, true><<<fb, kFoldBlock, 0, st>>>(P, S, PV, BV, pres, ps, hdt, dt, move_facets, kk);
        else
            fold_pairs_fp64<true, false><<<fb, kFoldBlock, 0, st>>>(P, S, PV, BV, pres, ps, hdt, dt, move_facets, kk);
    } else {
        if (unary)
            fold_pairs_fp64<false, true><<<fb, kFoldBlock, 0, st>>>(P, S, PV, BV, pres, ps, hdt, dt, move_facets, kk);
        else
            fold_pairs_fp64<false, false><<<fb, kFoldBlock, 0, st>>>(P, S, PV, BV, pres, ps, hdt, dt, move_facets, kk);
    }
    return total > 0 ? 2 : 1;
}

void launch_body_central(int64_t n, const dbl4 *x, const int32_t *agg, const double *centre, double kam, dbl4 *ea,
                         dbl4 *eal, cudaStream_t st) {
    const int threads = 64;
    const int64_t blocks = (n + threads - 1) / threads;
    if (blocks == 0) return;
    body_central<<<(unsigned)blocks, threads, 0, st>>>(n, x, agg, centre, kam, ea, eal);
}

void launch_kick_drift_fp64(int64_t n, dbl4 *x, dbl4 *v, dbl4 *th, dbl4 *w, const dbl4 *a,
                            const dbl4 *al, double dt, double hdt, const BondView &BV, const uint8_t *hold,
                            cudaStream_t st) {
    const int threads = 64;  // small blocks: all SMs get work at moderate n
    int64_t blocks = (n + threads - 1) / threads;
    if (blocks == 0) return;
    kick_drift_fp64<<<(unsigned)blocks, threads, 0, st>>>(n, x, v, th, w, a, al, dt, hdt, BV, hold);
}

void launch_list_build(int64_t n, const dbl4 *x, BatchView B, double rv, double r_near, int64_t max_cells,
                       ListScratch &ls, PairView oldv, PairView newv, BondView BV, int32_t *err, cudaStream_t st) {
    const int nparts = ls.nparts;
    bbox_partial<<<nparts, 256, 0, st>>>(n, x, B, ls.part);
    grid_setup<<<1, 256, 0, st>>>(nparts, ls.part, rv, newv.near_len ? r_near : 0.0, max_cells, ls.grid);
    cudaMemsetAsync(ls.count, 0, sizeof(int32_t) * (size_t)max_cells, st);
    cudaMemsetAsync(ls.fill, 0, sizeof(int32_t) * (size_t)max_cells, st);
    const int threads = 256;
    unsigned blocks = (unsigned)((n + threads - 1) / threads);
    cell_count<<<blocks, threads, 0, st>>>(n, x, B, ls.grid, ls.cell_of, ls.count, ls.x32);
    const unsigned tiles = (unsigned)((max_cells + kScanTile - 1) / kScanTile);
    scan_tile_sums<<<tiles, kScanThreads, 0, st>>>(ls.grid, ls.count, ls.tile);
    scan_tile_offsets<<<1, 1024, 0, st>>>(ls.grid, ls.tile);
    scan_tiles<<<tiles, kScanThreads, 0, st>>>(ls.grid, ls.count, ls.tile, ls.start);
    cell_scatter<<<blocks, threads, 0, st>>>(n, ls.cell_of, ls.start, ls.fill, ls.sorted);
    const unsigned b2 = (unsigned)((n + kBuildRows - 1) / kBuildRows);
    const size_t smem = build_smem_bytes(newv.cap, BV.bcap);
    static thread_local int attr_device = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (attr_device != dev) {  // room for the largest capacities (rows and bonds of up to 255 slots)
        cudaFuncSetAttribute(build_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)build_smem_bytes(255, 255));
        attr_device = dev;
    }
    build_rows<<<b2, kBuildRows * kBuildWarps, smem, st>>>(n, x, B, ls.x32, ls.grid, ls.start, ls.count, ls.sorted, ls.cell_of,
                                                           rv * rv, oldv, newv, BV, err, ls.max_row);
}

}  // namespace lg
