// lg_reduce.cu -- observables of the system state (test/compute_energy.cpp:7-58 and
// test/mass_distribution.cpp:7-27 of libgran) plus the potential-energy bookkeeping used for
// energy-balance checks, and the state transfers between the caller's [n][3] arrays and the
// device layout. Every sum is taken in a fixed order (per-particle rows reduced by one block, or
// block rows combined by the last block to finish), so results are identical run to run. No
// floating-point atomics.
#include "lg_common.cuh"
#include "lg_kernels.h"

namespace lg {

constexpr int kObs = 20;  // values per particle in the scratch rows

// Pair potential of the Hamaker functors: the exact integral of the force they apply. Full form
// U(h) = -A/6 [2r^2/((4r+h)h) + 2r^2/(2r+h)^2 + ln((4r+h)h/(2r+h)^2)] (its derivative is the
// bracket of hamaker_force.h:36-40), simplified form U(h) = -2Ar/h (force 2Ar/h^2,
// simplified_hamaker_force.h:18-31); linear below the saturation distance h0 (the force stays at
// its value there), and for the limited form shifted to vanish at the cutoff distance.
__device__ __forceinline__ double hamaker_u0(int mode, double A, double r, double h) {
    if (mode == LG_HAMAKER_SIMPLIFIED) return -2.0 * A * r / h;
    return -A / 6.0 *
           (2.0 * r * r / ((4.0 * r + h) * h) + 2.0 * r * r / ((2.0 * r + h) * (2.0 * r + h)) +
            log((4.0 * r + h) * h / ((2.0 * r + h) * (2.0 * r + h))));
}
__device__ __forceinline__ double hamaker_slope(int mode, double A, double r, double h) {
    if (mode == LG_HAMAKER_SIMPLIFIED) return 2.0 * A * r / (h * h);
    const double br = (4.0 * r + 2.0 * h) / (4.0 * r + h) / h - 2.0 / (2.0 * r + h) -
                      4.0 * r * r / ((2.0 * r + h) * (2.0 * r + h) * (2.0 * r + h)) -
                      2.0 * r * r * (4.0 * r + 2.0 * h) / ((4.0 * r + h) * (4.0 * r + h)) / (h * h);
    return -A / 6.0 * br;
}
__device__ __forceinline__ double hamaker_energy(int mode, const lg_hamaker_params &p, double dist) {
    const double r = p.r_part, h = dist - 2.0 * r;
    double u = h < p.h0 ? hamaker_u0(mode, p.A, r, p.h0) + hamaker_slope(mode, p.A, r, p.h0) * (h - p.h0)
                        : hamaker_u0(mode, p.A, r, h);
    if (mode == LG_HAMAKER_LIMITED) {
        const double hc = p.r_cutoff - 2.0 * r;
        u -= hc < p.h0 ? hamaker_u0(mode, p.A, r, p.h0) + hamaker_slope(mode, p.A, r, p.h0) * (hc - p.h0)
                       : hamaker_u0(mode, p.A, r, hc);
    }
    return u;
}

// Per-particle terms. Column layout of a scratch row:
//  0 e_tot  1 m|v|^2  2 I|w|^2  3-5 v  6-8 I w  9-11 x cross m v  12-14 x  15 potential energy
//  16 contacts  17 intact bonds
// Rows of particles row0 .. row0 + count - 1 into out rows 0 .. count - 1.
__global__ void obs_rows(Params P, StateView S, PairView PV, BondView BV, double m, double I, int pairs,
                         double *__restrict__ out, int64_t row0, int64_t count) {
    const int64_t n = P.n;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int64_t i = row0 + t;
    const d3 v = ld4(S.v, i), w = ld4(S.w, i), x = ld4(S.x, i);
    double *o = out + t * kObs;
    o[0] = m * dot(v, v) / 2.0 + I * dot(w, w) / 2.0;
    o[1] = m * dot(v, v);
    o[2] = I * dot(w, w);
    o[3] = v.x; o[4] = v.y; o[5] = v.z;
    d3 Iw = scl(I, w);
    o[6] = Iw.x; o[7] = Iw.y; o[8] = Iw.z;
    d3 L = crs(x, scl(m, v));
    o[9] = L.x; o[10] = L.y; o[11] = L.z;
    o[12] = x.x; o[13] = x.y; o[14] = x.z;
    double pe = 0.0, ncont = 0.0, nbond = 0.0;
    const bool ver = P.pairs == LG_PAIRS_VERLET;
    const int64_t len = !pairs ? 0 : ver ? (int64_t)PV.row_len[i] : n - 1;
    const int64_t xs = PV.cap * n, bs = (int64_t)BV.bcap * n;
    for (int64_t k = 0; k < len; ++k) {
        const int64_t e = k * n + i;
        const int64_t j = ver ? (int64_t)PV.nbr[e] : (k < i ? k : k + 1);
        const uint32_t fl = PV.flags[e];
        const double dist = nrm(sub(x, ld4(S.x, j)));
        double u = 0.0;
        if ((fl & kBonded) && BV.cn) {  // 5-connector model: the connector springs
            const int64_t be = (int64_t)bond_slot_of(fl) * n + i, ej = (int64_t)BV.rev[be] * n + j;
            for (int k = 0; k < 5; ++k) {
                const d3 ci = mk3(BV.cn[(3 * k) * bs + be], BV.cn[(3 * k + 1) * bs + be], BV.cn[(3 * k + 2) * bs + be]);
                const d3 cj = mk3(BV.cn[(3 * k) * bs + ej], BV.cn[(3 * k + 1) * bs + ej], BV.cn[(3 * k + 2) * bs + ej]);
                const double dl = (k < 4 ? 2.0 * P.contact.r_part : 0.0) - nrm(sub(cj, ci));
                u += 0.5 * P.connector.k_d * dl * dl;
            }
            nbond += 1.0;
        } else if (fl & kBonded) {
            const int64_t be = (int64_t)bond_slot_of(fl) * n + i;
            double dl = 2.0 * P.sinter.r_part - dist;
            u += 0.5 * P.sinter.k * dl * dl;
            const bool f = P.springs_ff != 0;
            d3 s0 = mk3(spring_load(BV.xi, spring_at(BV.aos, 0, be, bs), f), spring_load(BV.xi, spring_at(BV.aos, 1, be, bs), f), spring_load(BV.xi, spring_at(BV.aos, 2, be, bs), f));
            d3 s1 = mk3(spring_load(BV.xi, spring_at(BV.aos, 3, be, bs), f), spring_load(BV.xi, spring_at(BV.aos, 4, be, bs), f), spring_load(BV.xi, spring_at(BV.aos, 5, be, bs), f));
            d3 s2 = mk3(spring_load(BV.xi, spring_at(BV.aos, 6, be, bs), f), spring_load(BV.xi, spring_at(BV.aos, 7, be, bs), f), spring_load(BV.xi, spring_at(BV.aos, 8, be, bs), f));
            u += 0.5 * P.sinter.k_t * sqn(s0) + 0.5 * P.sinter.k_r * sqn(s1) + 0.5 * P.sinter.k_o * sqn(s2);
            nbond += 1.0;
        } else if (P.binary_model != LG_BINARY_NONE) {
            double dl = 2.0 * P.contact.r_part - dist;
            if (dl > 0) {
                u += 0.5 * P.contact.k * dl * dl;
                ncont += 1.0;
            }
            if (fl & kXiLive) {
                const bool f = P.springs_ff != 0;
                d3 s0 = mk3(spring_load(PV.xi, spring_at(PV.aos, 0, e, xs), f), spring_load(PV.xi, spring_at(PV.aos, 1, e, xs), f), spring_load(PV.xi, spring_at(PV.aos, 2, e, xs), f));
                d3 s1 = mk3(spring_load(PV.xi, spring_at(PV.aos, 3, e, xs), f), spring_load(PV.xi, spring_at(PV.aos, 4, e, xs), f), spring_load(PV.xi, spring_at(PV.aos, 5, e, xs), f));
                d3 s2 = mk3(spring_load(PV.xi, spring_at(PV.aos, 6, e, xs), f), spring_load(PV.xi, spring_at(PV.aos, 7, e, xs), f), spring_load(PV.xi, spring_at(PV.aos, 8, e, xs), f));
                u += 0.5 * P.contact.k_t * sqn(s0) + 0.5 * P.contact.k_r * sqn(s1) + 0.5 * P.contact.k_o * sqn(s2);
            }
        }
        if (P.hamaker_model == LG_HAMAKER_FULL || P.hamaker_model == LG_HAMAKER_SIMPLIFIED ||
            (P.hamaker_model == LG_HAMAKER_LIMITED && !(dist > P.hamaker.r_cutoff)))
            u += hamaker_energy(P.hamaker_model, P.hamaker, dist);
        pe += 0.5 * u;
    }
    o[15] = pe;
    o[16] = ncont;
    o[17] = nbond;
    o[18] = 0.0;
    o[19] = 0.0;
}

// |x - c|^2 per particle into column 18; c = (column sums 12..14) / n, read from device memory.
// One block of 1024 threads: thread t sums rows t, t + 1024, ... in order, then a fixed tree.
__global__ void __launch_bounds__(1024) obs_reduce(int64_t n, const double *__restrict__ rows, int c0, int c1,
                                                   double *__restrict__ out) {
    __shared__ double s[1024];
    for (int c = c0; c < c1; ++c) {
        double acc = 0.0;
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x) acc += rows[i * kObs + c];
        s[threadIdx.x] = acc;
        __syncthreads();
        for (int o = blockDim.x / 2; o > 0; o >>= 1) {
            if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[c] = s[0];
        __syncthreads();
    }
}

int64_t obs_scratch_doubles(int64_t n) { return n * kObs; }

// Per-particle observables (columns 0..14 of the row layout above, and 18) by a two-level
// fixed-order reduction: every block of 256 particles reduces its terms with a shared-memory tree
// into one row of partial sums, then one block sums the rows in order. Columns 12..14 (sum of x)
// give the centre of mass on the device, which the radius-of-gyration pass reads back.
constexpr int kObsBlock = 256;
constexpr int kObsCols = 16;  // 15 terms + |x - c|^2

// Block sums of C columns in a fixed order; the result row goes to part[blockIdx.x]. FP64 issues
// slowly on this GPU (a warp instruction occupies the SM's FP64 pipe for many cycles), so the warp
// level counts instructions: for C > 2 the warp's C x 32 terms are transposed through shared memory
// and lanes c and 16 + c add the halves of column c in lane order (16 instructions per warp instead of
// a 5-step butterfly per column); for C <= 2, a butterfly. Then thread c < C adds the kObsBlock / 32
// warp sums in warp order.
template <int C>
__device__ __forceinline__ void obs_block_row(double (&t)[C], double *__restrict__ part) {
    __shared__ double ws[kObsBlock / 32][C];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if constexpr (C <= 2) {
#pragma unroll
        for (int c = 0; c < C; ++c) {
            double v = t[c];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) ws[warp][c] = v;
        }
    } else {
        static_assert(C <= 16, "two lanes per column");
        __shared__ double tr[kObsBlock / 32][C][33];
#pragma unroll
        for (int c = 0; c < C; ++c) tr[warp][c][lane] = t[c];
        __syncwarp();
        const int c = lane & 15, h = lane >> 4;
        double r = 0.0;
        if (c < C) {
#pragma unroll
            for (int q = 0; q < 16; ++q) r += tr[warp][c][16 * h + q];
        }
        const double r2 = __shfl_down_sync(0xffffffffu, r, 16);
        if (lane < C) ws[warp][lane] = r + r2;
    }
    __syncthreads();
    if ((int)threadIdx.x < C) {
        double r = 0.0;
#pragma unroll
        for (int q = 0; q < kObsBlock / 32; ++q) r += ws[q][threadIdx.x];
        part[(int64_t)blockIdx.x * kObsCols + threadIdx.x] = r;
    }
}

// The last block of a grid to finish (counted in *ticket, which it resets) sums the nb rows of
// columns c0 .. c0 + C into out[out0 ..]: 16 threads per column take the rows b = g, g + 16, ...
// (g = thread / C), and their 16 partial sums are added in order (short dependent chains: a
// dependent FP64 add takes tens of cycles on this GPU). Returns without waiting on any block.
template <int C>
__device__ __forceinline__ void obs_last_block_combine(int nb, const double *__restrict__ part, int c0, int out0,
                                                       double *__restrict__ out, unsigned *ticket,
                                                       int64_t centre_n = 0) {
    static_assert(16 * C <= kObsBlock, "one thread per (column, group)");
    __shared__ bool last;
    __shared__ double pg[16][C];
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == (unsigned)nb - 1u;
    __syncthreads();
    if (!last) return;
    __threadfence();
    const int c = threadIdx.x % C, g = threadIdx.x / C;
    if (g < 16) {
        double acc = 0.0;
        for (int b = g; b < nb; b += 16) acc += ((volatile const double *)part)[(int64_t)b * kObsCols + c0 + c];
        pg[g][c] = acc;
    }
    __syncthreads();
    if ((int)threadIdx.x < C) {
        double acc = 0.0;
#pragma unroll
        for (int q = 0; q < 16; ++q) acc += pg[q][threadIdx.x];
        out[out0 + threadIdx.x] = acc;
        // with centre_n: the centre of mass (columns 12..14 over n) once, to out[20..22]
        const int col = out0 + (int)threadIdx.x;
        if (centre_n > 0 && col >= 12 && col < 15) out[20 + col - 12] = acc / (double)centre_n;
    }
    if (threadIdx.x == 0) *ticket = 0u;
}

__global__ void __launch_bounds__(kObsBlock) obs_state_terms(int64_t n, const dbl4 *__restrict__ x,
                                                             const dbl4 *__restrict__ v, const dbl4 *__restrict__ w,
                                                             double m, double I, double *__restrict__ part,
                                                             double *__restrict__ out, unsigned *ticket) {
    const int64_t i = blockIdx.x * (int64_t)kObsBlock + threadIdx.x;
    double t[15];
#pragma unroll
    for (int c = 0; c < 15; ++c) t[c] = 0.0;
    if (i < n) {
        const d3 vi = ld4(v, i), wi = ld4(w, i), xi = ld4(x, i);
        t[0] = m * dot(vi, vi) / 2.0 + I * dot(wi, wi) / 2.0;
        t[1] = m * dot(vi, vi);
        t[2] = I * dot(wi, wi);
        t[3] = vi.x; t[4] = vi.y; t[5] = vi.z;
        const d3 Iw = scl(I, wi);
        t[6] = Iw.x; t[7] = Iw.y; t[8] = Iw.z;
        const d3 L = crs(xi, scl(m, vi));
        t[9] = L.x; t[10] = L.y; t[11] = L.z;
        t[12] = xi.x; t[13] = xi.y; t[14] = xi.z;
    }
    obs_block_row<15>(t, part);
    obs_last_block_combine<15>((int)gridDim.x, part, 0, 0, out, ticket, n);
}

__global__ void __launch_bounds__(kObsBlock) obs_state_rg(int64_t n, const dbl4 *__restrict__ x,
                                                          const double *__restrict__ sums, double *__restrict__ part,
                                                          double *__restrict__ out, unsigned *ticket) {
    const int64_t i = blockIdx.x * (int64_t)kObsBlock + threadIdx.x;
    double t[1] = {0.0};
    if (i < n) {
        const d3 q = sub(ld4(x, i), mk3(sums[20], sums[21], sums[22]));  // the centre, sums[12..14] / n
        t[0] = dot(q, q);
    }
    obs_block_row<1>(t, part);
    obs_last_block_combine<1>((int)gridDim.x, part, 0, 18, out, ticket);
}

// Two kernels: the terms (with their sums and the centre of mass, by the last block to finish), then
// |x - c|^2 about that centre (out[18]). out holds at least 23 doubles; ticket: a zeroed device
// counter owned by the caller.
void launch_observables_state(int64_t n, const dbl4 *x, const dbl4 *v, const dbl4 *w, double mass, double inertia,
                              double *scratch, double *out, unsigned *ticket, cudaStream_t st) {
    const int nb = (int)((n + kObsBlock - 1) / kObsBlock);
    obs_state_terms<<<nb, kObsBlock, 0, st>>>(n, x, v, w, mass, inertia, scratch, out, ticket);
    obs_state_rg<<<nb, kObsBlock, 0, st>>>(n, x, out, scratch, out, ticket);
}

void launch_observables_pairs(const Params &P, const StateView &S, const PairView &PV, const BondView &BV, double mass,
                              double inertia, double *scratch, double *out, cudaStream_t st) {
    const int64_t n = P.n;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    obs_rows<<<blocks, 256, 0, st>>>(P, S, PV, BV, mass, inertia, 1, scratch, 0, P.n);
    obs_reduce<<<1, 1024, 0, st>>>(n, scratch, 15, 18, out);
}

// out receives the column sums 0..17 (the pair columns 15..17 are zero unless `pairs`). The caller
// synchronises the stream before reading out (device memory).
void launch_observables(const Params &P, const StateView &S, const PairView &PV, const BondView &BV, double mass,
                        double inertia, double *scratch, double *out, cudaStream_t st, bool pairs) {
    const int64_t n = P.n;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    obs_rows<<<blocks, 256, 0, st>>>(P, S, PV, BV, mass, inertia, pairs ? 1 : 0, scratch, 0, n);
    obs_reduce<<<1, 1024, 0, st>>>(n, scratch, 0, 18, out);
}

void launch_observables_range(const Params &P, const StateView &S, const PairView &PV, const BondView &BV,
                              double mass, double inertia, int64_t row0, int64_t count, double *scratch, double *out,
                              cudaStream_t st) {
    if (count <= 0) return;
    obs_rows<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(P, S, PV, BV, mass, inertia, 1, scratch, row0, count);
    obs_reduce<<<1, 1024, 0, st>>>(count, scratch, 0, 18, out);
}


// One block per system: fixed-order sums of the system's scratch rows (columns 0..17).
__global__ void __launch_bounds__(256) seg_sums(const int64_t *__restrict__ off, const double *__restrict__ rows,
                                                double *__restrict__ out) {
    __shared__ double s[256];
    const int64_t sys = blockIdx.x;
    const int64_t b = off[sys], e = off[sys + 1];
    for (int c = 0; c < 18; ++c) {
        double acc = 0.0;
        for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) acc += rows[i * kObs + c];
        s[threadIdx.x] = acc;
        __syncthreads();
        for (int o = blockDim.x / 2; o > 0; o >>= 1) {
            if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[sys * kObs + c] = s[0];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) seg_rg(const int64_t *__restrict__ off, const dbl4 *__restrict__ x,
                                              const double *__restrict__ centres, double *__restrict__ out) {
    __shared__ double s[256];
    const int64_t sys = blockIdx.x;
    const int64_t b = off[sys], e = off[sys + 1];
    const d3 c = mk3(centres[3 * sys], centres[3 * sys + 1], centres[3 * sys + 2]);
    double acc = 0.0;
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        d3 q = sub(ld4(x, i), c);
        acc += dot(q, q);
    }
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[sys * kObs + 18] = s[0];
}

void launch_segmented_sums(int64_t n_systems, const int64_t *offsets, const double *scratch, double *out,
                           cudaStream_t st) {
    if (n_systems > 0) seg_sums<<<(unsigned)n_systems, 256, 0, st>>>(offsets, scratch, out);
}

void launch_segmented_rg(int64_t n, int64_t n_systems, const int64_t *offsets, const dbl4 *x, const double *centres,
                         double *scratch, double *out, cudaStream_t st) {
    (void)n;
    (void)scratch;
    if (n_systems > 0) seg_rg<<<(unsigned)n_systems, 256, 0, st>>>(offsets, x, centres, out);
}

__global__ void aos_to_dev4(int64_t n, const double *__restrict__ aos, dbl4 *__restrict__ dst) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    st4(dst, i, mk3(aos[3 * i], aos[3 * i + 1], aos[3 * i + 2]));
}

__global__ void dev4_to_aos(int64_t n, const dbl4 *__restrict__ src, double *__restrict__ aos) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const d3 q = ld4(src, i);
    aos[3 * i] = q.x;
    aos[3 * i + 1] = q.y;
    aos[3 * i + 2] = q.z;
}

// The four state fields in one pass. in[f] / out[f]: [n][3] doubles in device memory or in pinned
// host memory the GPU reads and writes directly (x, v, theta, omega; null: field not moved).
// A block moves the 3 x kIoBlock consecutive doubles of its particles of every field through a
// shared-memory tile, so that the accesses to the caller's buffers are consecutive 16-byte words
// (io.wide) all issued before the first one is used: over the host link the transfer is bound by
// the number of requests in flight, not by the per-particle work.
// state_in also refreshes the mixed path's float-float copies (x32 non-null) from the new values,
// and with `uncovered` flags a position further than four times its system's extent from its origin
// (a plain store of 1: the flag may live in mapped host memory, zeroed by the caller).
constexpr int kIoBlock = 128;
constexpr int kIoChunks = (3 * kIoBlock / 2 + kIoBlock - 1) / kIoBlock;  // 16-byte words per thread and field

__device__ __forceinline__ void io_tile_load(const double *__restrict__ src, int64_t d0, int nd, bool wide,
                                             double *__restrict__ tile) {
    if (wide) {
        const double2 *s2 = reinterpret_cast<const double2 *>(src + d0);
        const int nw = nd / 2;
        double2 r[kIoChunks];
#pragma unroll
        for (int u = 0; u < kIoChunks; ++u) {
            const int c = (int)threadIdx.x + u * kIoBlock;
            if (c < nw) r[u] = s2[c];
        }
#pragma unroll
        for (int u = 0; u < kIoChunks; ++u) {
            const int c = (int)threadIdx.x + u * kIoBlock;
            if (c < nw) {
                tile[2 * c] = r[u].x;
                tile[2 * c + 1] = r[u].y;
            }
        }
        if ((nd & 1) && threadIdx.x == 0) tile[nd - 1] = src[d0 + nd - 1];
    } else {
        for (int c = threadIdx.x; c < nd; c += kIoBlock) tile[c] = src[d0 + c];
    }
}

__device__ __forceinline__ void io_tile_store(const double *__restrict__ tile, int64_t d0, int nd, bool wide,
                                              double *__restrict__ dst) {
    if (wide) {
        double2 *d2 = reinterpret_cast<double2 *>(dst + d0);
        const int nw = nd / 2;
#pragma unroll
        for (int u = 0; u < kIoChunks; ++u) {
            const int c = (int)threadIdx.x + u * kIoBlock;
            if (c < nw) d2[c] = make_double2(tile[2 * c], tile[2 * c + 1]);
        }
        if ((nd & 1) && threadIdx.x == 0) dst[d0 + nd - 1] = tile[nd - 1];
    } else {
        for (int c = threadIdx.x; c < nd; c += kIoBlock) dst[d0 + c] = tile[c];
    }
}

__global__ void __launch_bounds__(kIoBlock) state_in(int64_t n, StateIO io, dbl4 *__restrict__ x, dbl4 *__restrict__ v,
                                                     dbl4 *__restrict__ th, dbl4 *__restrict__ w,
                                                     float4 *__restrict__ x32, float4 *__restrict__ v32,
                                                     float4 *__restrict__ s32, double ox, double oy, double oz,
                                                     double oext, const int32_t *__restrict__ agg,
                                                     const dbl4 *__restrict__ orig, int32_t *uncovered) {
    __shared__ double tile[4][3 * kIoBlock];
    const int64_t p0 = (int64_t)blockIdx.x * kIoBlock;
    const int cnt = (int)(n - p0 < kIoBlock ? n - p0 : kIoBlock);
    const int64_t d0 = 3 * p0;
#pragma unroll
    for (int f = 0; f < 4; ++f)
        if (io.in[f]) io_tile_load(io.in[f], d0, 3 * cnt, io.wide != 0, tile[f]);
    __syncthreads();
    const int t = threadIdx.x;
    if (t >= cnt) return;
    const int64_t i = p0 + t;
    dbl4 *dst[4] = {x, v, th, w};
    d3 val[4];
#pragma unroll
    for (int f = 0; f < 4; ++f) {
        if (io.in[f]) {
            val[f] = mk3(tile[f][3 * t], tile[f][3 * t + 1], tile[f][3 * t + 2]);
            st4(dst[f], i, val[f]);
        } else {
            val[f] = ld4(dst[f], i);
        }
    }
    if (!x32 || !(io.in[0] || io.in[1] || io.in[3])) return;
    rel_ff(val[0], ox, oy, oz, agg, orig, i, n, x32);
    state_ff(val[1], val[3], i, n, v32, s32);
    if (uncovered) {
        if (agg) {
            const dbl4 o = orig[agg[i]];
            ox = o.x;
            oy = o.y;
            oz = o.z;
            oext = o.w;
        }
        const double lim = 4.0 * oext;
        const d3 q = val[0];
        if (!(fabs(q.x - ox) <= lim && fabs(q.y - oy) <= lim && fabs(q.z - oz) <= lim)) *(volatile int32_t *)uncovered = 1;
    }
}

__global__ void __launch_bounds__(kIoBlock) state_out(int64_t n, StateIO io, const dbl4 *__restrict__ x,
                                                      const dbl4 *__restrict__ v, const dbl4 *__restrict__ th,
                                                      const dbl4 *__restrict__ w) {
    __shared__ double tile[4][3 * kIoBlock];
    const int64_t p0 = (int64_t)blockIdx.x * kIoBlock;
    const int cnt = (int)(n - p0 < kIoBlock ? n - p0 : kIoBlock);
    const int t = threadIdx.x;
    const dbl4 *src[4] = {x, v, th, w};
    if (t < cnt) {
#pragma unroll
        for (int f = 0; f < 4; ++f)
            if (io.out[f]) {
                const d3 q = ld4(src[f], p0 + t);
                tile[f][3 * t] = q.x;
                tile[f][3 * t + 1] = q.y;
                tile[f][3 * t + 2] = q.z;
            }
    }
    __syncthreads();
#pragma unroll
    for (int f = 0; f < 4; ++f)
        if (io.out[f]) io_tile_store(tile[f], 3 * p0, 3 * cnt, io.wide != 0, io.out[f]);
}

void launch_state_in(int64_t n, const StateIO &io, dbl4 *x, dbl4 *v, dbl4 *th, dbl4 *w, float4 *x32, float4 *v32,
                     float4 *s32, const double *origin, const int32_t *agg, const dbl4 *orig, int32_t *uncovered,
                     cudaStream_t st) {
    if (n > 0)
        state_in<<<(unsigned)((n + kIoBlock - 1) / kIoBlock), kIoBlock, 0, st>>>(
            n, io, x, v, th, w, x32, v32, s32, origin[0], origin[1], origin[2], origin[3], agg, orig, uncovered);
}

void launch_state_out(int64_t n, const StateIO &io, const dbl4 *x, const dbl4 *v, const dbl4 *th, const dbl4 *w,
                      cudaStream_t st) {
    if (n > 0) state_out<<<(unsigned)((n + kIoBlock - 1) / kIoBlock), kIoBlock, 0, st>>>(n, io, x, v, th, w);
}

void launch_aos_to_dev4(int64_t n, const double *aos, dbl4 *dst, cudaStream_t st) {
    if (n > 0) aos_to_dev4<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, aos, dst);
}

void launch_dev4_to_aos(int64_t n, const dbl4 *src, double *aos, cudaStream_t st) {
    if (n > 0) dev4_to_aos<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, src, aos);
}

// ---- serving slots: partner indices of a copied block moved by an offset, positions filled ----
// p[r * pitch + c] += off for r < rows, c < width where the entry is a particle index (>= 0).
__global__ void offset_indices(int32_t *__restrict__ p, int64_t rows, int64_t pitch, int64_t width, int32_t off) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= rows * width) return;
    const int64_t e = (t / width) * pitch + t % width;
    const int32_t v = p[e];
    if (v >= 0) p[e] = v + off;
}

__global__ void fill_dbl4(dbl4 *__restrict__ p, int64_t count, double x, double y, double z) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < count) p[i] = make_double4_32a(x, y, z, 0.0);
}

void launch_offset_indices(int32_t *p, int64_t rows, int64_t pitch, int64_t width, int32_t off, cudaStream_t st) {
    const int64_t total = rows * width;
    if (total <= 0) return;
    offset_indices<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(p, rows, pitch, width, off);
}

void launch_fill_dbl4(dbl4 *p, int64_t count, double x, double y, double z, cudaStream_t st) {
    if (count <= 0) return;
    fill_dbl4<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(p, count, x, y, z);
}

}  // namespace lg
