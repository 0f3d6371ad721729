// lg_engine.cpp -- host side of the C ABI (include/libgran_gb300.h): handle lifetime, bond and
// connector set-up, state transfer, the step loop (CUDA graphs per rebuild period, the choice of
// force kernel and the autotuner), Verlet-list management, body forces, hooks and hold masks,
// snapshots and read-back.
//
// Built with -ffp-contract=off: the few host computations that feed the kernels (bond detection,
// facet area and normal) use the reference's arithmetic exactly.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "lg_engine_internal.h"
#include "lg_kernels.h"

using namespace lg;

// ------------------------------------------------------------------------------------------------
// Errors
// ------------------------------------------------------------------------------------------------
static thread_local std::string g_last_error;

int lg_fail(int code, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define LG_CUDA(call)                                                                                     \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) return lg_fail(LG_E_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                              __FILE__, __LINE__);                                        \
    } while (0)

extern "C" const char *lg_version(void) { return "libgran_gb300 0.1 sm_103a"; }
extern "C" const char *lg_last_error(void) { return g_last_error.c_str(); }

extern "C" int lg_device_count(int *count) {
    if (!count) return lg_fail(LG_E_INVALID, "lg_device_count: null pointer");
    int c = 0;
    cudaError_t e = cudaGetDeviceCount(&c);
    if (e != cudaSuccess) {
        *count = 0;
        cudaGetLastError();
        return LG_OK;
    }
    *count = c;
    return LG_OK;
}

// ------------------------------------------------------------------------------------------------
// Host vector helpers (reference evaluation order)
// ------------------------------------------------------------------------------------------------
static inline d3 hld(const double *p, int64_t i) { return mk3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }

// ------------------------------------------------------------------------------------------------
// Bond detection: the reference's double loop over i < j (alt_sinter_bridge.h:67-89,
// alt_breaking_sinter_bridge.h:65-76) tests |(|x_i - x_j| - 2r)| < critical_separation in
// lexicographic (i, j) order. Candidates are gathered through a cell grid and then processed in
// that same order; the cycle test "i and j already connected" is answered by a union-find, which
// gives the same decisions as the reference's subset relabelling.
// ------------------------------------------------------------------------------------------------
static int64_t uf_find(std::vector<int64_t> &p, int64_t a) {
    while (p[a] != a) {
        p[a] = p[p[a]];
        a = p[a];
    }
    return a;
}

int lg_detect_bonds(const double *x0, int64_t n, double r, double dc, bool cycle_free,
                    std::vector<std::pair<int32_t, int32_t>> &bonds, bool inclusive = false) {
    // the 5-connector model bonds at |g| <= dc (sinter_bridge.h:156), the alt models at |g| < dc
    auto bonded = [dc, inclusive](double g) { return inclusive ? !(std::fabs(g) > dc) : std::fabs(g) < dc; };
    bonds.clear();
    if (n < 2) return LG_OK;
    const double reach = 2.0 * r + dc;
    std::vector<std::pair<int32_t, int32_t>> cand;
    if (n <= 2048) {
        for (int64_t i = 0; i + 1 < n; ++i)
            for (int64_t j = i + 1; j < n; ++j) {
                double g = nrm(sub(hld(x0, i), hld(x0, j))) - 2.0 * r;
                if (bonded(g)) cand.emplace_back((int32_t)i, (int32_t)j);
            }
    } else {
        double lo[3] = {1e300, 1e300, 1e300};
        for (int64_t i = 0; i < n; ++i)
            for (int c = 0; c < 3; ++c) lo[c] = std::min(lo[c], x0[3 * i + c]);
        auto key = [&](int64_t a, int64_t b, int64_t c) { return (a * 2097152 + b) * 2097152 + c; };
        std::unordered_map<int64_t, std::vector<int32_t>> grid;
        grid.reserve((size_t)n);
        std::vector<int64_t> cc(3 * (size_t)n);
        for (int64_t i = 0; i < n; ++i) {
            for (int c = 0; c < 3; ++c) cc[3 * i + c] = (int64_t)std::floor((x0[3 * i + c] - lo[c]) / reach);
            grid[key(cc[3 * i], cc[3 * i + 1], cc[3 * i + 2])].push_back((int32_t)i);
        }
        for (int64_t i = 0; i < n; ++i) {
            for (int64_t dz = -1; dz <= 1; ++dz)
                for (int64_t dy = -1; dy <= 1; ++dy)
                    for (int64_t dx = -1; dx <= 1; ++dx) {
                        auto it = grid.find(key(cc[3 * i] + dx, cc[3 * i + 1] + dy, cc[3 * i + 2] + dz));
                        if (it == grid.end()) continue;
                        for (int32_t j : it->second) {
                            if (j <= i) continue;
                            double g = nrm(sub(hld(x0, i), hld(x0, j))) - 2.0 * r;
                            if (bonded(g)) cand.emplace_back((int32_t)i, j);
                        }
                    }
        }
        std::sort(cand.begin(), cand.end());
    }
    std::vector<int64_t> parent((size_t)n);
    for (int64_t i = 0; i < n; ++i) parent[i] = i;
    for (auto &pr : cand) {
        if (cycle_free) {
            int64_t a = uf_find(parent, pr.first), b = uf_find(parent, pr.second);
            if (a == b) continue;  // "preventing neck insertion to avoid a cycle"
            parent[b] = a;
        }
        bonds.push_back(pr);
    }
    return LG_OK;
}

// ------------------------------------------------------------------------------------------------
// Seeded synthetic aggregates (random sequential attachment)
// ------------------------------------------------------------------------------------------------
struct SplitMix {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }
    d3 unit() {
        for (;;) {
            double a = 2.0 * uniform() - 1.0, b = 2.0 * uniform() - 1.0, c = 2.0 * uniform() - 1.0;
            double s2 = (a * a + b * b) + c * c;
            if (s2 > 1e-6 && s2 <= 1.0) {
                double s = std::sqrt(s2);
                return mk3(a / s, b / s, c / s);
            }
        }
    }
};

// Each new sphere touches a uniformly chosen existing sphere in a uniformly random direction and is
// rejected when it overlaps any other sphere by more than 1e-12 r.
extern "C" int lg_generate_rsa_aggregate(uint64_t seed, int64_t n, double r, double *x) {
    if (n < 1 || !x || !(r > 0)) return lg_fail(LG_E_INVALID, "lg_generate_rsa_aggregate: bad arguments");
    SplitMix rng{seed};
    const double edge = 2.0 * r;
    const double lim = 2.0 * r - 1e-12 * r;
    const double lim2 = lim * lim;
    auto key = [](int64_t a, int64_t b, int64_t c) {
        return ((a + 1048576) * 2097152 + (b + 1048576)) * 2097152 + (c + 1048576);
    };
    std::unordered_map<int64_t, std::vector<int32_t>> grid;
    grid.reserve((size_t)n * 2);
    auto cell = [&](d3 p, int64_t *c) {
        c[0] = (int64_t)std::floor(p.x / edge);
        c[1] = (int64_t)std::floor(p.y / edge);
        c[2] = (int64_t)std::floor(p.z / edge);
    };
    x[0] = x[1] = x[2] = 0.0;
    int64_t c0[3];
    cell(mk3(0, 0, 0), c0);
    grid[key(c0[0], c0[1], c0[2])].push_back(0);
    for (int64_t k = 1; k < n; ++k) {
        for (int attempt = 0;; ++attempt) {
            if (attempt > 100000) return lg_fail(LG_E_STATE, "lg_generate_rsa_aggregate: no free site found");
            int64_t p = (int64_t)(rng.uniform() * (double)k);
            if (p >= k) p = k - 1;
            d3 dir = rng.unit();
            d3 c = add(hld(x, p), scl(2.0 * r, dir));
            int64_t cc[3];
            cell(c, cc);
            bool ok = true;
            for (int64_t dz = -1; dz <= 1 && ok; ++dz)
                for (int64_t dy = -1; dy <= 1 && ok; ++dy)
                    for (int64_t dx = -1; dx <= 1 && ok; ++dx) {
                        auto it = grid.find(key(cc[0] + dx, cc[1] + dy, cc[2] + dz));
                        if (it == grid.end()) continue;
                        for (int32_t q : it->second) {
                            if (q == p) continue;
                            if (sqn(sub(c, hld(x, q))) < lim2) {
                                ok = false;
                                break;
                            }
                        }
                    }
            if (!ok) continue;
            x[3 * k] = c.x;
            x[3 * k + 1] = c.y;
            x[3 * k + 2] = c.z;
            grid[key(cc[0], cc[1], cc[2])].push_back((int32_t)k);
            break;
        }
    }
    return LG_OK;
}

// Uniform random velocity components in [-vmax, vmax].
extern "C" int lg_generate_velocities(uint64_t seed, int64_t n, double vmax, double *v) {
    if (n < 0 || !v) return lg_fail(LG_E_INVALID, "lg_generate_velocities: bad arguments");
    SplitMix rng{seed ^ 0x5DEECE66Dull};
    for (int64_t q = 0; q < 3 * n; ++q) v[q] = (2.0 * rng.uniform() - 1.0) * vmax;
    return LG_OK;
}

// ------------------------------------------------------------------------------------------------
// Handle
// ------------------------------------------------------------------------------------------------
template <typename T>
static int dalloc(T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)p, sizeof(T) * count);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return lg_fail(LG_E_NOMEM, "cudaMalloc of %zu bytes failed: %s", sizeof(T) * count, cudaGetErrorString(e));
    }
    return LG_OK;
}

#define LG_TRY(expr)              \
    do {                          \
        int rc_ = (expr);         \
        if (rc_ != LG_OK) return rc_; \
    } while (0)

static void to_dev4(const double *aos, int64_t n, std::vector<dbl4> &tmp) {
    tmp.resize((size_t)n);
    for (int64_t i = 0; i < n; ++i) tmp[i] = make_double4_32a(aos[3 * i], aos[3 * i + 1], aos[3 * i + 2], 0.0);
}

static int upload4(dbl4 *dst, const double *aos, int64_t n, cudaStream_t st) {
    std::vector<dbl4> tmp;
    to_dev4(aos, n, tmp);
    LG_CUDA(cudaMemcpyAsync(dst, tmp.data(), sizeof(dbl4) * (size_t)n, cudaMemcpyHostToDevice, st));
    LG_CUDA(cudaStreamSynchronize(st));
    return LG_OK;
}

// Origin of one system's float-float positions (mixed precision): the centroid; out[3] receives
// the largest coordinate offset from it (at least 8 particle radii), which bounds the FP32
// rounding of the high parts.
static void origin_of(const double *x, int64_t b, int64_t e, double r_max, double out[4]) {
    for (int k = 0; k < 3; ++k) {
        double sum = 0.0;
        for (int64_t i = b; i < e; ++i) sum += x[3 * i + k];
        out[k] = e > b ? sum / (double)(e - b) : 0.0;
    }
    double ext = 8.0 * r_max;
    for (int64_t i = b; i < e; ++i)
        for (int k = 0; k < 3; ++k) ext = std::max(ext, std::fabs(x[3 * i + k] - out[k]));
    out[3] = ext;
}

// FP32 culling radii of the mixed kernels: the interaction radii with a relative margin of 2e-3
// (FP32 rounding of the squared distance) plus the rounding of two high parts (each within
// 2^-24 of the offset, taken with a fourfold allowance for the system spreading out).
static void set_cull_radii(lg_system *s) {
    const double m = 2.0 * 4.0 * s->ext_max * 5.9604644775390625e-8;
    auto sq = [&](double r) { return (float)((r * 1.002 + m) * (r * 1.002 + m)); };
    s->mx.near2 = sq(s->cull_near);
    s->mx.contact2f = sq(s->cull_contact);
}

static int set_mixed_origins(lg_system *s, const double *x) {
    origin_of(x, 0, s->P.n, s->r_max, s->origin);
    s->mx.ox = s->origin[0];
    s->mx.oy = s->origin[1];
    s->mx.oz = s->origin[2];
    s->mx.agg = s->d_agg;
    s->mx.orig = s->d_orig;
    s->ext_max = s->origin[3];
    if (s->n_systems > 0) {
        s->h_orig.assign((size_t)s->n_systems, make_double4_32a(0.0, 0.0, 0.0, 0.0));
        s->ext_max = 0.0;
        for (int64_t q = 0; q < s->n_systems; ++q) {
            double o[4];
            origin_of(x, s->sys_off[q], s->sys_off[q + 1], s->r_max, o);
            s->h_orig[(size_t)q] = make_double4_32a(o[0], o[1], o[2], o[3]);
            s->ext_max = std::max(s->ext_max, o[3]);
        }
        LG_CUDA(cudaMemcpyAsync(s->d_orig, s->h_orig.data(), sizeof(dbl4) * s->h_orig.size(), cudaMemcpyHostToDevice,
                                s->stream));
        LG_CUDA(cudaStreamSynchronize(s->stream));
    }
    return LG_OK;
}

// lg_get / lg_set of the accelerations: the caller's [n][3] array moves in one copy to device scratch
// (the observables scratch, n * 20 doubles, ordered with every other use on the handle's stream) and
// a kernel converts it to or from the padded device layout. (The state fields go through
// state_upload / state_download.)
static int upload_staged(lg_system *s, dbl4 *dst, const double *aos) {
    const int64_t n = s->P.n;
    LG_CUDA(cudaMemcpyAsync(s->obs_scratch, aos, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, s->stream));
    launch_aos_to_dev4(n, s->obs_scratch, dst, s->stream);
    s->launches += 1;
    LG_CUDA(cudaGetLastError());
    LG_CUDA(cudaStreamSynchronize(s->stream));  // the caller may reuse its buffer on return
    return LG_OK;
}

static int download_staged(lg_system *s, const dbl4 *src, double *aos) {
    const int64_t n = s->P.n;
    launch_dev4_to_aos(n, src, s->obs_scratch, s->stream);
    s->launches += 1;
    LG_CUDA(cudaGetLastError());
    LG_CUDA(cudaMemcpyAsync(aos, s->obs_scratch, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToHost, s->stream));
    LG_CUDA(cudaStreamSynchronize(s->stream));
    return LG_OK;
}

void lg_system::drop_graphs() {
    for (auto &g : graphs) cudaGraphExecDestroy(g.exec);
    graphs.clear();
}

void lg_system::release() {
    if (device >= 0) cudaSetDevice(device);
    drop_graphs();
    if (h_pin) {
        if (pooled) std::free(h_pin);
        else cudaFreeHost(h_pin);
    }
    h_pin = nullptr;
    for (void *p : allocations) {
        if (pooled && stream) cudaFreeAsync(p, stream);  // in stream order, after the handle's work
        else cudaFree(p);
    }
    allocations.clear();
    if (stream) cudaStreamDestroy(stream);
    if (side) cudaStreamDestroy(side);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (fork_ev) cudaEventDestroy(fork_ev);
    if (join_ev) cudaEventDestroy(join_ev);
    side = nullptr;
    fork_ev = join_ev = nullptr;
    for (cudaEvent_t e : tev) cudaEventDestroy(e);
    tev.clear();
    stream = nullptr;
}

template <typename U>
int lg_system::alloc(U **p, size_t count) {
    if (pooled && stream) {
        *p = nullptr;
        cudaError_t e = cudaMallocAsync((void **)p, sizeof(U) * std::max<size_t>(count, 1), stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);  // usable from any stream on return
        if (e != cudaSuccess) {
            cudaGetLastError();
            return lg_fail(LG_E_NOMEM, "cudaMallocAsync of %zu bytes failed: %s", sizeof(U) * count, cudaGetErrorString(e));
        }
    } else {
        LG_TRY(dalloc(p, count));
    }
    allocations.push_back((void *)*p);
    return LG_OK;
}

// Pair slots up to which an FP64 system keeps the pair-parallel kernel's scratch (48 bytes a slot),
// and up to which the automatic choice takes that kernel. Measured on GB300 (sinter + limited
// Hamaker, FP64, graph-replayed steps): it leads the row-group and compacted kernels from 19
// particles (37 vs 96 us a step) up to 8000 particles in Verlet mode (295 vs 313 us); the compacted
// kernel keeps the large systems, where full warps and no divergence decide.
constexpr int64_t kPairsMaxSlots = (int64_t)1 << 21;
constexpr int64_t kPairsAutoSlots = (int64_t)1 << 19;

static int choose_kernel(const lg_system *s, int requested) {
    if (requested == LG_FORCE_KERNEL_ROWGROUP || requested == LG_FORCE_KERNEL_COMPACT) return requested;
    if (requested == LG_FORCE_KERNEL_PERSISTENT) return s->precision == LG_PRECISION_MIXED ? requested : -1;
    if (requested == LG_FORCE_KERNEL_FP64_FAST) return s->precision == LG_PRECISION_FP64 ? requested : -1;
    if (requested == LG_FORCE_KERNEL_PAIRS) return s->pres ? requested : -1;
    const int64_t n = s->P.n;
    // mixed precision: the compacted kernels at every size (their float-float completion and fused
    // runs of steps also make small systems fastest: 19 particles 13.7 against 36.9 us a step, 1000
    // particles 15.4 against 47.7 us, on GB300 with the row-group kernel)
    if (s->precision == LG_PRECISION_MIXED) return LG_FORCE_KERNEL_COMPACT;
    if (s->pres && (int64_t)s->pv[0].cap * n <= kPairsAutoSlots) return LG_FORCE_KERNEL_PAIRS;
    if (s->P.pairs == LG_PAIRS_VERLET ? n >= 1024 : n >= 4096) return LG_FORCE_KERNEL_COMPACT;
    return LG_FORCE_KERNEL_ROWGROUP;
}

static int choose_threads_per_row(const lg_system *s) {
    const int64_t n = s->P.n;
    const int64_t want = 152 * 1024;
    int T = 1;
    while (T < 32 && n * T < want) T *= 2;
    const int64_t len = s->P.pairs == LG_PAIRS_VERLET ? 32 : n - 1;
    while (T > 1 && T * 2 > len) T /= 2;
    return T;
}

static int rebuild_list(lg_system *s) {
    PairView &oldv = s->pv[s->pcur];
    PairView &newv = s->pv[1 - s->pcur];
    PairView o = oldv;
    if (!s->list_built) o.row_len = nullptr;
    BatchView B{s->d_agg, s->d_hoff, s->P.hold};
    launch_list_build(s->P.n, s->x, B, s->P.r_verlet, s->r_near, s->max_cells, s->ls, o, newv, s->bv, s->err,
                      s->stream);
    s->launches += 9;
    s->pcur = 1 - s->pcur;
    s->list_built = true;
    LG_CUDA(cudaGetLastError());
    return LG_OK;
}

// The current buffers of the double-buffered float-float state (mixed precision).
static void set_ff_buffers(lg_system *s) {
    if (!s->x32buf) return;
    const int64_t n = s->P.n;
    s->x32 = s->x32buf + 2 * n * s->ffcur;
    s->v32 = s->v32buf + 3 * n * s->ffcur;
    s->mx.x32 = s->x32;
    s->mx.v32 = s->v32;
}

// Counters and Hamaker partial sums of the persistent step kernel (allocated when it is chosen).
static int ensure_step_buffers(lg_system *s) {
    if (s->step_ctr) return LG_OK;
    const int64_t n = s->P.n;
    const int64_t groups = (n + 31) / 32;
    const int sl = mixed_hamaker_slices(n);
    LG_TRY(s->alloc(&s->step_ctr, (size_t)(6 + groups)));
    LG_CUDA(cudaMemset(s->step_ctr, 0, sizeof(unsigned) * (size_t)(6 + groups)));
    LG_TRY(s->alloc(&s->hpart, 2 * (size_t)4 * (size_t)n));
    s->step_slices = sl;
    s->fstep = 0;
    return LG_OK;
}

static StateView state_view(lg_system *s, bool half_step_inputs) {
    StateView S{};
    S.x = s->x;
    S.th = s->th;
    S.v = s->v[s->vcur];
    S.w = s->w[s->vcur];
    S.a = s->a;
    S.al = s->al;
    S.v_out = s->v[1 - s->vcur];
    S.w_out = s->w[1 - s->vcur];
    S.sxi = s->sxi;
    S.facet_vert = s->fv[s->fcur];
    S.facet_vert_next = s->fv[1 - s->fcur];
    S.err = s->err;
    (void)half_step_inputs;
    return S;
}

static int launch_forces(lg_system *s, double hdt, double dt, int move_facets, bool fuse_kick = false,
                         bool prev_fused = false) {
    StateView S = state_view(s, true);
    cudaEvent_t stop_ev = nullptr;
    if (s->timing) {
        if (s->tev_used + 2 > s->tev.size()) {
            for (int q = 0; q < 64; ++q) {
                cudaEvent_t e;
                LG_CUDA(cudaEventCreate(&e));
                s->tev.push_back(e);
            }
        }
        LG_CUDA(cudaEventRecord(s->tev[s->tev_used], s->stream));
        stop_ev = s->tev[s->tev_used + 1];
        s->tev_used += 2;
    }
    const bool compact = s->kernel == LG_FORCE_KERNEL_COMPACT;
    int kernels = 1;
    if (s->body.model == LG_BODY_CENTRAL) {
        launch_body_central(s->P.n, s->x, s->n_systems > 0 ? s->d_agg : nullptr, s->d_centre, s->body.k_a / s->body.mass,
                            s->ext_a, s->ext_al, s->stream);
        s->launches += 1;
    } else if (s->hook) {
        lg_unary_hook_args ha{};
        ha.n = s->P.n;
        ha.x = (const double *)s->x;
        ha.v = (const double *)S.v;
        ha.theta = (const double *)s->th;
        ha.omega = (const double *)S.w;
        ha.a_out = (double *)s->ext_a;
        ha.alpha_out = (double *)s->ext_al;
        ha.system_of = s->n_systems > 0 ? s->d_agg : nullptr;
        ha.dt = dt;
        ha.stream = (void *)s->stream;
        const int hr = s->hook(&ha, s->hook_user);
        if (hr != 0) return lg_fail(LG_E_STATE, "unary hook returned %d", hr);
    }
    const bool persistent = s->kernel == LG_FORCE_KERNEL_PERSISTENT;
    // (all pairs take the compacted kernels: their contact rows use a warp per row there)
    if (s->precision == LG_PRECISION_MIXED && persistent && s->step_ctr && (fuse_kick || prev_fused) &&
        s->P.n_facets == 0 && !s->P.ext_a && !s->P.hold && s->s32 && s->P.pairs == LG_PAIRS_VERLET) {
        // one persistent launch: contacts, Hamaker and the float-float completion of this step
        const int64_t n = s->P.n;
        const PairView &pv = s->pv[s->pcur];
        StepArgs A{};
        const int nf = 1 - s->ffcur;
        A.x32n = s->x32buf + 2 * n * nf;
        A.v32n = s->v32buf + 3 * n * nf;
        A.hpart = s->hpart;
        A.ctr = s->step_ctr;
        A.par = (int)(s->fstep & 1);
        A.slices = s->step_slices;
        A.contacts = s->P.binary_model != LG_BINARY_NONE ? 1 : 0;
        A.hamaker = s->P.hamaker_model != LG_HAMAKER_NONE ? 1 : 0;
        A.last = fuse_kick ? 0 : 1;
        A.assign = s->step_assign;
        A.min_blocks = s->step_min_blocks;
        A.items = ((n + 31) / 32) * (2 * A.contacts + A.slices * A.hamaker);
        A.hdt_hi = (float)hdt;
        A.hdt_lo = (float)(hdt - (double)A.hdt_hi);
        A.dt_hi = (float)dt;
        A.dt_lo = (float)(dt - (double)A.dt_hi);
        MixedExtra MX = s->mx;
        MX.x64 = prev_fused ? nullptr : s->x;  // FP64 positions are current unless the last step ran in float-float
        kernels = launch_step_mixed(s->P, S, pv, s->bv, MX, A, s->stream, s->side, s->fork_ev, s->join_ev);
        s->fstep++;
        if (fuse_kick) {  // the next step reads the buffers this one wrote
            s->ffcur = nf;
            set_ff_buffers(s);
        }
    } else if (s->precision == LG_PRECISION_MIXED) {
        if (compact || persistent)
            kernels = launch_forces_compact_mixed(s->P, S, s->pv[s->pcur], s->bv, hdt, dt, move_facets, fuse_kick,
                                                  prev_fused, s->mx, s->stream, s->side, s->fork_ev, s->join_ev,
                                                  s->ham_slices, s->contact_lanes);
        else
            launch_forces_mixed(s->T, s->P, S, s->pv[s->pcur], s->bv, hdt, dt, move_facets, s->mx, s->stream);
    } else {
        if (s->kernel == LG_FORCE_KERNEL_PAIRS)
            kernels = launch_forces_pairs_fp64(s->P, S, s->pv[s->pcur], s->bv, s->pres, hdt, dt, move_facets,
                                               fuse_kick, s->stream);
        else if (compact || s->kernel == LG_FORCE_KERNEL_FP64_FAST)
            launch_forces_compact_fp64(s->P, S, s->pv[s->pcur], s->bv, hdt, dt, move_facets, s->stream,
                                       s->kernel == LG_FORCE_KERNEL_FP64_FAST);
        else
            launch_forces_fp64(s->T, s->P, S, s->pv[s->pcur], s->bv, hdt, dt, move_facets, s->stream);
    }
    s->launches += kernels;
    LG_CUDA(cudaGetLastError());
    if (stop_ev) LG_CUDA(cudaEventRecord(stop_ev, s->stream));
    return LG_OK;
}

// One velocity-Verlet step. `fuse_next`: the caller runs another step right after this one with no
// list rebuild in between; the mixed compacted path then folds that step's opening half kick and
// drift into this step's completion kernel (same operations, one pass over the state less).
static int step_once(lg_system *s, double dt, int64_t rebuild_every, bool fuse_next) {
    if (s->P.pairs == LG_PAIRS_VERLET && rebuild_every > 0 && (s->step_index % rebuild_every) == 0)
        LG_TRY(rebuild_list(s));
    const double hdt = dt / 2.0;
    const bool prev_fused = s->kick_done;
    if (!s->kick_done) {
        if (s->precision == LG_PRECISION_MIXED)
            launch_kick_drift_mixed(s->P.n, s->x, s->v[s->vcur], s->th, s->w[s->vcur], s->a, s->al, dt, hdt,
                                    s->origin, s->d_agg, s->d_orig, s->x32, s->v32, s->s32, s->P.hold, s->stream);
        else
            launch_kick_drift_fp64(s->P.n, s->x, s->v[s->vcur], s->th, s->w[s->vcur], s->a, s->al, dt, hdt, s->bv, s->P.hold,
                                   s->stream);
        s->launches += 1;
    }
    const int mv = (s->facet_auto_move && s->P.n_facets > 0) ? 1 : 0;
    const bool fuse = fuse_next && ((s->precision == LG_PRECISION_MIXED && (s->kernel == LG_FORCE_KERNEL_COMPACT ||
                                                                            s->kernel == LG_FORCE_KERNEL_PERSISTENT)) ||
                                    (s->precision == LG_PRECISION_FP64 && s->kernel == LG_FORCE_KERNEL_PAIRS));
    LG_TRY(launch_forces(s, hdt, dt, mv, fuse, prev_fused));
    s->kick_done = fuse;
    s->vcur = 1 - s->vcur;
    if (mv) s->fcur = 1 - s->fcur;
    s->step_index++;
    return LG_OK;
}

// Hold mask of n particles: only LG_HOLD_* bits.
static int validate_hold(const uint8_t *mask, int64_t n) {
    if (!mask) return LG_OK;
    for (int64_t i = 0; i < n; ++i)
        if (mask[i] & ~(LG_HOLD_X | LG_HOLD_V | LG_HOLD_THETA | LG_HOLD_OMEGA))
            return lg_fail(LG_E_INVALID, "hold mask: particle %lld has unknown bits 0x%x", (long long)i, mask[i]);
    return LG_OK;
}

// Body force (null: none) and unary hook (null: none): a known model, finite parameters, not both.
static int validate_unary(const lg_body_force *body, lg_unary_hook hook) {
    const int model = body ? body->model : LG_BODY_NONE;
    if (model != LG_BODY_NONE && model != LG_BODY_CENTRAL)
        return lg_fail(LG_E_INVALID, "body force: unknown model %d", model);
    if (model != LG_BODY_NONE && hook) return lg_fail(LG_E_INVALID, "a body force and a unary hook exclude each other");
    if (model == LG_BODY_CENTRAL) {
        if (!(body->mass > 0) || !std::isfinite(body->mass) || !std::isfinite(body->k_a))
            return lg_fail(LG_E_INVALID, "body force: mass must be positive and k_a finite");
        for (int c = 0; c < 3; ++c)
            if (!std::isfinite(body->centre[c])) return lg_fail(LG_E_INVALID, "body force: centre is not finite");
    }
    return LG_OK;
}

static int check_args(const lg_system_desc *d) {
    if (!d) return lg_fail(LG_E_INVALID, "lg_create: null descriptor");
    if (d->n_part < 1 || d->n_part > (int64_t)1 << 30) return lg_fail(LG_E_INVALID, "lg_create: n_part %lld out of range", (long long)d->n_part);
    if (d->binary_model < 0 || d->binary_model > 4) return lg_fail(LG_E_INVALID, "lg_create: unknown binary_model %d", d->binary_model);
    if (d->binary_model == LG_BINARY_SINTER_CONNECTORS && d->precision != LG_PRECISION_FP64)
        return lg_fail(LG_E_INVALID, "lg_create: the 5-connector sinter model runs in FP64 precision only");
    if (d->hamaker_model < 0 || d->hamaker_model > 3) return lg_fail(LG_E_INVALID, "lg_create: unknown hamaker_model %d", d->hamaker_model);
    if (d->binary_model == LG_BINARY_NONE && d->hamaker_model == LG_HAMAKER_NONE)
        return lg_fail(LG_E_INVALID, "lg_create: at least one binary force functor must be provided");
    if (d->pairs != LG_PAIRS_ALL && d->pairs != LG_PAIRS_VERLET) return lg_fail(LG_E_INVALID, "lg_create: unknown pairs mode %d", d->pairs);
    if (d->pairs == LG_PAIRS_VERLET && !(d->r_verlet > 0)) return lg_fail(LG_E_INVALID, "lg_create: r_verlet must be > 0");
    if (d->pairs == LG_PAIRS_ALL && d->n_part > 8192)
        return lg_fail(LG_E_INVALID, "lg_create: all-pairs mode holds n^2 spring slots; n_part %lld > 8192 needs LG_PAIRS_VERLET", (long long)d->n_part);
    if (d->precision != LG_PRECISION_FP64 && d->precision != LG_PRECISION_MIXED) return lg_fail(LG_E_INVALID, "lg_create: unknown precision %d", d->precision);
    if (d->precision == LG_PRECISION_MIXED && !lg::mixed_available()) return lg_fail(LG_E_INVALID, "lg_create: mixed precision is not built in this library");
    if (d->n_facets < 0 || d->n_facets > kMaxFacets) return lg_fail(LG_E_INVALID, "lg_create: n_facets %d out of range [0, %d]", d->n_facets, kMaxFacets);
    if (d->neck_mode != LG_NECK_PER_BOND && d->neck_mode != LG_NECK_REFERENCE_INDEXING) return lg_fail(LG_E_INVALID, "lg_create: unknown neck_mode %d", d->neck_mode);
    if (d->max_neighbors < 0 || d->max_neighbors > 255)
        return lg_fail(LG_E_INVALID, "lg_create: max_neighbors must be in [0, 255]");
    if (d->force_kernel < 0 || d->force_kernel > 5) return lg_fail(LG_E_INVALID, "lg_create: unknown force_kernel %d", d->force_kernel);
    if (d->force_kernel == LG_FORCE_KERNEL_FP64_FAST && d->precision != LG_PRECISION_FP64)
        return lg_fail(LG_E_INVALID, "lg_create: the fast FP64 kernel is FP64 precision only");
    if (d->force_kernel == LG_FORCE_KERNEL_PERSISTENT && d->precision != LG_PRECISION_MIXED)
        return lg_fail(LG_E_INVALID, "lg_create: the persistent step kernel is mixed precision only");
    LG_TRY(validate_hold(d->hold_mask, d->n_part));
    LG_TRY(validate_unary(&d->body, d->unary_hook));
    if (d->force_kernel == LG_FORCE_KERNEL_PAIRS && d->precision != LG_PRECISION_FP64)
        return lg_fail(LG_E_INVALID, "lg_create: the pair-parallel force kernel is FP64 only");
    {
        int T = d->threads_per_row;
        if (T != 0 && T != 1 && T != 2 && T != 4 && T != 8 && T != 16 && T != 32)
            return lg_fail(LG_E_INVALID, "lg_create: threads_per_row must be 0 or a power of two <= 32");
    }
    return LG_OK;
}

// Hold mask (LG_HOLD_* bits per particle); null clears it. Params are captured by value in the
// CUDA graphs, so the graphs are dropped.
static int apply_hold(lg_system *s, const uint8_t *mask) {
    LG_TRY(validate_hold(mask, s->P.n));
    s->drop_graphs();
    if (!mask) {
        s->P.hold = nullptr;
        return LG_OK;
    }
    if (!s->d_hold) LG_TRY(s->alloc(&s->d_hold, (size_t)s->P.n));
    LG_CUDA(cudaMemcpyAsync(s->d_hold, mask, (size_t)s->P.n, cudaMemcpyHostToDevice, s->stream));
    LG_CUDA(cudaStreamSynchronize(s->stream));
    s->P.hold = s->d_hold;
    return LG_OK;
}

// Body force or unary hook (at most one); both write the per-particle unary terms that the force
// kernels fold after the facets.
static int apply_unary(lg_system *s, const lg_body_force *body, lg_unary_hook hook, void *user) {
    LG_TRY(validate_unary(body, hook));
    const int model = body ? body->model : LG_BODY_NONE;
    s->drop_graphs();
    const bool on = model != LG_BODY_NONE || hook;
    if (on && !s->ext_a) {
        LG_TRY(s->alloc(&s->ext_a, (size_t)s->P.n));
        LG_TRY(s->alloc(&s->ext_al, (size_t)s->P.n));
    }
    if (model == LG_BODY_CENTRAL) {
        const int64_t nsys = std::max<int64_t>(1, s->n_systems);
        if (!s->d_centre) LG_TRY(s->alloc(&s->d_centre, 3 * (size_t)nsys));
        std::vector<double> c(3 * (size_t)nsys);
        for (int64_t q = 0; q < nsys; ++q)
            for (int k = 0; k < 3; ++k) c[3 * q + k] = body->centre[k];
        LG_CUDA(cudaMemcpyAsync(s->d_centre, c.data(), sizeof(double) * c.size(), cudaMemcpyHostToDevice, s->stream));
        LG_CUDA(cudaStreamSynchronize(s->stream));
    }
    s->body = lg_body_force{};
    if (model != LG_BODY_NONE) s->body = *body;
    s->hook = hook;
    s->hook_user = hook ? user : nullptr;
    s->P.ext_a = on ? s->ext_a : nullptr;
    s->P.ext_al = on ? s->ext_al : nullptr;
    return LG_OK;
}

// A serving arena (lg_arena_create): a batch whose systems are slots that start empty -- every
// particle inactive, no bonds -- on a lattice of the given spacing, with bond capacity bcap per
// particle and float-float extents allowed up to ext.
struct ArenaSpec {
    int32_t bcap;
    double lattice, ext;
};

static int create_impl(const lg_system_desc *d, const double *x0, const double *v0, const double *th0, const double *om0,
                       const lg_facet_desc *facets, const double *neck, int64_t n_neck, int device, lg_system *s,
                       int64_t n_sys = 0, const int64_t *sizes = nullptr, const ArenaSpec *arena = nullptr) {
    LG_TRY(check_args(d));
    if (!x0 || !v0 || !th0 || !om0) return lg_fail(LG_E_INVALID, "lg_create: null state pointer");
    if (d->n_facets > 0 && !facets) return lg_fail(LG_E_INVALID, "lg_create: n_facets > 0 but facets is null");
    const int64_t n = d->n_part;
    if (n_sys > 0) {
        if (!sizes) return lg_fail(LG_E_INVALID, "lg_batch_create: null sizes");
        if (d->pairs != LG_PAIRS_VERLET) return lg_fail(LG_E_INVALID, "lg_batch_create: batches need LG_PAIRS_VERLET");
        s->n_systems = n_sys;
        s->sys_off.assign((size_t)n_sys + 1, 0);
        for (int64_t q = 0; q < n_sys; ++q) {
            if (sizes[q] < 1) return lg_fail(LG_E_INVALID, "lg_batch_create: system %lld has size %lld", (long long)q, (long long)sizes[q]);
            s->sys_off[q + 1] = s->sys_off[q] + sizes[q];
        }
        if (s->sys_off[n_sys] != n)
            return lg_fail(LG_E_INVALID, "lg_batch_create: sizes add up to %lld, desc.n_part is %lld",
                           (long long)s->sys_off[n_sys], (long long)n);
    }
    s->device = device;
    LG_CUDA(cudaSetDevice(device));
    LG_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    LG_CUDA(cudaEventCreate(&s->ev0));
    LG_CUDA(cudaEventCreate(&s->ev1));
    s->desc = *d;
    s->precision = d->precision;
    if (d->n_facets > 0) s->facet_descs.assign(facets, facets + d->n_facets);
    if (neck && n_neck > 0) s->neck_copy.assign(neck, neck + n_neck);
    if (n_sys > 0) s->sizes_copy.assign(sizes, sizes + n_sys);
    s->facet_auto_move = d->facet_auto_move != 0;

    Params &P = s->P;
    memset(&P, 0, sizeof(P));
    P.n = n;
    P.binary_model = d->binary_model;
    P.hamaker_model = d->hamaker_model;
    P.neck_mode = d->neck_mode;
    P.pairs = d->pairs;
    P.contact = d->contact;
    P.sinter = d->sinter;
    P.hamaker = d->hamaker;
    P.r_verlet = d->r_verlet;
    P.n_facets = d->n_facets;
    const double cr = 2.0 * d->contact.r_part;
    P.contact_skip_d2 = cr * cr * (1.0 + 1e-9);
    P.hamaker_skip_d2 = d->hamaker.r_cutoff * d->hamaker.r_cutoff * (1.0 + 1e-9);
    P.springs_ff = d->precision == LG_PRECISION_MIXED ? 1 : 0;
    P.connector = d->connector;
    for (int f = 0; f < d->n_facets; ++f) {
        const lg_facet_desc &fd = facets[f];
        FacetDev &o = P.facets[f];
        for (int c = 0; c < 3; ++c) o.v[c] = fd.v_facet[c];
        d3 v0_ = mk3(fd.vertices[0], fd.vertices[1], fd.vertices[2]);
        d3 v1_ = mk3(fd.vertices[3], fd.vertices[4], fd.vertices[5]);
        d3 v2_ = mk3(fd.vertices[6], fd.vertices[7], fd.vertices[8]);
        d3 u = sub(v1_, v0_), w = sub(v2_, v0_);
        o.area = 1.0 / 2.0 * nrm(crs(u, w));  // triangular_facet.h:23-27
        d3 N = nrmz(crs(u, w));
        o.normal[0] = N.x;
        o.normal[1] = N.y;
        o.normal[2] = N.z;
        o.has_contact = fd.has_contact;
        o.has_hamaker = fd.has_hamaker;
        o.contact = fd.contact;
        o.hamaker = fd.hamaker;
    }

    // bonds
    std::vector<std::pair<int32_t, int32_t>> bonds;
    const bool sinter = d->binary_model == LG_BINARY_SINTER || d->binary_model == LG_BINARY_BREAKING_SINTER;
    if (arena) {  // empty slots: bonds arrive with their occupants
        if (d->binary_model == LG_BINARY_SINTER_CONNECTORS)
            return lg_fail(LG_E_INVALID, "serving slots do not hold the 5-connector model");
        s->n_bonds_initial_sys.assign((size_t)s->n_systems, 0);
    } else if (sinter) {
        if (s->n_systems == 0) {
            LG_TRY(lg_detect_bonds(x0, n, d->sinter.r_part, d->sinter.critical_separation,
                                   d->binary_model == LG_BINARY_SINTER, bonds));
        } else {  // every system's bonds are found alone, in the order a standalone system finds them
            s->n_bonds_initial_sys.assign((size_t)s->n_systems, 0);
            std::vector<std::pair<int32_t, int32_t>> local;
            for (int64_t q = 0; q < s->n_systems; ++q) {
                const int64_t b = s->sys_off[q], e = s->sys_off[q + 1];
                LG_TRY(lg_detect_bonds(x0 + 3 * b, e - b, d->sinter.r_part, d->sinter.critical_separation,
                                       d->binary_model == LG_BINARY_SINTER, local));
                for (auto &pr : local) bonds.emplace_back((int32_t)(pr.first + b), (int32_t)(pr.second + b));
                s->n_bonds_initial_sys[q] = 2 * (int64_t)local.size();
            }
        }
    }
    const bool connectors = d->binary_model == LG_BINARY_SINTER_CONNECTORS;
    if (connectors && !arena) {  // sinter_functor ctor, sinter_bridge.h:146-160: no cycle check, |g| <= dc
        const double r = d->contact.r_part, dc = d->connector.critical_separation;
        if (s->n_systems == 0) {
            LG_TRY(lg_detect_bonds(x0, n, r, dc, false, bonds, true));
        } else {
            s->n_bonds_initial_sys.assign((size_t)s->n_systems, 0);
            std::vector<std::pair<int32_t, int32_t>> local;
            for (int64_t q = 0; q < s->n_systems; ++q) {
                const int64_t b = s->sys_off[q], e = s->sys_off[q + 1];
                LG_TRY(lg_detect_bonds(x0 + 3 * b, e - b, r, dc, false, local, true));
                for (auto &pr : local) bonds.emplace_back((int32_t)(pr.first + b), (int32_t)(pr.second + b));
                s->n_bonds_initial_sys[q] = 2 * (int64_t)local.size();
            }
        }
        if (!d->connector_axes || d->n_connector_axes != (int64_t)bonds.size())
            return lg_fail(LG_E_INVALID, "lg_create: %lld connector axes given but %zu bonds were detected",
                           (long long)d->n_connector_axes, bonds.size());
    }
    if (d->binary_model == LG_BINARY_BREAKING_SINTER && n_neck != 0 && n_neck != (int64_t)bonds.size())
        return lg_fail(LG_E_INVALID, "lg_create: %lld neck strengths given but %zu bonds were detected", (long long)n_neck,
                       bonds.size());
    std::vector<int32_t> deg((size_t)n, 0);
    for (auto &b : bonds) {
        deg[b.first]++;
        deg[b.second]++;
    }
    int32_t bcap = arena ? std::max<int32_t>(1, arena->bcap) : 1;
    for (int64_t i = 0; i < n; ++i) bcap = std::max(bcap, deg[i]);
    if (bcap > 255) return lg_fail(LG_E_INVALID, "lg_create: a particle has %d bonds (max 255)", bcap);
    s->bv.bcap = bcap;
    s->bv.aos = s->precision == LG_PRECISION_MIXED ? 1 : 0;
    s->n_bonds_initial = 2 * (int64_t)bonds.size();
    {
        const size_t bs = (size_t)bcap * (size_t)n;
        std::vector<int32_t> bj(bs, -1);
        std::vector<int8_t> bint(bs, 0);
        std::vector<double> bstr(bs, 0.0);
        std::vector<double> pstr((size_t)n, 0.0);  // particle-indexed strengths of the reference
        std::vector<int32_t> fill((size_t)n, 0);
        for (size_t b = 0; b < bonds.size(); ++b) {
            double sv = (neck && n_neck > 0) ? neck[b] : INFINITY;
            pstr[bonds[b].first] = sv;
            pstr[bonds[b].second] = sv;
        }
        for (size_t b = 0; b < bonds.size(); ++b) {
            double sv = (neck && n_neck > 0) ? neck[b] : INFINITY;
            int32_t i = bonds[b].first, j = bonds[b].second;
            int32_t si = fill[i]++, sj = fill[j]++;
            size_t ei = (size_t)si * n + i, ej = (size_t)sj * n + j;
            bj[ei] = j;
            bj[ej] = i;
            bint[ei] = bint[ej] = 1;
            if (d->neck_mode == LG_NECK_REFERENCE_INDEXING) {
                bstr[ei] = (i == 0) ? pstr[j] : 0.0;  // neck_strengths[i*n + j] is set only where i == 0
                bstr[ej] = (j == 0) ? pstr[i] : 0.0;
            } else {
                bstr[ei] = bstr[ej] = sv;
            }
        }
        LG_TRY(s->alloc(&s->bv.j, bs));
        LG_TRY(s->alloc(&s->bv.intact, bs));
        LG_TRY(s->alloc(&s->bv.strength, bs));
        LG_TRY(s->alloc(&s->bv.xi, 9 * bs));
        LG_CUDA(cudaMemcpy(s->bv.j, bj.data(), sizeof(int32_t) * bs, cudaMemcpyHostToDevice));
        LG_CUDA(cudaMemcpy(s->bv.intact, bint.data(), sizeof(int8_t) * bs, cudaMemcpyHostToDevice));
        LG_CUDA(cudaMemcpy(s->bv.strength, bstr.data(), sizeof(double) * bs, cudaMemcpyHostToDevice));
        LG_CUDA(cudaMemset(s->bv.xi, 0, sizeof(double) * 9 * bs));
        if (connectors) {
            // the connectors of each bond, sinter_bridge.h:163-197 (evaluated in the reference's
            // order; this file is compiled without contraction)
            std::vector<double> cn(15 * bs, 0.0);
            std::vector<int32_t> rev(bs, -1);
            std::vector<int32_t> slot((size_t)n, 0);
            const double r = d->contact.r_part;
            for (size_t b = 0; b < bonds.size(); ++b) {
                const int32_t i = bonds[b].first, j = bonds[b].second;
                const d3 pi = hld(x0, i), pj = hld(x0, j);
                const d3 ni = nrmz(sub(pj, pi)), nj = neg(ni);
                const d3 v = hld(d->connector_axes, (int64_t)b);
                d3 db = crs(v, nj);
                if (nrm(db) == 0.0)
                    return lg_fail(LG_E_INVALID, "lg_create: connector axis %zu is parallel to its bond", b);
                d3 ds = sub(v, scl(dot(v, ni), ni));
                db = nrmz(db);
                ds = nrmz(ds);
                const d3 ci[5] = {add(pi, scl(r, ds)), sub(pi, scl(r, ds)), add(pi, scl(r, db)), sub(pi, scl(r, db)),
                                  add(pi, scl(r, ni))};
                const d3 cj[5] = {add(pj, scl(r, ds)), sub(pj, scl(r, ds)), add(pj, scl(r, db)), sub(pj, scl(r, db)),
                                  add(pj, scl(r, nj))};
                const int32_t si = slot[i]++, sj = slot[j]++;
                const size_t ei = (size_t)si * n + i, ej = (size_t)sj * n + j;
                for (int k = 0; k < 5; ++k) {
                    cn[(3 * k) * bs + ei] = ci[k].x; cn[(3 * k + 1) * bs + ei] = ci[k].y; cn[(3 * k + 2) * bs + ei] = ci[k].z;
                    cn[(3 * k) * bs + ej] = cj[k].x; cn[(3 * k + 1) * bs + ej] = cj[k].y; cn[(3 * k + 2) * bs + ej] = cj[k].z;
                }
                rev[ei] = sj;
                rev[ej] = si;
            }
            LG_TRY(s->alloc(&s->bv.cn, 15 * bs));
            LG_TRY(s->alloc(&s->bv.rev, bs));
            LG_CUDA(cudaMemcpy(s->bv.cn, cn.data(), sizeof(double) * cn.size(), cudaMemcpyHostToDevice));
            LG_CUDA(cudaMemcpy(s->bv.rev, rev.data(), sizeof(int32_t) * rev.size(), cudaMemcpyHostToDevice));
        }
        s->host_bond_j = std::move(bj);
    }

    // state
    LG_TRY(s->alloc(&s->x, n));
    LG_TRY(s->alloc(&s->th, n));
    LG_TRY(s->alloc(&s->v[0], n));
    LG_TRY(s->alloc(&s->v[1], n));
    LG_TRY(s->alloc(&s->w[0], n));
    LG_TRY(s->alloc(&s->w[1], n));
    LG_TRY(s->alloc(&s->a, n));
    LG_TRY(s->alloc(&s->al, n));
    LG_TRY(s->alloc(&s->err, 1));
    LG_CUDA(cudaMemset(s->err, 0, sizeof(int32_t)));
    LG_CUDA(cudaMemset(s->a, 0, sizeof(dbl4) * n));
    LG_CUDA(cudaMemset(s->al, 0, sizeof(dbl4) * n));
    LG_TRY(upload4(s->x, x0, n, s->stream));
    LG_TRY(upload4(s->v[0], v0, n, s->stream));
    LG_TRY(upload4(s->th, th0, n, s->stream));
    LG_TRY(upload4(s->w[0], om0, n, s->stream));
    s->vcur = 0;

    if (arena) {  // every particle of an empty slot takes no part (no cell, no row, no motion)
        LG_TRY(s->alloc(&s->d_hold, (size_t)n));
        LG_CUDA(cudaMemset(s->d_hold, (int)kHoldInactive, (size_t)n));
        P.hold = s->d_hold;
    }

    // batch segmentation: system index per particle, hashing offsets that keep systems apart
    if (s->n_systems > 0) {
        const int64_t ns = s->n_systems;
        std::vector<int32_t> agg((size_t)n);
        std::vector<double> cen(3 * (size_t)ns), rad((size_t)ns, 0.0);
        double rmax = 0.0;
        for (int64_t q = 0; q < ns; ++q) {
            const int64_t b = s->sys_off[q], e = s->sys_off[q + 1];
            for (int k = 0; k < 3; ++k) {
                double sum = 0.0;
                for (int64_t i = b; i < e; ++i) sum += x0[3 * i + k];
                cen[3 * q + k] = sum / (double)(e - b);
            }
            for (int64_t i = b; i < e; ++i) {
                agg[i] = (int32_t)q;
                double r2 = 0.0;
                for (int k = 0; k < 3; ++k) r2 += (x0[3 * i + k] - cen[3 * q + k]) * (x0[3 * i + k] - cen[3 * q + k]);
                rad[q] = std::max(rad[q], std::sqrt(r2));
            }
            rmax = std::max(rmax, rad[q]);
        }
        // lattice spacing: two system radii, room for growth, and two list radii
        const double L = arena ? arena->lattice : 4.0 * rmax + 2.0 * d->r_verlet + 8.0 * d->contact.r_part + 1e-12;
        int64_t m = 1;
        while (m * m * m < ns) ++m;
        std::vector<dbl4> hoff((size_t)ns);
        for (int64_t q = 0; q < ns; ++q) {
            const double gx = (double)(q % m) * L, gy = (double)((q / m) % m) * L, gz = (double)(q / (m * m)) * L;
            hoff[q] = make_double4_32a(gx - cen[3 * q], gy - cen[3 * q + 1], gz - cen[3 * q + 2], 0.0);
        }
        LG_TRY(s->alloc(&s->d_agg, (size_t)n));
        LG_TRY(s->alloc(&s->d_hoff, (size_t)ns));
        LG_TRY(s->alloc(&s->d_sys_off, (size_t)ns + 1));
        LG_TRY(s->alloc(&s->d_centres, 3 * (size_t)ns));
        LG_TRY(s->alloc(&s->d_sys_obs, 20 * (size_t)ns));
        LG_CUDA(cudaMemcpy(s->d_agg, agg.data(), sizeof(int32_t) * agg.size(), cudaMemcpyHostToDevice));
        LG_CUDA(cudaMemcpy(s->d_hoff, hoff.data(), sizeof(dbl4) * hoff.size(), cudaMemcpyHostToDevice));
        LG_CUDA(cudaMemcpy(s->d_sys_off, s->sys_off.data(), sizeof(int64_t) * s->sys_off.size(), cudaMemcpyHostToDevice));
    }

    // facets
    const int nf = std::max(d->n_facets, 1);
    LG_TRY(s->alloc(&s->fv[0], 9 * (size_t)nf));
    LG_TRY(s->alloc(&s->fv[1], 9 * (size_t)nf));
    LG_TRY(s->alloc(&s->sxi, 9 * (size_t)nf * (size_t)n));
    LG_CUDA(cudaMemset(s->sxi, 0, sizeof(double) * 9 * (size_t)nf * (size_t)n));
    if (d->n_facets > 0) {
        std::vector<double> fvh(9 * (size_t)d->n_facets);
        for (int f = 0; f < d->n_facets; ++f)
            for (int q = 0; q < 9; ++q) fvh[9 * f + q] = facets[f].vertices[q];
        LG_CUDA(cudaMemcpy(s->fv[0], fvh.data(), sizeof(double) * fvh.size(), cudaMemcpyHostToDevice));
        LG_CUDA(cudaMemcpy(s->fv[1], fvh.data(), sizeof(double) * fvh.size(), cudaMemcpyHostToDevice));
    }
    s->fcur = 0;

    // pair slots
    if (d->pairs == LG_PAIRS_ALL) {
        const int64_t cap = std::max<int64_t>(n - 1, 1);
        PairView &pv = s->pv[0];
        pv.cap = cap;
        pv.aos = s->precision == LG_PRECISION_MIXED ? 1 : 0;
        pv.nbr = nullptr;
        pv.row_len = nullptr;
        LG_TRY(s->alloc(&pv.flags, (size_t)(cap * n)));
        LG_TRY(s->alloc(&pv.xi, 9 * (size_t)(cap * n)));
        LG_CUDA(cudaMemset(pv.xi, 0, sizeof(double) * 9 * (size_t)(cap * n)));
        std::vector<uint32_t> fl((size_t)(cap * n), 0u);
        for (int64_t b = 0; b < bcap; ++b)
            for (int64_t i = 0; i < n; ++i) {
                int32_t j = s->host_bond_j[(size_t)b * n + i];
                if (j < 0) continue;
                int64_t k = j < i ? j : j - 1;
                fl[(size_t)(k * n + i)] = kBonded | ((uint32_t)b << 8);
            }
        LG_CUDA(cudaMemcpy(pv.flags, fl.data(), sizeof(uint32_t) * fl.size(), cudaMemcpyHostToDevice));
        s->pv[1] = pv;
        s->pcur = 0;
    } else {
        int64_t cap = d->max_neighbors > 0 ? d->max_neighbors : 48;
        cap = std::min<int64_t>(cap, std::max<int64_t>(n - 1, 1));
        // mixed precision: contact candidates are listed per row at each build (PairView::near_*),
        // within the contact reach plus the Verlet skin (the list radius minus the largest
        // interaction radius); without a Hamaker cutoff the skin is unknown and every slot is near
        if (s->precision == LG_PRECISION_MIXED && d->binary_model != LG_BINARY_NONE) {
            const double creach = std::max(d->binary_model == LG_BINARY_CONTACT ? 2.0 * d->contact.r_part : 0.0,
                                           sinter ? std::max(2.0 * d->sinter.r_part, 2.0 * d->contact.r_part) : 0.0);
            double reach = creach;
            if (d->hamaker_model == LG_HAMAKER_LIMITED) reach = std::max(reach, d->hamaker.r_cutoff);
            const bool capped = d->hamaker_model == LG_HAMAKER_NONE || d->hamaker_model == LG_HAMAKER_LIMITED;
            s->r_near = capped ? std::min(d->r_verlet, creach + std::max(d->r_verlet - reach, 0.0)) : d->r_verlet;
        }
        auto alloc_rows = [&](int64_t c) -> int {
            for (int q = 0; q < 2; ++q) {
                PairView &pv = s->pv[q];
                pv.cap = c;
                pv.aos = s->precision == LG_PRECISION_MIXED ? 1 : 0;
                LG_TRY(s->alloc(&pv.nbr, (size_t)(c * n)));
                LG_TRY(s->alloc(&pv.row_len, (size_t)n));
                LG_TRY(s->alloc(&pv.flags, (size_t)(c * n)));
                LG_TRY(s->alloc(&pv.xi, 9 * (size_t)(c * n)));
                LG_CUDA(cudaMemset(pv.row_len, 0, sizeof(int32_t) * n));
                if (s->r_near > 0) {
                    LG_TRY(s->alloc(&pv.near_j, (size_t)(c * n)));
                    LG_TRY(s->alloc(&pv.near_k, (size_t)(c * n)));
                    LG_TRY(s->alloc(&pv.near_len, (size_t)n));
                    LG_CUDA(cudaMemset(pv.near_len, 0, sizeof(int32_t) * n));
                }
            }
            return LG_OK;
        };
        LG_TRY(alloc_rows(cap));
        s->pcur = 0;
        s->max_cells = std::max<int64_t>(64, (s->n_systems > 0 ? 8 : 4) * n);
        if (arena) {  // the slot lattice at cells of about r_verlet (capped at 2^25 cells)
            int64_t m = 1;
            while (m * m * m < s->n_systems) ++m;
            const double per = (double)m * arena->lattice / d->r_verlet + 2.0;
            s->max_cells = std::max<int64_t>(s->max_cells, (int64_t)std::min(per * per * per, 33554432.0));
        }
        s->ls.nparts = 256;
        LG_TRY(s->alloc(&s->ls.part, 6 * 256));
        LG_TRY(s->alloc(&s->ls.grid, 1));
        LG_TRY(s->alloc(&s->ls.cell_of, (size_t)n));
        LG_TRY(s->alloc(&s->ls.count, (size_t)s->max_cells));
        LG_TRY(s->alloc(&s->ls.start, (size_t)s->max_cells));
        LG_TRY(s->alloc(&s->ls.fill, (size_t)s->max_cells));
        LG_TRY(s->alloc(&s->ls.sorted, (size_t)n));
        LG_TRY(s->alloc(&s->ls.tile, (size_t)(s->max_cells / 4096 + 1)));
        LG_TRY(s->alloc(&s->ls.x32, (size_t)n));
        LG_TRY(s->alloc(&s->ls.max_row, 1));
        LG_CUDA(cudaMemset(s->ls.max_row, 0, sizeof(int32_t)));
        LG_TRY(rebuild_list(s));
        // without an explicit max_neighbors the row capacity follows the initial state: rows get
        // 1.5x the longest initial row (at most 255)
        int32_t mr = 0;
        LG_CUDA(cudaMemcpy(&mr, s->ls.max_row, sizeof(int32_t), cudaMemcpyDeviceToHost));
        const int64_t want = std::min<int64_t>(255, std::max<int64_t>(8, (int64_t)(1.5 * mr) + 1));
        if (d->max_neighbors == 0 && want > cap && cap < std::max<int64_t>(n - 1, 1)) {
            for (int q = 0; q < 2; ++q) {
                PairView &pv = s->pv[q];
                void *old_ptrs[7] = {pv.nbr, pv.row_len, pv.flags, pv.xi, pv.near_j, pv.near_k, pv.near_len};
                for (void *o : old_ptrs) {
                    if (!o) continue;
                    cudaFree(o);
                    s->allocations.erase(std::find(s->allocations.begin(), s->allocations.end(), o));
                }
            }
            cap = std::min<int64_t>(want, std::max<int64_t>(n - 1, 1));
            LG_TRY(alloc_rows(cap));
            s->list_built = false;
            s->pcur = 0;
            LG_CUDA(cudaMemset(s->err, 0, sizeof(int32_t)));
            LG_TRY(rebuild_list(s));
        }
    }
    if (s->precision == LG_PRECISION_FP64 && (int64_t)s->pv[0].cap * n <= kPairsMaxSlots)
        LG_TRY(s->alloc(&s->pres, 6 * (size_t)(s->pv[0].cap * n)));
    LG_TRY(s->alloc(&s->obs_scratch, (size_t)obs_scratch_doubles(n)));
    LG_TRY(s->alloc(&s->d_ticket, 1));
    LG_CUDA(cudaMemset(s->d_ticket, 0, sizeof(unsigned)));
    if (s->pooled) {  // plain host memory: freeing pinned memory can synchronise the device
        s->h_pin = (double *)std::malloc(64 * sizeof(double));
        if (!s->h_pin) return lg_fail(LG_E_NOMEM, "lg_create: host allocation failed");
    } else {
        LG_CUDA(cudaMallocHost(&s->h_pin, 64 * sizeof(double)));
    }
    LG_TRY(s->alloc(&s->obs_out, 32));

    if (s->precision == LG_PRECISION_MIXED) {
        LG_TRY(s->alloc(&s->x32buf, 4 * (size_t)n));  // two buffers of float-float positions (hi, lo interleaved)
        LG_TRY(s->alloc(&s->v32buf, 6 * (size_t)n));  // two buffers of v high parts, v low parts, spins
        s->ffcur = 0;
        s->x32 = s->x32buf;
        s->v32 = s->v32buf;
        LG_TRY(s->alloc(&s->s32, 5 * (size_t)n));  // spin low parts, displacement and rotation of a run
        LG_TRY(s->alloc(&s->csum, 3 * (size_t)n));
        LG_TRY(s->alloc(&s->d_flag, 1));
        LG_TRY(s->alloc(&s->hsum, 2 * (size_t)n));
        LG_CUDA(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking));
        LG_CUDA(cudaEventCreateWithFlags(&s->fork_ev, cudaEventDisableTiming));
        LG_CUDA(cudaEventCreateWithFlags(&s->join_ev, cudaEventDisableTiming));
        if (s->n_systems > 0) LG_TRY(s->alloc(&s->d_orig, (size_t)s->n_systems));
        s->r_max = std::max(d->contact.r_part, std::max(d->sinter.r_part, d->hamaker.r_part));
        LG_TRY(set_mixed_origins(s, x0));
        if (arena) s->ext_max = std::max(s->ext_max, arena->ext);  // room for the widest occupant
        launch_mixed_copies(n, s->x, s->v[s->vcur], s->w[s->vcur], s->th, s->origin, s->d_agg, s->d_orig, s->x32, s->v32, s->s32,
                            s->stream);
        double near = 0.0;
        if (d->binary_model != LG_BINARY_NONE) near = std::max(near, 2.0 * d->contact.r_part);
        if (sinter) near = std::max(near, 2.0 * d->sinter.r_part);
        if (d->hamaker_model == LG_HAMAKER_LIMITED) near = std::max(near, d->hamaker.r_cutoff);
        if (d->hamaker_model == LG_HAMAKER_FULL || d->hamaker_model == LG_HAMAKER_SIMPLIFIED)
            near = std::max(near, 7.0 * d->hamaker.r_part);
        s->mx.x32 = s->x32;
        s->mx.v32 = s->v32;
        s->mx.s32 = s->s32;
        s->mx.csum = s->csum;
        s->mx.hsum = s->hsum;
        double cnear = 0.0;
        if (d->binary_model != LG_BINARY_NONE) cnear = std::max(cnear, 2.0 * d->contact.r_part);
        if (sinter) cnear = std::max(cnear, 2.0 * d->sinter.r_part);
        s->cull_near = near;
        s->cull_contact = cnear;
        set_cull_radii(s);
        s->mx.inv_mass_h = d->hamaker.mass > 0 ? (float)(1.0 / d->hamaker.mass) : 0.f;
        s->mx.inv_mass_c = d->contact.mass > 0 ? 1.0 / d->contact.mass : 0.0;
        s->mx.inv_inertia_c = d->contact.inertia > 0 ? 1.0 / d->contact.inertia : 0.0;
        s->mx.inv_mass_b = d->sinter.mass > 0 ? 1.0 / d->sinter.mass : 0.0;
        s->mx.inv_inertia_b = d->sinter.inertia > 0 ? 1.0 / d->sinter.inertia : 0.0;
        s->mx.four_rc2 = 4.0 * d->contact.r_part * d->contact.r_part;
        s->mx.four_rb2 = 4.0 * d->sinter.r_part * d->sinter.r_part;
        s->mx.four_rh2 = 4.0 * d->hamaker.r_part * d->hamaker.r_part;
        const lg_contact_params &C = d->contact;
        const lg_sinter_params &B = d->sinter;
        MixedExtra &M = s->mx;
        M.c_k = (float)C.k; M.c_gn = (float)C.gamma_n; M.c_kt = (float)C.k_t; M.c_gt = (float)C.gamma_t;
        M.c_mus = (float)C.mu_s; M.c_phid = (float)C.phi_d; M.c_kr = (float)C.k_r; M.c_gr = (float)C.gamma_r;
        M.c_mur = (float)C.mu_r; M.c_phir = (float)C.phi_r; M.c_ko = (float)C.k_o; M.c_go = (float)C.gamma_o;
        M.c_muo = (float)C.mu_o; M.c_phio = (float)C.phi_o; M.c_r = (float)C.r_part; M.c_dt = (float)C.dt;
        M.b_k = (float)B.k; M.b_gn = (float)B.gamma_n; M.b_kt = (float)B.k_t; M.b_gt = (float)B.gamma_t;
        M.b_kr = (float)B.k_r; M.b_gr = (float)B.gamma_r; M.b_ko = (float)B.k_o; M.b_go = (float)B.gamma_o;
        M.b_r = (float)B.r_part; M.b_dt = (float)B.dt;
        M.h_A = (float)d->hamaker.A; M.h_h0 = (float)d->hamaker.h0; M.h_r = (float)d->hamaker.r_part;
        s->mx.rcut2 = d->hamaker.r_cutoff * d->hamaker.r_cutoff;
        auto split = [](double v, float &hi, float &lo) {
            hi = (float)v;
            lo = (float)(v - (double)hi);
        };
        split(s->mx.four_rh2, M.h_fr_hi, M.h_fr_lo);
        split(s->mx.four_rc2, M.c_fr_hi, M.c_fr_lo);
        split(s->mx.four_rb2, M.b_fr_hi, M.b_fr_lo);
        M.h_qcut = (float)(s->mx.rcut2 - s->mx.four_rh2);
        M.bin_im = (float)(sinter ? s->mx.inv_mass_b : s->mx.inv_mass_c);
        M.bin_iI = (float)(sinter ? s->mx.inv_inertia_b : s->mx.inv_inertia_c);
        // contact threshold band: |q| <= 1e-10 (2r)^2, i.e. |overlap| <~ 5e-11 r, far above the
        // float-float error of q and far below the overlaps of loaded contacts
        M.q_marg = (float)(1e-10 * s->mx.four_rc2);
        M.x64 = nullptr;
    }
    s->T = d->threads_per_row > 0 ? d->threads_per_row : choose_threads_per_row(s);
    s->kernel = choose_kernel(s, d->force_kernel);
    if (s->kernel < 0)
        return lg_fail(LG_E_INVALID, "lg_create: the pair-parallel force kernel takes at most %lld pair slots",
                       (long long)kPairsMaxSlots);
    if (s->kernel == LG_FORCE_KERNEL_PERSISTENT) LG_TRY(ensure_step_buffers(s));
    if (d->threads_per_row > 0 && d->force_kernel == LG_FORCE_KERNEL_AUTO) s->kernel = LG_FORCE_KERNEL_ROWGROUP;
    if (!arena) LG_TRY(apply_hold(s, d->hold_mask));
    LG_TRY(apply_unary(s, &d->body, d->unary_hook, d->unary_hook_user));
    // initial accelerations (the first half kick needs them); velocities are unchanged (hdt = 0)
    LG_TRY(launch_forces(s, 0.0, 0.0, 0));
    LG_CUDA(cudaStreamSynchronize(s->stream));
    return LG_OK;
}

extern "C" int lg_create(const lg_system_desc *desc, const double *x0, const double *v0, const double *theta0,
                         const double *omega0, const lg_facet_desc *facets, const double *neck_strengths,
                         int64_t n_neck_strengths, int device, lg_system **out) {
    if (!out) return lg_fail(LG_E_INVALID, "lg_create: null output handle");
    *out = nullptr;
    lg_system *s = new (std::nothrow) lg_system();
    if (!s) return lg_fail(LG_E_NOMEM, "lg_create: host allocation failed");
    int rc = create_impl(desc, x0, v0, theta0, omega0, facets, neck_strengths, n_neck_strengths, device, s);
    if (rc != LG_OK) {
        std::string keep = g_last_error;
        s->release();
        delete s;
        g_last_error = keep;
        return rc;
    }
    *out = s;
    return LG_OK;
}

extern "C" int lg_destroy(lg_system *s) {
    if (!s) return LG_OK;
    s->release();
    delete s;
    return LG_OK;
}

#define LG_HANDLE(s)                                                   \
    do {                                                               \
        if (!(s)) return lg_fail(LG_E_INVALID, "null system handle"); \
        LG_CUDA(cudaSetDevice((s)->device));                           \
    } while (0)

// Run `period` steps as one CUDA graph (captured on first use for this pointer parity). The host
// bookkeeping (buffer parities, step index) advances exactly as step_once advances it.
static int run_period_graph(lg_system *s, double dt, int64_t period, int64_t rebuild_every) {
    lg_system::GraphKey key{dt,      period,  s->kernel, s->T, s->vcur, s->pcur, s->fcur, s->ffcur, (int)(s->fstep & 1),
                            s->contact_lanes};
    for (auto &g : s->graphs) {
        if (!(g.key == key)) continue;
        LG_CUDA(cudaGraphLaunch(g.exec, s->stream));
        s->ffcur ^= g.ff_flips;
        s->fstep += g.f_launches;
        set_ff_buffers(s);
        // replay the host-side state transitions of `period` steps
        for (int64_t k = 0; k < period; ++k) {
            if (s->P.pairs == LG_PAIRS_VERLET && rebuild_every > 0 && (s->step_index % rebuild_every) == 0) {
                s->pcur = 1 - s->pcur;
                s->list_built = true;
            }
            s->vcur = 1 - s->vcur;
            if (s->facet_auto_move && s->P.n_facets > 0) s->fcur = 1 - s->fcur;
            s->step_index++;
        }
        s->launches += g.launches;
        return LG_OK;
    }
    const int64_t l0 = s->launches;
    const int ff0 = s->ffcur;
    const int64_t fs0 = s->fstep;
    LG_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    int rc = LG_OK;
    for (int64_t k = 0; k < period && rc == LG_OK; ++k) rc = step_once(s, dt, rebuild_every, k + 1 < period);
    cudaGraph_t graph = nullptr;
    cudaError_t ec = cudaStreamEndCapture(s->stream, &graph);
    if (rc != LG_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (ec != cudaSuccess) return lg_fail(LG_E_CUDA, "stream capture failed: %s", cudaGetErrorString(ec));
    cudaGraphExec_t exec = nullptr;
    ec = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ec != cudaSuccess) return lg_fail(LG_E_CUDA, "graph instantiation failed: %s", cudaGetErrorString(ec));
    s->graphs.push_back({key, exec, s->launches - l0, s->ffcur ^ ff0, s->fstep - fs0});
    LG_CUDA(cudaGraphLaunch(exec, s->stream));
    return LG_OK;
}

extern "C" int lg_step(lg_system *s, double dt, int64_t nsteps, int64_t rebuild_every) {
    LG_HANDLE(s);
    if (nsteps < 0) return lg_fail(LG_E_INVALID, "lg_step: nsteps < 0");
    if (!std::isfinite(dt)) return lg_fail(LG_E_INVALID, "lg_step: dt is not finite");
    const bool verlet = s->P.pairs == LG_PAIRS_VERLET;
    const int64_t period = (verlet && rebuild_every > 0) ? rebuild_every : 16;
    int64_t k = 0;
    while (k < nsteps) {
        const bool aligned = !(verlet && rebuild_every > 0) || (s->step_index % rebuild_every) == 0;
        if (s->use_graphs && !s->timing && aligned && nsteps - k >= period && s->periods_run > 0 && period <= 4096) {
            LG_TRY(run_period_graph(s, dt, period, rebuild_every));
            k += period;
            s->periods_run++;
            continue;
        }
        // eager steps: up to the next period boundary
        int64_t stop = nsteps;
        if (verlet && rebuild_every > 0) {
            const int64_t to_boundary = rebuild_every - (s->step_index % rebuild_every);
            stop = std::min<int64_t>(nsteps, k + to_boundary);
        } else {
            stop = std::min<int64_t>(nsteps, k + period);
        }
        for (; k < stop; ++k) LG_TRY(step_once(s, dt, rebuild_every, k + 1 < stop));
        s->periods_run++;
    }
    return LG_OK;
}

extern "C" int lg_set_graphs(lg_system *s, int32_t enable) {
    LG_HANDLE(s);
    s->use_graphs = enable != 0;
    if (!s->use_graphs) s->drop_graphs();
    return LG_OK;
}

extern "C" int lg_step_timed(lg_system *s, double dt, int64_t nsteps, int64_t rebuild_every, float *ms) {
    LG_HANDLE(s);
    if (!ms) return lg_fail(LG_E_INVALID, "lg_step_timed: null output");
    LG_CUDA(cudaEventRecord(s->ev0, s->stream));
    LG_TRY(lg_step(s, dt, nsteps, rebuild_every));
    LG_CUDA(cudaEventRecord(s->ev1, s->stream));
    LG_CUDA(cudaEventSynchronize(s->ev1));
    LG_CUDA(cudaEventElapsedTime(ms, s->ev0, s->ev1));
    return LG_OK;
}

extern "C" int lg_update_neighbor_list(lg_system *s) {
    LG_HANDLE(s);
    if (s->P.pairs != LG_PAIRS_VERLET) return LG_OK;
    return rebuild_list(s);
}

static dbl4 *field_ptr(lg_system *s, int field) {
    switch (field) {
        case LG_FIELD_X: return s->x;
        case LG_FIELD_V: return s->v[s->vcur];
        case LG_FIELD_THETA: return s->th;
        case LG_FIELD_OMEGA: return s->w[s->vcur];
        case LG_FIELD_A: return s->a;
        case LG_FIELD_ALPHA: return s->al;
        default: return nullptr;
    }
}

static int state_slot(int field) {
    switch (field) {
        case LG_FIELD_X: return 0;
        case LG_FIELD_V: return 1;
        case LG_FIELD_THETA: return 2;
        case LG_FIELD_OMEGA: return 3;
        default: return -1;
    }
}

static int state_upload(lg_system *s, const double *const host[4]);
static int state_download(lg_system *s, double *const host[4]);

extern "C" int lg_get(lg_system *s, int field, double *out) {
    LG_HANDLE(s);
    dbl4 *p = field_ptr(s, field);
    if (!p || !out) return lg_fail(LG_E_INVALID, "lg_get: bad field %d or null output", field);
    const int q = state_slot(field);
    if (q < 0) return download_staged(s, p, out);
    double *host[4] = {nullptr, nullptr, nullptr, nullptr};
    host[q] = out;
    return state_download(s, host);
}

extern "C" int lg_set(lg_system *s, int field, const double *in) {
    LG_HANDLE(s);
    dbl4 *p = field_ptr(s, field);
    if (!p || !in) return lg_fail(LG_E_INVALID, "lg_set: bad field %d or null input", field);
    const int q = state_slot(field);
    if (q < 0) return upload_staged(s, p, in);
    const double *host[4] = {nullptr, nullptr, nullptr, nullptr};
    host[q] = in;
    return state_upload(s, host);
}

// Device address of a caller's host buffer when it is pinned (the GPU then reads or writes it
// directly over the host link), or null for pageable memory (staged through device scratch).
static const void *mapped_host(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// 16-byte accesses for a transfer whose buffers all start on a 16-byte boundary.
static int32_t io_wide(const StateIO &io) {
    for (int f = 0; f < 4; ++f) {
        if ((reinterpret_cast<uintptr_t>(io.in[f]) | reinterpret_cast<uintptr_t>(io.out[f])) & 15u) return 0;
    }
    return 1;
}

// State upload of any of x, v, theta, omega (host [n][3] arrays, null: unchanged) in one kernel,
// which also refreshes the mixed path's float-float copies. The origins (and the CUDA graphs that
// hold them) are kept while every position stays within four times its system's extent from its
// origin; the kernel checks that, and only when it fails are the origins set up again from x.
static int state_upload(lg_system *s, const double *const host[4]) {
    if (!host[0] && !host[1] && !host[2] && !host[3]) return LG_OK;
    const int64_t n = s->P.n;
    const size_t bytes = sizeof(double) * 3 * (size_t)n;
    StateIO io{};
    for (int f = 0; f < 4; ++f) {
        if (!host[f]) continue;
        const void *m = mapped_host(host[f]);
        if (m) {
            io.in[f] = (const double *)m;
        } else {  // staged in the observables scratch (20 n doubles >= 4 x 3 n)
            LG_CUDA(cudaMemcpyAsync(s->obs_scratch + 3 * n * f, host[f], bytes, cudaMemcpyHostToDevice, s->stream));
            io.in[f] = s->obs_scratch + 3 * n * f;
        }
    }
    io.wide = io_wide(io);
    const bool refresh = s->x32 && (host[0] || host[1] || host[3]);
    // the coverage flag: written by the kernel straight into the handle's pinned word when that word
    // is mapped, else a device word copied back
    volatile int32_t *hflag = reinterpret_cast<volatile int32_t *>(s->h_pin + 63);
    int32_t *flag = nullptr;
    const bool want_flag = refresh && host[0];
    if (want_flag) {
        *hflag = 0;
        flag = s->pooled ? nullptr : (int32_t *)mapped_host((const void *)hflag);
        if (!flag) {
            flag = s->d_flag;
            LG_CUDA(cudaMemsetAsync(flag, 0, sizeof(int32_t), s->stream));
        }
    }
    launch_state_in(n, io, s->x, s->v[s->vcur], s->th, s->w[s->vcur], refresh ? s->x32 : nullptr, s->v32, s->s32,
                    s->origin, s->d_agg, s->d_orig, flag, s->stream);
    s->launches += 1;
    LG_CUDA(cudaGetLastError());
    if (flag && flag == s->d_flag)
        LG_CUDA(cudaMemcpyAsync((void *)hflag, flag, sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream));
    LG_CUDA(cudaStreamSynchronize(s->stream));  // the caller may reuse its buffers on return
    if (want_flag && *hflag) {
        LG_TRY(set_mixed_origins(s, host[0]));  // positions moved far: new origins and culling radii
        set_cull_radii(s);
        s->drop_graphs();
        launch_mixed_copies(n, s->x, s->v[s->vcur], s->w[s->vcur], s->th, s->origin, s->d_agg, s->d_orig, s->x32,
                            s->v32, s->s32, s->stream);
        s->launches += 1;
        LG_CUDA(cudaGetLastError());
        LG_CUDA(cudaStreamSynchronize(s->stream));
    }
    return LG_OK;
}

// State download into host [n][3] arrays (null: skipped), one kernel.
static int state_download(lg_system *s, double *const host[4]) {
    if (!host[0] && !host[1] && !host[2] && !host[3]) return LG_OK;
    const int64_t n = s->P.n;
    const size_t bytes = sizeof(double) * 3 * (size_t)n;
    StateIO io{};
    bool staged[4] = {false, false, false, false};
    for (int f = 0; f < 4; ++f) {
        if (!host[f]) continue;
        void *m = const_cast<void *>(mapped_host(host[f]));
        staged[f] = m == nullptr;
        io.out[f] = staged[f] ? s->obs_scratch + 3 * n * f : (double *)m;
    }
    io.wide = io_wide(io);
    launch_state_out(n, io, s->x, s->v[s->vcur], s->th, s->w[s->vcur], s->stream);
    s->launches += 1;
    LG_CUDA(cudaGetLastError());
    for (int f = 0; f < 4; ++f)
        if (staged[f])
            LG_CUDA(cudaMemcpyAsync(host[f], s->obs_scratch + 3 * n * f, bytes, cudaMemcpyDeviceToHost, s->stream));
    LG_CUDA(cudaStreamSynchronize(s->stream));
    return LG_OK;
}

extern "C" int lg_get_state(lg_system *s, double *x, double *v, double *th, double *w) {
    LG_HANDLE(s);
    double *const host[4] = {x, v, th, w};
    return state_download(s, host);
}

extern "C" int lg_set_state(lg_system *s, const double *x, const double *v, const double *th, const double *w) {
    LG_HANDLE(s);
    const double *const host[4] = {x, v, th, w};
    return state_upload(s, host);
}

extern "C" int lg_set_step_shape(lg_system *s, int32_t min_blocks, int32_t slices, int32_t assign) {
    LG_HANDLE(s);
    if (s->precision != LG_PRECISION_MIXED) return lg_fail(LG_E_INVALID, "lg_set_step_shape: mixed precision only");
    if (min_blocks != 0 && min_blocks != 4 && min_blocks != 5 && min_blocks != 6)
        return lg_fail(LG_E_INVALID, "lg_set_step_shape: min_blocks must be 0, 4, 5 or 6");
    if (slices != 0 && slices != 1 && slices != 2 && slices != 4)
        return lg_fail(LG_E_INVALID, "lg_set_step_shape: slices must be 0, 1, 2 or 4");
    if (assign < 0 || assign > 2) return lg_fail(LG_E_INVALID, "lg_set_step_shape: assign must be 0, 1 or 2");
    LG_TRY(ensure_step_buffers(s));
    s->step_min_blocks = min_blocks ? min_blocks : 4;
    s->step_slices = slices ? slices : mixed_hamaker_slices(s->P.n);
    s->ham_slices = slices;  // the two-stream kernels follow an explicit slice count too
    s->step_assign = assign;
    s->drop_graphs();  // the graphs hold the previous shape's launches
    return LG_OK;
}

extern "C" int lg_get_step_shape(lg_system *s, int32_t *min_blocks, int32_t *slices, int32_t *assign) {
    LG_HANDLE(s);
    if (min_blocks) *min_blocks = s->step_min_blocks;
    if (slices) *slices = s->step_slices ? s->step_slices : mixed_hamaker_slices(s->P.n);
    if (assign) *assign = s->step_assign;
    return LG_OK;
}

extern "C" int lg_set_threads_per_row(lg_system *s, int32_t T) {
    LG_HANDLE(s);
    if (T == 0) {
        s->T = choose_threads_per_row(s);
        return LG_OK;
    }
    if (T != 1 && T != 2 && T != 4 && T != 8 && T != 16 && T != 32)
        return lg_fail(LG_E_INVALID, "lg_set_threads_per_row: T must be 0 or a power of two <= 32");
    s->T = T;
    return LG_OK;
}

extern "C" int lg_set_force_kernel(lg_system *s, int32_t variant) {
    LG_HANDLE(s);
    if (variant < 0 || variant > 5) return lg_fail(LG_E_INVALID, "lg_set_force_kernel: unknown variant %d", variant);
    const int k = choose_kernel(s, variant);
    if (k < 0 && variant == LG_FORCE_KERNEL_PERSISTENT)
        return lg_fail(LG_E_INVALID, "lg_set_force_kernel: the persistent step kernel is mixed precision only");
    if (k < 0 && variant == LG_FORCE_KERNEL_FP64_FAST)
        return lg_fail(LG_E_INVALID, "lg_set_force_kernel: the fast FP64 kernel is FP64 precision only");
    if (k < 0)
        return lg_fail(LG_E_INVALID, "lg_set_force_kernel: the pair-parallel kernel is FP64 only and takes at most "
                       "%lld pair slots", (long long)kPairsMaxSlots);
    if (k == LG_FORCE_KERNEL_PERSISTENT) LG_TRY(ensure_step_buffers(s));
    s->kernel = k;
    s->tuned_ms = 0.0;
    return LG_OK;
}

extern "C" int lg_set_hold_mask(lg_system *s, const uint8_t *mask) {
    LG_HANDLE(s);
    return apply_hold(s, mask);
}

extern "C" int lg_set_body_force(lg_system *s, const lg_body_force *force) {
    LG_HANDLE(s);
    return apply_unary(s, force, nullptr, nullptr);
}

extern "C" int lg_set_body_centre(lg_system *s, const double *centres) {
    LG_HANDLE(s);
    if (!centres) return lg_fail(LG_E_INVALID, "lg_set_body_centre: null centres");
    if (s->body.model != LG_BODY_CENTRAL) return lg_fail(LG_E_STATE, "lg_set_body_centre: no central body force is set");
    const int64_t nsys = std::max<int64_t>(1, s->n_systems);
    for (int64_t q = 0; q < 3 * nsys; ++q)
        if (!std::isfinite(centres[q])) return lg_fail(LG_E_INVALID, "lg_set_body_centre: centre %lld is not finite", (long long)(q / 3));
    LG_CUDA(cudaMemcpyAsync(s->d_centre, centres, sizeof(double) * 3 * (size_t)nsys, cudaMemcpyHostToDevice, s->stream));
    LG_CUDA(cudaStreamSynchronize(s->stream));
    return LG_OK;
}

extern "C" int lg_set_unary_hook(lg_system *s, lg_unary_hook hook, void *user) {
    LG_HANDLE(s);
    return apply_unary(s, nullptr, hook, user);
}

extern "C" int lg_reset_acceleration_buffers(lg_system *s) {
    LG_HANDLE(s);
    LG_CUDA(cudaMemsetAsync(s->a, 0, sizeof(dbl4) * s->P.n, s->stream));
    LG_CUDA(cudaMemsetAsync(s->al, 0, sizeof(dbl4) * s->P.n, s->stream));
    return LG_OK;
}

extern "C" int lg_get_device_errors(lg_system *s, int32_t *errors) {
    LG_HANDLE(s);
    if (!errors) return lg_fail(LG_E_INVALID, "lg_get_device_errors: null output");
    LG_CUDA(cudaMemcpyAsync(errors, s->err, sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream));
    LG_CUDA(cudaStreamSynchronize(s->stream));
    return LG_OK;
}

extern "C" int lg_get_observables_select(lg_system *s, int32_t parts, lg_observables *o) {
    LG_HANDLE(s);
    if (!o) return lg_fail(LG_E_INVALID, "lg_get_observables: null output");
    if (parts & ~(LG_OBS_STATE | LG_OBS_PAIRS)) return lg_fail(LG_E_INVALID, "lg_get_observables: unknown parts %d", parts);
    const Params &P = s->P;
    double m, I;
    if (P.binary_model == LG_BINARY_SINTER || P.binary_model == LG_BINARY_BREAKING_SINTER) {
        m = P.sinter.mass;
        I = P.sinter.inertia;
    } else if (P.binary_model == LG_BINARY_CONTACT || P.binary_model == LG_BINARY_SINTER_CONNECTORS) {
        m = P.contact.mass;
        I = P.contact.inertia;
    } else {
        m = P.hamaker.mass;
        I = P.contact.inertia;
    }
    memset(o, 0, sizeof(*o));
    o->n_bonds_initial = s->n_bonds_initial;
    if (!parts) return LG_OK;
    // every pass stays on the device; one copy back at the end
    StateView S = state_view(s, false);
    if (parts & LG_OBS_STATE) {
        launch_observables_state(P.n, s->x, s->v[s->vcur], s->w[s->vcur], m, I, s->obs_scratch, s->obs_out, s->d_ticket,
                                 s->stream);
        s->launches += 2;
    }
    if (parts & LG_OBS_PAIRS) {
        launch_observables_pairs(P, S, s->pv[s->pcur], s->bv, m, I, s->obs_scratch, s->obs_out, s->stream);
        s->launches += 2;
    }
    LG_CUDA(cudaGetLastError());
    LG_CUDA(cudaMemcpyAsync(s->h_pin, s->obs_out, sizeof(double) * 19, cudaMemcpyDeviceToHost, s->stream));
    LG_CUDA(cudaStreamSynchronize(s->stream));
    double h[19];
    std::memcpy(h, s->h_pin, sizeof(h));
    const double nn = (double)P.n;
    if (parts & LG_OBS_STATE) {
        o->ke_total = h[0];
        o->ke_translational = h[1] / 2.0;
        o->ke_rotational = h[2] / 2.0;
        o->linear_momentum = m * std::sqrt((h[3] * h[3] + h[4] * h[4]) + h[5] * h[5]);
        double L[3] = {h[6] + h[9], h[7] + h[10], h[8] + h[11]};
        o->angular_momentum = std::sqrt((L[0] * L[0] + L[1] * L[1]) + L[2] * L[2]);
        for (int k = 0; k < 3; ++k) o->center_of_mass[k] = h[12 + k] / nn;
        o->radius_of_gyration = std::sqrt(h[18] / nn);
    }
    if (parts & LG_OBS_PAIRS) {
        o->potential_energy = h[15];
        o->n_contacts = (int64_t)h[16];
        o->n_bonds = (int64_t)h[17];
    }
    return LG_OK;
}

extern "C" int lg_get_observables(lg_system *s, lg_observables *o) {
    return lg_get_observables_select(s, LG_OBS_STATE | LG_OBS_PAIRS, o);
}

extern "C" int lg_get_bonds(lg_system *s, int64_t *n_bonds, int64_t *pairs, int64_t cap) {
    LG_HANDLE(s);
    if (!n_bonds) return lg_fail(LG_E_INVALID, "lg_get_bonds: null count");
    const int64_t n = s->P.n;
    const size_t bs = (size_t)s->bv.bcap * (size_t)n;
    std::vector<int8_t> intact(bs);
    LG_CUDA(cudaMemcpyAsync(intact.data(), s->bv.intact, bs, cudaMemcpyDeviceToHost, s->stream));
    LG_CUDA(cudaStreamSynchronize(s->stream));
    std::vector<std::pair<int64_t, int64_t>> out;
    for (size_t b = 0; b < (size_t)s->bv.bcap; ++b)
        for (int64_t i = 0; i < n; ++i) {
            size_t e = b * (size_t)n + (size_t)i;
            if (s->host_bond_j[e] >= 0 && intact[e]) out.emplace_back(i, s->host_bond_j[e]);
        }
    std::sort(out.begin(), out.end());
    *n_bonds = (int64_t)out.size();
    if (pairs)
        for (int64_t k = 0; k < (int64_t)out.size() && k < cap; ++k) {
            pairs[2 * k] = out[k].first;
            pairs[2 * k + 1] = out[k].second;
        }
    return LG_OK;
}

// Raw 8-byte spring slots -> values: mixed-precision handles store float-float pairs (hi, lo).
static void spring_values(const lg_system *s, double *v9) {
    if (!s->P.springs_ff) return;
    for (int q = 0; q < 9; ++q) {
        float hl[2];
        std::memcpy(hl, &v9[q], sizeof(hl));
        v9[q] = (double)hl[0] + (double)hl[1];
    }
}

extern "C" int lg_get_pair_springs(lg_system *s, int64_t i, int64_t j, double *out9) {
    LG_HANDLE(s);
    if (!out9) return lg_fail(LG_E_INVALID, "lg_get_pair_springs: null output");
    const int64_t n = s->P.n;
    if (i < 0 || j < 0 || i >= n || j >= n || i == j) return lg_fail(LG_E_INVALID, "lg_get_pair_springs: bad pair");
    for (int q = 0; q < 9; ++q) out9[q] = 0.0;
    LG_CUDA(cudaStreamSynchronize(s->stream));
    // an intact bond reports its bond springs
    for (int b = 0; b < s->bv.bcap; ++b) {
        size_t be = (size_t)b * n + i;
        if (s->host_bond_j[be] != j) continue;
        int8_t in = 0;
        LG_CUDA(cudaMemcpy(&in, s->bv.intact + be, 1, cudaMemcpyDeviceToHost));
        if (in) {
            const size_t bs = (size_t)s->bv.bcap * n;
            for (int q = 0; q < 9; ++q)
                LG_CUDA(cudaMemcpy(out9 + q, s->bv.xi + spring_at(s->bv.aos, q, be, bs), sizeof(double), cudaMemcpyDeviceToHost));
            spring_values(s, out9);
            return LG_OK;
        }
    }
    const PairView &pv = s->pv[s->pcur];
    int64_t k = -1;
    if (s->P.pairs == LG_PAIRS_ALL) {
        k = j < i ? j : j - 1;
    } else {
        int32_t len = 0;
        LG_CUDA(cudaMemcpy(&len, pv.row_len + i, sizeof(int32_t), cudaMemcpyDeviceToHost));
        for (int64_t q = 0; q < len; ++q) {
            int32_t jj = 0;
            LG_CUDA(cudaMemcpy(&jj, pv.nbr + q * n + i, sizeof(int32_t), cudaMemcpyDeviceToHost));
            if (jj == j) {
                k = q;
                break;
            }
        }
    }
    if (k < 0) return LG_OK;
    const size_t e = (size_t)(k * n + i), xs = (size_t)(pv.cap * n);
    uint32_t fl = 0;
    LG_CUDA(cudaMemcpy(&fl, pv.flags + e, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (!(fl & kXiLive)) return LG_OK;  // springs of a slot that is not live are zero
    for (int q = 0; q < 9; ++q)
        LG_CUDA(cudaMemcpy(out9 + q, pv.xi + spring_at(pv.aos, q, e, xs), sizeof(double), cudaMemcpyDeviceToHost));
    spring_values(s, out9);
    return LG_OK;
}

extern "C" int lg_facet_update_positions(lg_system *s, int32_t facet, double dt) {
    LG_HANDLE(s);
    if (facet < 0 || facet >= s->P.n_facets) return lg_fail(LG_E_INVALID, "lg_facet_update_positions: bad facet");
    double h[9];
    LG_CUDA(cudaMemcpyAsync(h, s->fv[s->fcur] + 9 * facet, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
    LG_CUDA(cudaStreamSynchronize(s->stream));
    for (int q = 0; q < 9; ++q) h[q] = h[q] + s->P.facets[facet].v[q % 3] * dt;
    LG_CUDA(cudaMemcpyAsync(s->fv[s->fcur] + 9 * facet, h, sizeof(h), cudaMemcpyHostToDevice, s->stream));
    LG_CUDA(cudaStreamSynchronize(s->stream));
    return LG_OK;
}

extern "C" int lg_facet_get_vertices(lg_system *s, int32_t facet, double *out9) {
    LG_HANDLE(s);
    if (facet < 0 || facet >= s->P.n_facets || !out9) return lg_fail(LG_E_INVALID, "lg_facet_get_vertices: bad facet");
    LG_CUDA(cudaMemcpyAsync(out9, s->fv[s->fcur] + 9 * facet, sizeof(double) * 9, cudaMemcpyDeviceToHost, s->stream));
    LG_CUDA(cudaStreamSynchronize(s->stream));
    return LG_OK;
}

extern "C" int lg_get_launch_count(lg_system *s, int64_t *count) {
    if (!s || !count) return lg_fail(LG_E_INVALID, "lg_get_launch_count: null argument");
    *count = s->launches;
    return LG_OK;
}

extern "C" int lg_enable_kernel_timing(lg_system *s, int32_t enable) {
    LG_HANDLE(s);
    LG_CUDA(cudaStreamSynchronize(s->stream));
    s->timing = enable != 0;
    s->tev_used = 0;
    return LG_OK;
}

extern "C" int lg_get_force_kernel_time(lg_system *s, double *ms_total, int64_t *launches) {
    LG_HANDLE(s);
    if (!ms_total || !launches) return lg_fail(LG_E_INVALID, "lg_get_force_kernel_time: null output");
    LG_CUDA(cudaStreamSynchronize(s->stream));
    double tot = 0.0;
    for (size_t q = 0; q + 1 < s->tev_used; q += 2) {
        float ms = 0.f;
        LG_CUDA(cudaEventElapsedTime(&ms, s->tev[q], s->tev[q + 1]));
        tot += ms;
    }
    *ms_total = tot;
    *launches = (int64_t)(s->tev_used / 2);
    s->tev_used = 0;
    return LG_OK;
}

extern "C" int lg_get_pair_stats(lg_system *s, lg_pair_stats *out) {
    LG_HANDLE(s);
    if (!out) return lg_fail(LG_E_INVALID, "lg_get_pair_stats: null output");
    const int64_t n = s->P.n;
    const PairView &pv = s->pv[s->pcur];
    LG_CUDA(cudaStreamSynchronize(s->stream));
    std::vector<int32_t> len((size_t)n, (int32_t)(n - 1));
    if (s->P.pairs == LG_PAIRS_VERLET)
        LG_CUDA(cudaMemcpy(len.data(), pv.row_len, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
    std::vector<uint32_t> fl((size_t)(pv.cap * n));
    LG_CUDA(cudaMemcpy(fl.data(), pv.flags, sizeof(uint32_t) * fl.size(), cudaMemcpyDeviceToHost));
    double sum = 0.0;
    int64_t mx = 0, live = 0, bonded = 0;
    for (int64_t i = 0; i < n; ++i) {
        sum += len[i];
        mx = std::max<int64_t>(mx, len[i]);
        for (int64_t k = 0; k < len[i]; ++k) {
            uint32_t f = fl[(size_t)(k * n + i)];
            if (f & kBonded) ++bonded;
            else if (f & kXiLive) ++live;
        }
    }
    out->mean_row_length = sum / (double)n;
    out->max_row_length = mx;
    out->live_contact_slots = live;
    out->bonded_slots = bonded;
    return LG_OK;
}

// ------------------------------------------------------------------------------------------------
// Batches
// ------------------------------------------------------------------------------------------------
extern "C" int lg_batch_create(const lg_system_desc *desc, int64_t n_systems, const int64_t *sizes, const double *x0,
                               const double *v0, const double *theta0, const double *omega0,
                               const lg_facet_desc *facets, const double *neck_strengths, int64_t n_neck_strengths,
                               int device, lg_system **out) {
    if (!out) return lg_fail(LG_E_INVALID, "lg_batch_create: null output handle");
    *out = nullptr;
    if (n_systems < 1) return lg_fail(LG_E_INVALID, "lg_batch_create: n_systems < 1");
    lg_system *s = new (std::nothrow) lg_system();
    if (!s) return lg_fail(LG_E_NOMEM, "lg_batch_create: host allocation failed");
    int rc = create_impl(desc, x0, v0, theta0, omega0, facets, neck_strengths, n_neck_strengths, device, s, n_systems,
                         sizes);
    if (rc != LG_OK) {
        std::string keep = g_last_error;
        s->release();
        delete s;
        g_last_error = keep;
        return rc;
    }
    *out = s;
    return LG_OK;
}

extern "C" int lg_batch_info(lg_system *s, int64_t *n_systems, int64_t *offsets) {
    LG_HANDLE(s);
    if (!n_systems) return lg_fail(LG_E_INVALID, "lg_batch_info: null count");
    *n_systems = s->n_systems;
    if (offsets)
        for (int64_t q = 0; q <= s->n_systems; ++q) offsets[q] = s->sys_off[q];
    return LG_OK;
}

// Observables of every system of a batch (out[n_systems]).
extern "C" int lg_batch_get_observables(lg_system *s, lg_observables *out) {
    LG_HANDLE(s);
    if (!out) return lg_fail(LG_E_INVALID, "lg_batch_get_observables: null output");
    if (s->n_systems == 0) return lg_get_observables(s, out);
    const Params &P = s->P;
    const bool sint = P.binary_model == LG_BINARY_SINTER || P.binary_model == LG_BINARY_BREAKING_SINTER;
    const bool cmass = P.binary_model == LG_BINARY_CONTACT || P.binary_model == LG_BINARY_SINTER_CONNECTORS;
    const double m = sint ? P.sinter.mass : (cmass ? P.contact.mass : P.hamaker.mass);
    const double I = sint ? P.sinter.inertia : P.contact.inertia;
    StateView S = state_view(s, false);
    // per-particle rows (the single-system reduction is launched too; its result is unused)
    launch_observables(P, S, s->pv[s->pcur], s->bv, m, I, s->obs_scratch, s->obs_out, s->stream);
    launch_segmented_sums(s->n_systems, s->d_sys_off, s->obs_scratch, s->d_sys_obs, s->stream);
    s->launches += 3;
    LG_CUDA(cudaGetLastError());
    const int64_t ns = s->n_systems;
    std::vector<double> h((size_t)(20 * ns));
    LG_CUDA(cudaMemcpyAsync(h.data(), s->d_sys_obs, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s->stream));
    LG_CUDA(cudaStreamSynchronize(s->stream));
    std::vector<double> c((size_t)(3 * ns));
    for (int64_t q = 0; q < ns; ++q) {
        const double nn = (double)(s->sys_off[q + 1] - s->sys_off[q]);
        for (int k = 0; k < 3; ++k) c[3 * q + k] = h[20 * q + 12 + k] / nn;
    }
    LG_CUDA(cudaMemcpyAsync(s->d_centres, c.data(), sizeof(double) * c.size(), cudaMemcpyHostToDevice, s->stream));
    launch_segmented_rg(P.n, ns, s->d_sys_off, s->x, s->d_centres, s->obs_scratch, s->d_sys_obs, s->stream);
    s->launches += 1;
    LG_CUDA(cudaGetLastError());
    LG_CUDA(cudaMemcpyAsync(h.data(), s->d_sys_obs, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s->stream));
    LG_CUDA(cudaStreamSynchronize(s->stream));
    for (int64_t q = 0; q < ns; ++q) {
        const double *hq = h.data() + 20 * q;
        const double nn = (double)(s->sys_off[q + 1] - s->sys_off[q]);
        lg_observables &o = out[q];
        memset(&o, 0, sizeof(o));
        o.ke_total = hq[0];
        o.ke_translational = hq[1] / 2.0;
        o.ke_rotational = hq[2] / 2.0;
        o.linear_momentum = m * std::sqrt((hq[3] * hq[3] + hq[4] * hq[4]) + hq[5] * hq[5]);
        double L[3] = {hq[6] + hq[9], hq[7] + hq[10], hq[8] + hq[11]};
        o.angular_momentum = std::sqrt((L[0] * L[0] + L[1] * L[1]) + L[2] * L[2]);
        for (int k = 0; k < 3; ++k) o.center_of_mass[k] = c[3 * q + k];
        o.radius_of_gyration = std::sqrt(hq[18] / nn);
        o.potential_energy = hq[15];
        o.n_contacts = (int64_t)hq[16];
        o.n_bonds = (int64_t)hq[17];
        o.n_bonds_initial = s->n_bonds_initial_sys.empty() ? 0 : s->n_bonds_initial_sys[q];
    }
    return LG_OK;
}

// ------------------------------------------------------------------------------------------------
// Serving slots: a batch handle whose systems are slots that requests occupy in turn
// ------------------------------------------------------------------------------------------------
// Radius bound of a seeded aggregate of `cap` spheres about its centroid, with room to spread: the
// random-sequential-attachment aggregates measure about 3 r cap^0.3 (8192 spheres: 40 r), and the
// bound takes 1.5 times that (at least 8 r).
double lg_arena_radius_bound(int64_t cap, double r_part) {
    return std::max(8.0 * r_part, 1.5 * 3.0 * r_part * std::pow((double)std::max<int64_t>(cap, 1), 0.3));
}

int lg_arena_create(const lg_system_desc *tmpl, int64_t n_slots, const int64_t *caps, int device, lg_system **out) {
    if (!tmpl || !caps || !out || n_slots < 1) return lg_fail(LG_E_INVALID, "lg_arena_create: bad arguments");
    *out = nullptr;
    if (tmpl->pairs != LG_PAIRS_VERLET) return lg_fail(LG_E_INVALID, "serving slots need LG_PAIRS_VERLET");
    if (tmpl->n_facets != 0 || tmpl->hold_mask || tmpl->unary_hook || tmpl->body.model != LG_BODY_NONE)
        return lg_fail(LG_E_INVALID, "serving slots hold no facets, hold masks or unary terms");
    int64_t n = 0, cmax = 0;
    for (int64_t q = 0; q < n_slots; ++q) {
        if (caps[q] < 1) return lg_fail(LG_E_INVALID, "lg_arena_create: slot %lld has capacity %lld", (long long)q, (long long)caps[q]);
        n += caps[q];
        cmax = std::max(cmax, caps[q]);
    }
    lg_system_desc d = *tmpl;
    d.n_part = n;
    if (d.max_neighbors <= 0) d.max_neighbors = 96;  // imports need the standalone handles' row capacity
    d.force_kernel = LG_FORCE_KERNEL_COMPACT;
    d.threads_per_row = 0;
    const double r = std::max(d.contact.r_part, std::max(d.sinter.r_part, d.hamaker.r_part));
    const double R = lg_arena_radius_bound(cmax, r);
    ArenaSpec spec{16, 2.0 * R + 2.0 * d.r_verlet + 8.0 * r, R + 8.0 * r};
    int64_t m = 1;
    while (m * m * m < n_slots) ++m;
    std::vector<double> pos(3 * (size_t)n_slots), x0(3 * (size_t)n), zero(3 * (size_t)n, 0.0);
    int64_t k = 0;
    for (int64_t q = 0; q < n_slots; ++q) {
        pos[3 * q] = (double)(q % m) * spec.lattice;
        pos[3 * q + 1] = (double)((q / m) % m) * spec.lattice;
        pos[3 * q + 2] = (double)(q / (m * m)) * spec.lattice;
        for (int64_t i = 0; i < caps[q]; ++i, ++k)
            for (int c = 0; c < 3; ++c) x0[3 * k + c] = pos[3 * q + c];
    }
    lg_system *s = new (std::nothrow) lg_system();
    if (!s) return lg_fail(LG_E_NOMEM, "lg_arena_create: host allocation failed");
    int rc = create_impl(&d, x0.data(), zero.data(), zero.data(), zero.data(), nullptr, nullptr, 0, device, s, n_slots,
                         caps, &spec);
    if (rc != LG_OK) {
        std::string keep = g_last_error;
        s->release();
        delete s;
        g_last_error = keep;
        return rc;
    }
    s->arena = true;
    s->arena_lattice = spec.lattice;
    s->slot_pos = std::move(pos);
    *out = s;
    return LG_OK;
}

int lg_create_staged(const lg_system_desc *desc, const double *x0, const double *v0, int device, lg_system **out) {
    if (!desc || !x0 || !v0 || !out) return lg_fail(LG_E_INVALID, "lg_create_staged: bad arguments");
    *out = nullptr;
    lg_system *s = new (std::nothrow) lg_system();
    if (!s) return lg_fail(LG_E_NOMEM, "lg_create_staged: host allocation failed");
    s->pooled = true;
    static std::mutex pool_mu;
    static std::vector<int> pool_set;  // devices whose default pool keeps freed memory for reuse
    {
        std::lock_guard<std::mutex> lk(pool_mu);
        if (std::find(pool_set.begin(), pool_set.end(), device) == pool_set.end()) {
            cudaMemPool_t pool = nullptr;
            if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
                uint64_t keep = UINT64_MAX;
                cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
            }
            cudaGetLastError();
            pool_set.push_back(device);
        }
    }
    const std::vector<double> zeros(3 * (size_t)std::max<int64_t>(desc->n_part, 1), 0.0);
    int rc = create_impl(desc, x0, v0, zeros.data(), zeros.data(), nullptr, nullptr, 0, device, s);
    if (rc != LG_OK) {
        std::string keep = g_last_error;
        s->release();
        delete s;
        g_last_error = keep;
        return rc;
    }
    *out = s;
    return LG_OK;
}

int lg_arena_import(lg_system *A, int64_t q, lg_system *S, const double *x0) {
    if (!A || !S || !x0 || !A->arena || q < 0 || q >= A->n_systems)
        return lg_fail(LG_E_INVALID, "lg_arena_import: bad arguments");
    const int64_t off = A->sys_off[q], C = A->sys_off[q + 1] - off, n = S->P.n, N = A->P.n;
    if (S->n_systems != 0 || n > C || S->precision != A->precision || S->P.binary_model != A->P.binary_model ||
        S->P.hamaker_model != A->P.hamaker_model || S->P.pairs != LG_PAIRS_VERLET || S->pv[0].cap > A->pv[0].cap ||
        S->bv.bcap > A->bv.bcap || S->bv.aos != A->bv.aos || (S->pv[0].near_len != nullptr) != (A->pv[0].near_len != nullptr) ||
        S->bv.cn || S->kick_done || A->kick_done)
        return lg_fail(LG_E_INVALID, "lg_arena_import: the request does not fit slot %lld (n %lld of %lld, %d of %d bond "
                       "slots, %lld of %lld row slots)", (long long)q, (long long)n, (long long)C, S->bv.bcap, A->bv.bcap,
                       (long long)S->pv[0].cap, (long long)A->pv[0].cap);
    double c[3] = {0.0, 0.0, 0.0}, rad = 0.0;
    for (int k = 0; k < 3; ++k) {
        for (int64_t i = 0; i < n; ++i) c[k] += x0[3 * i + k];
        c[k] /= (double)n;
    }
    for (int64_t i = 0; i < n; ++i) {
        double r2 = 0.0;
        for (int k = 0; k < 3; ++k) r2 += (x0[3 * i + k] - c[k]) * (x0[3 * i + k] - c[k]);
        rad = std::max(rad, std::sqrt(r2));
    }
    if (rad > 0.5 * A->arena_lattice - A->P.r_verlet)
        return lg_fail(LG_E_INVALID, "lg_arena_import: the aggregate (radius %g) is too wide for the slot lattice (%g)", rad,
                       A->arena_lattice);
    LG_CUDA(cudaStreamSynchronize(S->stream));
    const cudaStream_t st = A->stream;
    const int64_t tail = C - n;
    auto cp = [&](void *dst, const void *src, size_t bytes) {
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st);
    };
    auto cp2 = [&](void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, size_t height) {
        return height == 0 ? cudaSuccess : cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, height, cudaMemcpyDeviceToDevice, st);
    };
    const size_t d4 = sizeof(dbl4);
    // state of the occupant; the rest of the slot at its centroid, at rest
    LG_CUDA(cp(A->x + off, S->x, d4 * n));
    LG_CUDA(cp(A->th + off, S->th, d4 * n));
    LG_CUDA(cp(A->a + off, S->a, d4 * n));
    LG_CUDA(cp(A->al + off, S->al, d4 * n));
    LG_CUDA(cp(A->v[A->vcur] + off, S->v[S->vcur], d4 * n));
    LG_CUDA(cp(A->w[A->vcur] + off, S->w[S->vcur], d4 * n));
    launch_fill_dbl4(A->x + off + n, tail, c[0], c[1], c[2], st);
    for (dbl4 *p : {A->th, A->a, A->al, A->v[0], A->v[1], A->w[0], A->w[1]})
        LG_CUDA(cudaMemsetAsync(p + off + n, 0, d4 * tail, st));
    // hold bits: the occupant's (none in a request template), inactive for the rest
    std::vector<uint8_t> hold((size_t)C, (uint8_t)kHoldInactive);
    if (S->P.hold) LG_CUDA(cudaMemcpy(hold.data(), S->P.hold, (size_t)n, cudaMemcpyDeviceToHost));
    else std::fill(hold.begin(), hold.begin() + n, (uint8_t)0);
    LG_CUDA(cudaMemcpyAsync(A->d_hold + off, hold.data(), (size_t)C, cudaMemcpyHostToDevice, st));
    // bonds (bond slot b of particle i at b * N + i), partners moved by the slot offset
    const int32_t ba = A->bv.bcap, bsz = S->bv.bcap;
    LG_CUDA(cudaMemset2DAsync(A->bv.j + off, sizeof(int32_t) * N, 0xFF, sizeof(int32_t) * C, ba, st));
    LG_CUDA(cudaMemset2DAsync(A->bv.intact + off, (size_t)N, 0, (size_t)C, ba, st));
    LG_CUDA(cp2(A->bv.j + off, sizeof(int32_t) * N, S->bv.j, sizeof(int32_t) * n, sizeof(int32_t) * n, bsz));
    launch_offset_indices(A->bv.j + off, bsz, N, n, (int32_t)off, st);
    LG_CUDA(cp2(A->bv.intact + off, (size_t)N, S->bv.intact, (size_t)n, (size_t)n, bsz));
    LG_CUDA(cp2(A->bv.strength + off, sizeof(double) * N, S->bv.strength, sizeof(double) * n, sizeof(double) * n, bsz));
    if (A->bv.aos) {  // one 9-component record per bond slot
        LG_CUDA(cp2(A->bv.xi + 9 * off, 72 * (size_t)N, S->bv.xi, 72 * (size_t)n, 72 * (size_t)n, bsz));
    } else {
        for (int k = 0; k < 9; ++k)
            LG_CUDA(cp2(A->bv.xi + (size_t)k * ba * N + off, sizeof(double) * N, S->bv.xi + (size_t)k * bsz * n,
                        sizeof(double) * n, sizeof(double) * n, bsz));
    }
    for (int64_t b = 0; b < ba; ++b)
        for (int64_t i = 0; i < C; ++i) {
            int32_t j = -1;
            if (b < bsz && i < n && S->host_bond_j[(size_t)(b * n + i)] >= 0) j = S->host_bond_j[(size_t)(b * n + i)] + (int32_t)off;
            A->host_bond_j[(size_t)(b * N + off + i)] = j;
        }
    // pair rows (slot k of row i at k * N + i) with their springs, partners moved by the offset; a
    // small system's rows hold fewer slots (n - 1), and no row is longer than its capacity
    PairView &PA = A->pv[A->pcur];
    const PairView &PS = S->pv[S->pcur];
    const int64_t cap = PS.cap;
    LG_CUDA(cp2(PA.nbr + off, sizeof(int32_t) * N, PS.nbr, sizeof(int32_t) * n, sizeof(int32_t) * n, cap));
    launch_offset_indices(PA.nbr + off, cap, N, n, (int32_t)off, st);
    LG_CUDA(cp(PA.row_len + off, PS.row_len, sizeof(int32_t) * n));
    LG_CUDA(cudaMemsetAsync(PA.row_len + off + n, 0, sizeof(int32_t) * tail, st));
    LG_CUDA(cp2(PA.flags + off, sizeof(uint32_t) * N, PS.flags, sizeof(uint32_t) * n, sizeof(uint32_t) * n, cap));
    if (PA.aos) {
        LG_CUDA(cp2(PA.xi + 9 * off, 72 * (size_t)N, PS.xi, 72 * (size_t)n, 72 * (size_t)n, cap));
    } else {
        for (int k = 0; k < 9; ++k)
            LG_CUDA(cp2(PA.xi + (size_t)k * PA.cap * N + off, sizeof(double) * N, PS.xi + (size_t)k * cap * n,
                        sizeof(double) * n, sizeof(double) * n, cap));
    }
    if (PA.near_len) {
        LG_CUDA(cp2(PA.near_j + off, sizeof(int32_t) * N, PS.near_j, sizeof(int32_t) * n, sizeof(int32_t) * n, cap));
        launch_offset_indices(PA.near_j + off, cap, N, n, (int32_t)off, st);
        LG_CUDA(cp2(PA.near_k + off, (size_t)N, PS.near_k, (size_t)n, (size_t)n, cap));
        LG_CUDA(cp(PA.near_len + off, PS.near_len, sizeof(int32_t) * n));
        LG_CUDA(cudaMemsetAsync(PA.near_len + off + n, 0, sizeof(int32_t) * tail, st));
    }
    // float-float origin (the standalone handle's) and hashing offset to the slot's lattice point
    dbl4 orig = make_double4_32a(S->origin[0], S->origin[1], S->origin[2], S->origin[3]);
    const dbl4 hoff = make_double4_32a(A->slot_pos[3 * q] - c[0], A->slot_pos[3 * q + 1] - c[1],
                                       A->slot_pos[3 * q + 2] - c[2], 0.0);
    if (A->precision == LG_PRECISION_MIXED) {
        A->h_orig[(size_t)q] = orig;
        LG_CUDA(cudaMemcpyAsync(A->d_orig + q, &orig, d4, cudaMemcpyHostToDevice, st));
    }
    LG_CUDA(cudaMemcpyAsync(A->d_hoff + q, &hoff, d4, cudaMemcpyHostToDevice, st));
    A->n_bonds_initial_sys[(size_t)q] = S->n_bonds_initial;
    LG_CUDA(cudaGetLastError());
    LG_CUDA(cudaStreamSynchronize(st));  // host buffers above are released on return
    return LG_OK;
}

int lg_arena_clear(lg_system *A, int64_t q) {
    if (!A || !A->arena || q < 0 || q >= A->n_systems) return lg_fail(LG_E_INVALID, "lg_arena_clear: bad arguments");
    const int64_t off = A->sys_off[q], C = A->sys_off[q + 1] - off, N = A->P.n;
    const cudaStream_t st = A->stream;
    const size_t d4 = sizeof(dbl4);
    launch_fill_dbl4(A->x + off, C, A->slot_pos[3 * q], A->slot_pos[3 * q + 1], A->slot_pos[3 * q + 2], st);
    for (dbl4 *p : {A->th, A->a, A->al, A->v[0], A->v[1], A->w[0], A->w[1]})
        LG_CUDA(cudaMemsetAsync(p + off, 0, d4 * C, st));
    LG_CUDA(cudaMemsetAsync(A->d_hold + off, (int)kHoldInactive, (size_t)C, st));
    LG_CUDA(cudaMemset2DAsync(A->bv.j + off, sizeof(int32_t) * N, 0xFF, sizeof(int32_t) * C, A->bv.bcap, st));
    LG_CUDA(cudaMemset2DAsync(A->bv.intact + off, (size_t)N, 0, (size_t)C, A->bv.bcap, st));
    for (int64_t b = 0; b < A->bv.bcap; ++b)
        for (int64_t i = 0; i < C; ++i) A->host_bond_j[(size_t)(b * N + off + i)] = -1;
    for (int k = 0; k < 2; ++k) {
        PairView &pv = A->pv[k];
        LG_CUDA(cudaMemsetAsync(pv.row_len + off, 0, sizeof(int32_t) * C, st));
        if (pv.near_len) LG_CUDA(cudaMemsetAsync(pv.near_len + off, 0, sizeof(int32_t) * C, st));
    }
    const dbl4 zero = make_double4_32a(0.0, 0.0, 0.0, 0.0);
    LG_CUDA(cudaMemcpyAsync(A->d_hoff + q, &zero, d4, cudaMemcpyHostToDevice, st));
    A->n_bonds_initial_sys[(size_t)q] = 0;
    LG_CUDA(cudaGetLastError());
    LG_CUDA(cudaStreamSynchronize(st));
    return LG_OK;
}

int lg_arena_observables(lg_system *A, int64_t q, int64_t n, lg_observables *o) {
    if (!A || !o || !A->arena || q < 0 || q >= A->n_systems || n < 1 || n > A->sys_off[q + 1] - A->sys_off[q])
        return lg_fail(LG_E_INVALID, "lg_arena_observables: bad arguments");
    const Params &P = A->P;
    const bool sint = P.binary_model == LG_BINARY_SINTER || P.binary_model == LG_BINARY_BREAKING_SINTER;
    const bool cmass = P.binary_model == LG_BINARY_CONTACT;
    const double m = sint ? P.sinter.mass : (cmass ? P.contact.mass : P.hamaker.mass);
    const double I = sint ? P.sinter.inertia : P.contact.inertia;
    StateView S = state_view(A, false);
    launch_observables_range(P, S, A->pv[A->pcur], A->bv, m, I, A->sys_off[q], n, A->obs_scratch, A->obs_out, A->stream);
    A->launches += 2;
    LG_CUDA(cudaGetLastError());
    double h[20];
    LG_CUDA(cudaMemcpyAsync(h, A->obs_out, sizeof(double) * 18, cudaMemcpyDeviceToHost, A->stream));
    LG_CUDA(cudaStreamSynchronize(A->stream));
    memset(o, 0, sizeof(*o));
    o->ke_total = h[0];
    o->ke_translational = h[1] / 2.0;
    o->ke_rotational = h[2] / 2.0;
    o->linear_momentum = m * std::sqrt((h[3] * h[3] + h[4] * h[4]) + h[5] * h[5]);
    const double L[3] = {h[6] + h[9], h[7] + h[10], h[8] + h[11]};
    o->angular_momentum = std::sqrt((L[0] * L[0] + L[1] * L[1]) + L[2] * L[2]);
    for (int k = 0; k < 3; ++k) o->center_of_mass[k] = h[12 + k] / (double)n;
    o->potential_energy = h[15];
    o->n_contacts = (int64_t)h[16];
    o->n_bonds = (int64_t)h[17];
    o->n_bonds_initial = A->n_bonds_initial_sys[(size_t)q];
    return LG_OK;
}

int lg_arena_read(lg_system *A, int64_t q, int64_t n, double *x, double *v, double *th, double *w) {
    if (!A || !A->arena || q < 0 || q >= A->n_systems || n < 1 || n > A->sys_off[q + 1] - A->sys_off[q])
        return lg_fail(LG_E_INVALID, "lg_arena_read: bad arguments");
    const int64_t off = A->sys_off[q];
    double *host[4] = {x, v, th, w};
    StateIO io{};
    for (int f = 0; f < 4; ++f) io.out[f] = host[f] ? A->obs_scratch + 3 * n * f : nullptr;
    io.wide = io_wide(io);
    launch_state_out(n, io, A->x + off, A->v[A->vcur] + off, A->th + off, A->w[A->vcur] + off, A->stream);
    A->launches += 1;
    LG_CUDA(cudaGetLastError());
    for (int f = 0; f < 4; ++f)
        if (host[f])
            LG_CUDA(cudaMemcpyAsync(host[f], A->obs_scratch + 3 * n * f, sizeof(double) * 3 * (size_t)n,
                                    cudaMemcpyDeviceToHost, A->stream));
    LG_CUDA(cudaStreamSynchronize(A->stream));
    return LG_OK;
}

// ------------------------------------------------------------------------------------------------
// Autotuner: force kernel and lanes per row, measured on a clone of the system
// ------------------------------------------------------------------------------------------------
#include <map>
#include <mutex>
#include <tuple>

// Autotuner cache: (precision, pairs, binary model, Hamaker model, log2 n, batch) -> choice.
using TuneKey = std::tuple<int, int, int, int, int, int>;
static std::mutex g_tune_mu;
static std::map<TuneKey, lg_tuning> g_tune_cache;

static TuneKey tune_key(int precision, int pairs, int bm, int hm, int64_t n, int batch) {
    int lg2 = 0;
    while (((int64_t)1 << (lg2 + 1)) <= n) ++lg2;
    return std::make_tuple(precision, pairs, bm, hm, lg2, batch ? 1 : 0);
}

// threads_per_row of a record: row-group lanes, or for the mixed compacted kernels the contact
// kernel's lanes per row
static bool compact_mixed(const lg_system *s, int kernel) {
    return kernel == LG_FORCE_KERNEL_COMPACT && s->precision == LG_PRECISION_MIXED;
}

static lg_tuning tuning_of(const lg_system *s) {
    lg_tuning t{};
    t.force_kernel = s->kernel;
    t.threads_per_row = compact_mixed(s, s->kernel) ? s->contact_lanes : s->T;
    t.step_min_blocks = s->step_min_blocks;
    t.step_slices = s->step_slices ? s->step_slices : mixed_hamaker_slices(s->P.n);
    t.step_assign = s->step_assign;
    t.ms_per_step = s->tuned_ms;
    return t;
}

static int apply_tuning(lg_system *s, const lg_tuning &t) {
    if (t.force_kernel == LG_FORCE_KERNEL_PERSISTENT) {
        if (s->precision != LG_PRECISION_MIXED) return lg_fail(LG_E_INVALID, "tuning: persistent kernel on FP64");
        LG_TRY(ensure_step_buffers(s));
    }
    // the shape fields follow the record whatever the kernel (they only act on the persistent one)
    s->step_min_blocks = t.step_min_blocks;
    s->step_slices = t.step_slices;
    s->step_assign = t.step_assign;
    if (t.force_kernel == LG_FORCE_KERNEL_PAIRS && !s->pres) return lg_fail(LG_E_INVALID, "tuning: no pair-parallel scratch");
    s->kernel = t.force_kernel;
    if (compact_mixed(s, t.force_kernel))
        s->contact_lanes = t.threads_per_row == 1 ? 1 : 2;
    else
        s->T = t.threads_per_row;
    s->tuned_ms = t.ms_per_step;
    return LG_OK;
}

extern "C" int lg_get_tuning(lg_system *s, lg_tuning *out) {
    LG_HANDLE(s);
    if (!out) return lg_fail(LG_E_INVALID, "lg_get_tuning: null output");
    *out = tuning_of(s);
    return LG_OK;
}

extern "C" int lg_autotune_cache_lookup(const lg_system_desc *d, int64_t n, int32_t batch, lg_tuning *out) {
    if (!d || !out || n < 1) return lg_fail(LG_E_INVALID, "lg_autotune_cache_lookup: bad arguments");
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(tune_key(d->precision, d->pairs, d->binary_model, d->hamaker_model, n, batch));
    if (it == g_tune_cache.end()) return lg_fail(LG_E_STATE, "lg_autotune_cache_lookup: no entry");
    *out = it->second;
    return LG_OK;
}

extern "C" int lg_autotune_cache_save(const char *path) {
    if (!path) return lg_fail(LG_E_INVALID, "lg_autotune_cache_save: null path");
    FILE *f = std::fopen(path, "w");
    if (!f) return lg_fail(LG_E_INVALID, "lg_autotune_cache_save: cannot open %s", path);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    std::fprintf(f, "# libgran_gb300 autotune cache: precision pairs binary hamaker log2n batch : kernel T "
                    "min_blocks slices assign ms_per_step\n");
    for (auto &e : g_tune_cache) {
        const TuneKey &k = e.first;
        const lg_tuning &t = e.second;
        std::fprintf(f, "%d %d %d %d %d %d : %d %d %d %d %d %.9g\n", std::get<0>(k), std::get<1>(k), std::get<2>(k),
                     std::get<3>(k), std::get<4>(k), std::get<5>(k), t.force_kernel, t.threads_per_row,
                     t.step_min_blocks, t.step_slices, t.step_assign, t.ms_per_step);
    }
    const bool ok = std::fclose(f) == 0;
    return ok ? LG_OK : lg_fail(LG_E_INVALID, "lg_autotune_cache_save: write to %s failed", path);
}

extern "C" int lg_autotune_cache_load(const char *path) {
    if (!path) return lg_fail(LG_E_INVALID, "lg_autotune_cache_load: null path");
    FILE *f = std::fopen(path, "r");
    if (!f) return lg_fail(LG_E_INVALID, "lg_autotune_cache_load: cannot open %s", path);
    char line[512];
    int lineno = 0, rc = LG_OK;
    std::map<TuneKey, lg_tuning> add;
    while (std::fgets(line, sizeof line, f)) {
        ++lineno;
        if (line[0] == '#' || line[0] == '\n') continue;
        int k[6];
        lg_tuning t{};
        if (std::sscanf(line, "%d %d %d %d %d %d : %d %d %d %d %d %lf", &k[0], &k[1], &k[2], &k[3], &k[4], &k[5],
                        &t.force_kernel, &t.threads_per_row, &t.step_min_blocks, &t.step_slices, &t.step_assign,
                        &t.ms_per_step) != 12 ||
            t.force_kernel < 1 || t.force_kernel > 5 || t.threads_per_row < 1 || t.threads_per_row > 32 ||
            (t.step_min_blocks < 4 || t.step_min_blocks > 6) || (t.step_slices != 1 && t.step_slices != 2 && t.step_slices != 4) ||
            (t.step_assign != 0 && t.step_assign != 1)) {
            rc = lg_fail(LG_E_INVALID, "lg_autotune_cache_load: %s line %d is not a cache entry", path, lineno);
            break;
        }
        add[std::make_tuple(k[0], k[1], k[2], k[3], k[4], k[5])] = t;
    }
    std::fclose(f);
    if (rc != LG_OK) return rc;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (auto &e : add) g_tune_cache[e.first] = e.second;
    return LG_OK;
}

extern "C" int lg_autotune_cache_clear(void) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache.clear();
    return LG_OK;
}

static int snapshot_take(lg_system *s) {
    if (s->snap.empty()) {
        const int64_t n = s->P.n;
        auto addb = [&](void *live, size_t bytes) { s->snap.push_back({live, nullptr, bytes}); };
        addb(s->x, sizeof(dbl4) * n);
        addb(s->th, sizeof(dbl4) * n);
        for (int q = 0; q < 2; ++q) {
            addb(s->v[q], sizeof(dbl4) * n);
            addb(s->w[q], sizeof(dbl4) * n);
        }
        addb(s->a, sizeof(dbl4) * n);
        addb(s->al, sizeof(dbl4) * n);
        const int nf = std::max(s->P.n_facets, 1);
        addb(s->sxi, sizeof(double) * 9 * (size_t)nf * (size_t)n);
        addb(s->fv[0], sizeof(double) * 9 * (size_t)nf);
        addb(s->fv[1], sizeof(double) * 9 * (size_t)nf);
        addb(s->err, sizeof(int32_t));
        if (s->x32buf) addb(s->x32buf, sizeof(float4) * 4 * n);
        if (s->v32buf) addb(s->v32buf, sizeof(float4) * 6 * n);
        if (s->s32) addb(s->s32, sizeof(float4) * 5 * n);
        const int npv = s->P.pairs == LG_PAIRS_VERLET ? 2 : 1;
        for (int q = 0; q < npv; ++q) {
            PairView &pv = s->pv[q];
            const size_t slots = (size_t)(pv.cap * n);
            if (pv.nbr) addb(pv.nbr, sizeof(int32_t) * slots);
            if (pv.row_len) addb(pv.row_len, sizeof(int32_t) * n);
            addb(pv.flags, sizeof(uint32_t) * slots);
            addb(pv.xi, sizeof(double) * 9 * slots);
            if (pv.near_len) {
                addb(pv.near_j, sizeof(int32_t) * slots);
                addb(pv.near_k, slots);
                addb(pv.near_len, sizeof(int32_t) * n);
            }
        }
        const size_t bs = (size_t)s->bv.bcap * (size_t)n;
        addb(s->bv.intact, bs);
        addb(s->bv.xi, sizeof(double) * 9 * bs);
        if (s->bv.cn) addb(s->bv.cn, sizeof(double) * 15 * bs);
        for (auto &b : s->snap) {
            void *p = nullptr;
            cudaError_t e = cudaMalloc(&p, b.bytes);
            if (e != cudaSuccess) {
                cudaGetLastError();
                for (auto &c : s->snap)
                    if (c.copy) cudaFree(c.copy);
                s->snap.clear();
                return lg_fail(LG_E_NOMEM, "snapshot: cudaMalloc of %zu bytes failed", b.bytes);
            }
            b.copy = p;
            s->allocations.push_back(p);
        }
    }
    for (auto &b : s->snap) LG_CUDA(cudaMemcpyAsync(b.copy, b.live, b.bytes, cudaMemcpyDeviceToDevice, s->stream));
    s->snap_vcur = s->vcur;
    s->snap_pcur = s->pcur;
    s->snap_fcur = s->fcur;
    s->snap_ffcur = s->ffcur;
    s->snap_step = s->step_index;
    s->snap_built = s->list_built;
    return LG_OK;
}

static int snapshot_restore(lg_system *s) {
    if (s->snap.empty()) return lg_fail(LG_E_STATE, "snapshot: nothing to restore");
    for (auto &b : s->snap) LG_CUDA(cudaMemcpyAsync(b.live, b.copy, b.bytes, cudaMemcpyDeviceToDevice, s->stream));
    s->vcur = s->snap_vcur;
    s->pcur = s->snap_pcur;
    s->fcur = s->snap_fcur;
    s->ffcur = s->snap_ffcur;
    set_ff_buffers(s);
    s->step_index = s->snap_step;
    s->list_built = s->snap_built;
    return LG_OK;
}

extern "C" int lg_snapshot(lg_system *s) {
    LG_HANDLE(s);
    return snapshot_take(s);
}

extern "C" int lg_restore(lg_system *s) {
    LG_HANDLE(s);
    return snapshot_restore(s);
}

extern "C" int lg_autotune(lg_system *s, double dt, int64_t probe_steps, int64_t rebuild_every, int32_t *kernel_out,
                           int32_t *T_out, int32_t use_cache) {
    LG_HANDLE(s);
    if (probe_steps < 1) return lg_fail(LG_E_INVALID, "lg_autotune: probe_steps < 1");
    const TuneKey key = tune_key(s->precision, s->P.pairs, s->P.binary_model, s->P.hamaker_model, s->P.n,
                                 s->n_systems > 0 ? 1 : 0);
    if (use_cache) {
        lg_tuning hit{};
        bool found = false;
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            auto it = g_tune_cache.find(key);
            if (it != g_tune_cache.end()) {
                hit = it->second;
                found = true;
            }
        }
        if (found && apply_tuning(s, hit) == LG_OK) {
            s->drop_graphs();
            if (kernel_out) *kernel_out = s->kernel;
            if (T_out) *T_out = tuning_of(s).threads_per_row;
            return LG_OK;
        }
    }
    // candidates run on the live system between a snapshot and its restore
    LG_TRY(snapshot_take(s));
    const lg_tuning keep = tuning_of(s);
    const int64_t keep_launch = s->launches;
    std::vector<lg_tuning> cands;
    auto add = [&](int k, int T, int mb, int sl, int asg) {
        lg_tuning t{};
        t.force_kernel = k;
        t.threads_per_row = T;
        t.step_min_blocks = mb;
        t.step_slices = sl;
        t.step_assign = asg;
        cands.push_back(t);
    };
    const int sl0 = mixed_hamaker_slices(s->P.n);
    add(LG_FORCE_KERNEL_COMPACT, s->precision == LG_PRECISION_MIXED ? 2 : 1, 4, sl0, 0);
    if (s->precision == LG_PRECISION_MIXED) add(LG_FORCE_KERNEL_COMPACT, 1, 4, sl0, 0);  // one contact lane per row
    if (s->pres) add(LG_FORCE_KERNEL_PAIRS, 1, 4, sl0, 0);
    for (int T = 1; T <= 32; T *= 2) add(LG_FORCE_KERNEL_ROWGROUP, T, 4, sl0, 0);
    if (s->precision == LG_PRECISION_MIXED)
        for (int mb = 4; mb <= 6; ++mb)
            for (int sl = 1; sl <= 4; sl *= 2)
                for (int asg = 0; asg <= 2; ++asg) add(LG_FORCE_KERNEL_PERSISTENT, 1, mb, sl, asg);
    double best = 1e300;
    lg_tuning pick = keep;
    for (auto &c : cands) {
        int rc = apply_tuning(s, c);
        float ms = 0.f, ms2 = 0.f;
        if (rc == LG_OK) rc = lg_step(s, dt, probe_steps, rebuild_every);  // warm-up (and graph capture)
        if (rc == LG_OK) rc = snapshot_restore(s);
        if (rc == LG_OK) rc = lg_step_timed(s, dt, probe_steps, rebuild_every, &ms);
        if (rc == LG_OK) rc = snapshot_restore(s);
        if (rc == LG_OK) rc = lg_step_timed(s, dt, probe_steps, rebuild_every, &ms2);
        const int rc2 = snapshot_restore(s);
        if (rc != LG_OK || rc2 != LG_OK) {
            apply_tuning(s, keep);
            return rc != LG_OK ? rc : rc2;
        }
        const double t = std::min(ms, ms2) / (double)probe_steps;
        if (!(t > 0.0)) {  // an event pair that measured nothing cannot rank a candidate
            apply_tuning(s, keep);
            return lg_fail(LG_E_CUDA, "lg_autotune: a candidate timed %g ms", t);
        }
        if (t < best) {
            best = t;
            pick = c;
            pick.ms_per_step = t;
        }
    }
    LG_CUDA(cudaStreamSynchronize(s->stream));
    s->launches = keep_launch;
    LG_TRY(apply_tuning(s, pick));
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = pick;
    }
    if (kernel_out) *kernel_out = s->kernel;
    if (T_out) *T_out = tuning_of(s).threads_per_row;
    return LG_OK;
}
