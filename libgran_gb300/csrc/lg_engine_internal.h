// lg_engine_internal.h -- the handle behind the opaque lg_system pointer of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "lg_kernels.h"

struct lg_system {
    int device = -1;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // mixed precision: a second stream on which the contact kernel runs beside the Hamaker kernel
    // (fork / join events on the handle's stream; captured into the step graphs as two branches)
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    lg_system_desc desc{};
    lg::Params P{};
    int precision = LG_PRECISION_FP64;
    bool facet_auto_move = false;

    // state (32-byte slots); v and w ping-pong between the half-step and full-step buffers
    lg::dbl4 *x = nullptr, *th = nullptr, *a = nullptr, *al = nullptr;
    lg::dbl4 *v[2] = {nullptr, nullptr}, *w[2] = {nullptr, nullptr};
    int vcur = 0;
    double *sxi = nullptr;               // surface springs
    double *fv[2] = {nullptr, nullptr};  // facet vertices (current / next)
    int fcur = 0;
    int32_t *err = nullptr;

    // pairs and bonds
    lg::PairView pv[2]{};
    int pcur = 0;
    bool list_built = false;
    int64_t max_cells = 0;
    lg::ListScratch ls{};
    lg::BondView bv{};
    std::vector<int32_t> host_bond_j;
    int64_t n_bonds_initial = 0;

    // observables
    double *obs_scratch = nullptr;
    double *obs_out = nullptr;

    // mixed precision: FP32 position copy for culling
    float4 *x32 = nullptr;  // mixed: [2n] float-float positions (the current one of the two buffers)
    float4 *v32 = nullptr;  // mixed: [3n] float-float velocities, FP32 spins (current buffer)
    // mixed: both buffers of the double-buffered float-float positions ([2][2n]) and velocities
    // ([2][3n]); the persistent step kernel reads one and writes the other, ffcur names the current
    float4 *x32buf = nullptr, *v32buf = nullptr;
    int ffcur = 0;
    int64_t fstep = 0;             // persistent step launches so far (their item counters alternate)
    unsigned *step_ctr = nullptr;  // persistent step: [2 + groups] item and arrival counters
    float4 *hpart = nullptr;       // persistent step: [4][2n] Hamaker partial sums (up to 4 slices)
    // persistent step shape: Hamaker slices per group, register budget (resident blocks per SM),
    // item assignment (0 pulled from a counter, 1 round robin)
    int step_slices = 0, step_min_blocks = 4, step_assign = 0;
    double tuned_ms = 0.0;         // the autotuner's time per step of the handle's current choice
    int ham_slices = 0;            // mixed: Hamaker slices of the two-stream kernels (0: size rule)
    int contact_lanes = 2;         // mixed: lanes per row of the two-stream contact kernel (1 or 2)
    // serving arena (lg_arena_create): a batch whose systems are slots; lattice point of each slot
    bool arena = false;
    double arena_lattice = 0.0;
    std::vector<double> slot_pos;  // [3 * slots]
    float4 *s32 = nullptr;  // mixed: [5n] spin low parts, a run's displacement and rotation (float-float)
    float4 *csum = nullptr;    // mixed: [3n] contact sums (float-float)
    float4 *hsum = nullptr;    // mixed: [2n] Hamaker sums (float-float)
    int32_t *d_flag = nullptr;  // mixed: device flag of the float-float copy check
    double *pres = nullptr;     // FP64 pair-parallel kernel: per-slot pair values [6][cap * n]
    unsigned *d_ticket = nullptr;  // zeroed counter of the reductions' last-block combine
    double *h_pin = nullptr;       // pinned host buffer (64 doubles) for small results read back
    uint8_t *d_hold = nullptr;  // [n] LG_HOLD_* bits (allocated on first use)
    lg::dbl4 *ext_a = nullptr, *ext_al = nullptr;  // [n] unary body-force terms (allocated on first use)
    double *d_centre = nullptr; // [3 * systems] centres of the central body force
    lg_body_force body{};       // model LG_BODY_NONE: no body force
    lg_unary_hook hook = nullptr;
    void *hook_user = nullptr;
    double origin[4] = {0.0, 0.0, 0.0, 0.0};  // mixed: origin of the float-float positions, extent in [3]
    double r_max = 0.0;                        // mixed: largest particle radius of the functors
    double ext_max = 0.0;                      // mixed: largest extent of a system about its origin
    double r_near = 0.0;                       // mixed, Verlet: radius of the contact-candidate lists
    bool kick_done = false;                    // the last step already ran the next one's half kick and drift
    double cull_near = 0.0, cull_contact = 0.0;  // mixed: culling radii before margins
    lg::MixedExtra mx{};

    // force-kernel timing (bench instrumentation)
    bool timing = false;
    std::vector<cudaEvent_t> tev;  // pairs: start, stop
    size_t tev_used = 0;

    // batch segmentation (n_systems == 0 for a single system)
    int64_t n_systems = 0;
    std::vector<int64_t> sys_off;        // host prefix offsets [n_systems + 1]
    int64_t *d_sys_off = nullptr;        // device copy
    int32_t *d_agg = nullptr;            // [n] system of every particle
    lg::dbl4 *d_hoff = nullptr;          // [n_systems] hashing offsets
    lg::dbl4 *d_orig = nullptr;          // [n_systems] float-float origins (x, y, z; w: extent), mixed
    std::vector<lg::dbl4> h_orig;        // host copy of d_orig
    double *d_centres = nullptr;         // [3 n_systems] scratch for per-system observables
    double *d_sys_obs = nullptr;         // [20 n_systems]
    std::vector<int64_t> n_bonds_initial_sys;

    // CUDA graphs of whole rebuild periods, keyed by the state that determines their pointers
    struct GraphKey {
        double dt;
        int64_t period;
        int kernel, T, vcur, pcur, fcur, ffcur, fpar, lanes;
        bool operator==(const GraphKey &o) const {
            return dt == o.dt && period == o.period && kernel == o.kernel && T == o.T && vcur == o.vcur &&
                   pcur == o.pcur && fcur == o.fcur && ffcur == o.ffcur && fpar == o.fpar && lanes == o.lanes;
        }
    };
    struct GraphEntry {
        GraphKey key;
        cudaGraphExec_t exec;
        int64_t launches;
        int ff_flips;        // float-float buffer swaps of the period (persistent steps)
        int64_t f_launches;  // persistent step launches of the period
    };
    std::vector<GraphEntry> graphs;
    bool use_graphs = true;
    int64_t periods_run = 0;

    // device-state snapshot (autotuner, serving): list of (live buffer, copy, bytes)
    struct SnapBuf {
        void *live;
        void *copy;
        size_t bytes;
    };
    std::vector<SnapBuf> snap;
    int snap_vcur = 0, snap_pcur = 0, snap_fcur = 0, snap_ffcur = 0;
    int64_t snap_step = 0;
    bool snap_built = false;

    // inputs kept for cloning (autotuner)
    std::vector<lg_facet_desc> facet_descs;
    std::vector<double> neck_copy;
    std::vector<int64_t> sizes_copy;

    int T = 1;  // lanes per row group of the force kernel
    int kernel = LG_FORCE_KERNEL_ROWGROUP;  // resolved force kernel
    int64_t step_index = 0;
    int64_t launches = 0;
    std::vector<void *> allocations;
    // device memory from the stream-ordered pool (cudaMallocAsync / cudaFreeAsync on the handle's
    // stream): releasing such a handle does not synchronise the device (serving's staging handles)
    bool pooled = false;

    template <typename U>
    int alloc(U **p, size_t count);
    void release();
    void drop_graphs();
};

int lg_fail(int code, const char *fmt, ...);

// Serving slots (lg_engine.cpp), for the serving loop. An arena is a batch handle whose systems
// are slots of fixed capacities (caps) on a lattice; a slot holds one request (its first n
// particles) or nothing, and its other particles are inactive (no cell, no row, no motion). All
// occupants advance in the same launches. lg_arena_import moves a standalone handle built from the
// same template (the request after its construction force evaluation, at a rebuild boundary) into
// slot q: state, bonds with their springs, pair rows with their springs (partner indices moved by
// the slot's offset), float-float origin and hashing offset; the occupant then evolves exactly as
// the standalone handle would. lg_arena_clear empties a slot; lg_arena_read copies an occupant's
// state (host arrays of 3n doubles, null: skipped). The caller keeps the arena at a rebuild
// boundary and idle (synchronised) around imports and clears.
int lg_arena_create(const lg_system_desc *tmpl, int64_t n_slots, const int64_t *caps, int device, lg_system **out);
// A standalone handle whose device memory comes from the stream-ordered pool (lg_create otherwise).
int lg_create_staged(const lg_system_desc *desc, const double *x0, const double *v0, int device, lg_system **out);
double lg_arena_radius_bound(int64_t cap, double r_part);
int lg_arena_import(lg_system *arena, int64_t q, lg_system *src, const double *x0);
int lg_arena_clear(lg_system *arena, int64_t q);
int lg_arena_read(lg_system *arena, int64_t q, int64_t n, double *x, double *v, double *theta, double *omega);
// Observables of slot q's occupant (its first n particles; the radius of gyration is left at 0).
int lg_arena_observables(lg_system *arena, int64_t q, int64_t n, lg_observables *out);
