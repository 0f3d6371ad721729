// lg_kernels.h -- launchers shared between the engine host code and the kernel translation units.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "lg_common.cuh"

namespace lg {

struct GridDev {
    double lo[3];
    double edge;
    int64_t dim[3];
    int64_t ncell;
    float rv2_lo, rv2_hi;  // FP32 accept / reject bounds of the squared list radius
    float rn2_hi;          // FP32 bound of the squared near radius (contact candidates), < 0: none
};

// Batch segmentation (null pointers for a single system): system index of every particle and the
// spatial offset of every system used only for cell hashing.
struct BatchView {
    const int32_t *agg;    // [n]
    const dbl4 *hoff;      // [n_systems]
    const uint8_t *hold;   // [n] hold bits (null: none); inactive particles are left out of the list
};

struct ListScratch {
    int nparts;        // blocks of the bounding-box pass
    double *part;      // [nparts * 6]
    GridDev *grid;     // device grid description
    int32_t *cell_of;  // [n]
    int32_t *count;    // [max_cells]
    int32_t *start;    // [max_cells]
    int32_t *fill;     // [max_cells]
    int32_t *sorted;   // [n]
    int32_t *tile;     // [max_cells / 4096 + 1] cell-scan tile totals, then their offsets
    float4 *x32;       // [n] positions relative to the grid origin, FP32 (candidate filter)
    int32_t *max_row;  // [1] longest row found by the last build (before truncation)
};

// FP64 path (lg_forces_fp64.cu, compiled with --fmad=false)
void launch_forces_fp64(int T, const Params &P, const StateView &S, const PairView &PV, const BondView &BV, double hdt,
                        double dt, int move_facets, cudaStream_t st);
// Pair-parallel FP64 evaluation for small systems: per-slot pair values into pres [6][PV.cap * n],
// then an ordered per-row fold; kick: also runs the next step's half kick and drift. Returns the
// number of kernels launched.
int launch_forces_pairs_fp64(const Params &P, const StateView &S, const PairView &PV, const BondView &BV,
                             double *pres, double hdt, double dt, int move_facets, bool kick, cudaStream_t st);
// With connectors (BV.cn non-null) the drift also carries the 5-connector model's connectors.
// hold: per-particle LG_HOLD_* bits (null: none).
void launch_kick_drift_fp64(int64_t n, dbl4 *x, dbl4 *v, dbl4 *th, dbl4 *w, const dbl4 *a,
                            const dbl4 *al, double dt, double hdt, const BondView &BV, const uint8_t *hold,
                            cudaStream_t st);
// Central body force (LG_BODY_CENTRAL) into ea / eal; centre: 3 doubles per system (agg: system of
// each particle, null for one system); kam = k_a / mass.
void launch_body_central(int64_t n, const dbl4 *x, const int32_t *agg, const double *centre, double kam, dbl4 *ea,
                         dbl4 *eal, cudaStream_t st);
// Rebuilds the Verlet rows into newv (springs carried from oldv). With r_near > 0 it also lists each
// row's contact candidates (newv.near_*): slots within r_near or bonded; springs of the other slots
// are not carried (those pairs are apart, so their springs reset).
void launch_list_build(int64_t n, const dbl4 *x, BatchView B, double rv, double r_near, int64_t max_cells,
                       ListScratch &ls, PairView oldv, PairView newv, BondView BV, int32_t *err, cudaStream_t st);

// Mixed-precision path (lg_forces_mixed.cu)
struct MixedExtra {
    // [2n] positions relative to the system origin as interleaved float-float pairs: x32[2i] = FP32
    // rounding of x_i - origin (culling, and the high part), x32[2i + 1] = FP32 rounding of the
    // remainder; hi + lo holds the position to about 2^-48 of its magnitude, and a partner's pair
    // is one 32-byte sector
    float4 *x32;
    // [3n] velocities of the force evaluation: v32[i] / v32[n + i] = high / low FP32 parts of v_i,
    // v32[2n + i] = FP32 rounding of omega_i (compacted kernel's contact and bond pairs)
    float4 *v32;
    // [5n] the rest of the float-float state that runs of fused steps carry (the completion kernel
    // integrates in float-float between a run's first and last steps): s32[i] = low FP32 parts of
    // omega_i; s32[n + i], s32[2n + i] = displacement since the run's first step (hi, lo);
    // s32[3n + i], s32[4n + i] = rotation since then (hi, lo)
    float4 *s32;
    // compacted kernels' scratch: per particle the float-float (hi, lo) pairs of the contact sums
    // (csum, [3n]: a.x a.y / a.z alpha.x / alpha.y alpha.z) and of the Hamaker sum (hsum, [2n])
    float4 *csum;
    float4 *hsum;
    // origins of the float-float positions (for the completion kernel's fused kick and drift)
    const int32_t *agg;  // [n] system of each particle (batch), or null
    const dbl4 *orig;    // [n_systems] origins of the systems of a batch
    double ox, oy, oz;   // origin of a single system
    float near2;      // squared culling radius (FP32 positions); beyond it a pair cannot touch and the
                      // limited Hamaker force is zero
    float contact2f;  // squared contact-candidate radius (FP32 positions, with margin)
    double rcut2;     // squared limited-Hamaker cutoff (FP64 separation)
    float inv_mass_h; // 1 / mass of the Hamaker functor
    double inv_mass_c, inv_inertia_c;  // 1 / mass, 1 / inertia of the contact functor
    double inv_mass_b, inv_inertia_b;  // 1 / mass, 1 / inertia of the sintered-bond functor
    double four_rc2, four_rb2, four_rh2;  // (2r)^2 of the contact, bond and Hamaker functors
    // FP32 copies of the functor parameters (converted once, not per pair)
    float c_k, c_gn, c_kt, c_gt, c_mus, c_phid, c_kr, c_gr, c_mur, c_phir, c_ko, c_go, c_muo, c_phio, c_r, c_dt;
    float b_k, b_gn, b_kt, b_gt, b_kr, b_gr, b_ko, b_go, b_r, b_dt;
    float h_A, h_h0, h_r;
    // compacted kernel: (2r)^2 of the Hamaker functor as hi + lo, the limited-Hamaker cutoff as a
    // bound on |d|^2 - (2r)^2, and the reciprocal mass and inertia of the binary functor in use
    float h_fr_hi, h_fr_lo, h_qcut;
    float c_fr_hi, c_fr_lo, b_fr_hi, b_fr_lo;
    float bin_im, bin_iI;
    // contact decisions at the threshold: a non-bonded pair whose float-float q lies within q_marg
    // of zero is in contact when the FP64 overlap of the FP64 path, 2r - dx.(dx/|dx|) from x64, is
    // positive; x64 is set only for evaluations whose FP64 positions are current (null inside a run
    // of steps integrated in float-float)
    const dbl4 *x64;
    float q_marg;
};
bool mixed_available();
void launch_forces_mixed(int T, const Params &P, const StateView &S, const PairView &PV, const BondView &BV,
                         double hdt, double dt, int move_facets, const MixedExtra &MX, cudaStream_t st);
// Float-float copies for the mixed kernels: x32 (2n entries) from the positions, v32 (3n entries)
// from the velocities and spins (see MixedExtra); origin[0..2] is the origin of a single system,
// orig[] those of each system of a batch.
// With `uncovered`, also sets *uncovered when a position lies beyond four times its system's extent
// (origin[3], orig[].w) from the origin: the origins must then be set up again.
void launch_mixed_copies(int64_t n, const dbl4 *x, const dbl4 *v, const dbl4 *w, const dbl4 *th, const double *origin,
                         const int32_t *agg, const dbl4 *orig, float4 *x32, float4 *v32, float4 *s32, cudaStream_t st,
                         int32_t *uncovered = nullptr);
// Kick + drift of the mixed path; also refreshes x32, v32 and s32.
void launch_kick_drift_mixed(int64_t n, dbl4 *x, dbl4 *v, dbl4 *th, dbl4 *w, const dbl4 *a, const dbl4 *al, double dt,
                             double hdt, const double *origin, const int32_t *agg, const dbl4 *orig, float4 *x32,
                             float4 *v32, float4 *s32, const uint8_t *hold, cudaStream_t st);

// Slices per 32-row group of the mixed Hamaker work (launch size rule shared by both mixed paths:
// the same slicing gives the same bits).
int mixed_hamaker_slices(int64_t n);

// Persistent step of the mixed path (lg_step_mixed.cu): the force evaluation and float-float
// completion of one step inside a run of steps as one launch whose warps pull work items (per
// 32-row group: two contact items, `slices` Hamaker items) from a device counter; the warp that
// finishes a group's last item completes its rows. For plain runs only (no facets, body terms or
// held particles).
struct StepArgs {
    float4 *x32n, *v32n;  // the other buffers of the double-buffered float-float state (written)
    float4 *hpart;        // [slices][2n] Hamaker partial sums per slice
    unsigned *ctr;        // [6 + groups]: item counters (two pairs), then group arrivals (ctr + 6)
    int par;              // item counter of this launch within its pair (0 / 1, alternating by step)
    int slices;           // Hamaker items per group
    int contacts, hamaker;  // which item kinds exist
    int last;             // the run's last step: write the FP64 state instead of the next step's
    int assign;           // 0: warps pull items from a counter; 1: warp g takes items g, g + W, ...;
                          // 2: two launches side by side (contact items on the side stream, Hamaker
                          // items on the main stream), each pulling from its own counter
    int min_blocks;       // register budget: resident blocks per SM (4, 5 or 6)
    int64_t items;        // groups * (2 * contacts + slices * hamaker)
    float hdt_hi, hdt_lo, dt_hi, dt_lo;  // dt / 2 and dt as float-float values
};
// One step as one launch on st, or (A.assign == 2) as two launches on side and st joined through the
// two events; returns the number of kernels launched.
int launch_step_mixed(const Params &P, const StateView &S, const PairView &PV, const BondView &BV,
                      const MixedExtra &MX, const StepArgs &A, cudaStream_t st, cudaStream_t side = nullptr,
                      cudaEvent_t fork = nullptr, cudaEvent_t join = nullptr);

// Warp-compacted force kernels (lg_forces_compact.cu, compiled once per precision)
// fast: LG_FORCE_KERNEL_FP64_FAST (reciprocals instead of repeated divisions; within 1e-12).
void launch_forces_compact_fp64(const Params &P, const StateView &S, const PairView &PV, const BondView &BV, double hdt,
                                double dt, int move_facets, cudaStream_t st, bool fast = false);
// Mixed precision: the contact/bond kernel (if the system has a binary model) on `side`, beside the
// Hamaker kernel on `st` (fork / join through the two events), then the completion kernel on `st`;
// returns the number of kernels launched.
// With `kick`, the completion kernel goes on to the next step's opening half kick and drift (and the
// float-float copies), exactly as launch_kick_drift_mixed would.
// kick: another step follows (the completion also runs its opening half kick and drift);
// prev_fused: the step before was such a step (its state may be float-float only).
// slices: Hamaker slices per 32-row group (0: mixed_hamaker_slices(P.n)); contact_lanes: lanes per
// row of the contact kernel over candidate lists (1 or 2; all pairs take a warp per row).
int launch_forces_compact_mixed(const Params &P, const StateView &S, const PairView &PV, const BondView &BV, double hdt,
                                double dt, int move_facets, bool kick, bool prev_fused, const MixedExtra &MX,
                                cudaStream_t st, cudaStream_t side, cudaEvent_t fork, cudaEvent_t join, int slices = 0,
                                int contact_lanes = 2);

// Layout conversion between a caller's [n][3] doubles (already in device memory) and the padded
// device layout (lg_reduce.cu).
// State transfers: up to four [n][3] fields (x, v, theta, omega) per launch, device or pinned host.
struct StateIO {
    const double *in[4];
    double *out[4];
    int32_t wide;  // every non-null in / out pointer is 16-byte aligned: 16-byte accesses
};
void launch_state_in(int64_t n, const StateIO &io, dbl4 *x, dbl4 *v, dbl4 *th, dbl4 *w, float4 *x32, float4 *v32,
                     float4 *s32, const double *origin, const int32_t *agg, const dbl4 *orig, int32_t *uncovered,
                     cudaStream_t st);
void launch_state_out(int64_t n, const StateIO &io, const dbl4 *x, const dbl4 *v, const dbl4 *th, const dbl4 *w,
                      cudaStream_t st);
void launch_aos_to_dev4(int64_t n, const double *aos, dbl4 *dst, cudaStream_t st);
void launch_dev4_to_aos(int64_t n, const dbl4 *src, double *aos, cudaStream_t st);

// Serving slots (lg_reduce.cu): p[r * pitch + c] += off wherever the entry is an index (>= 0), for
// r < rows, c < width; and count positions set to (x, y, z).
void launch_offset_indices(int32_t *p, int64_t rows, int64_t pitch, int64_t width, int32_t off, cudaStream_t st);
void launch_fill_dbl4(dbl4 *p, int64_t count, double x, double y, double z, cudaStream_t st);

// Observables (lg_reduce.cu). scratch: at least obs_scratch_doubles(n) doubles of device memory;
// out: 20 doubles of device memory (column sums, see lg_reduce.cu).
int64_t obs_scratch_doubles(int64_t n);
void launch_observables(const Params &P, const StateView &S, const PairView &PV, const BondView &BV, double mass,
                        double inertia, double *scratch, double *out, cudaStream_t st, bool pairs = true);
// Column sums 0..17 over the particles row0 .. row0 + count - 1 only (one system of a batch).
void launch_observables_range(const Params &P, const StateView &S, const PairView &PV, const BondView &BV,
                              double mass, double inertia, int64_t row0, int64_t count, double *scratch, double *out,
                              cudaStream_t st);
// Handle observables: out[0..14] and out[18] from the particles (launch_observables_state), out[15..17]
// from the pair slots (launch_observables_pairs); scratch as above.
void launch_observables_state(int64_t n, const dbl4 *x, const dbl4 *v, const dbl4 *w, double mass, double inertia,
                              double *scratch, double *out, unsigned *ticket, cudaStream_t st);
void launch_observables_pairs(const Params &P, const StateView &S, const PairView &PV, const BondView &BV, double mass,
                              double inertia, double *scratch, double *out, cudaStream_t st);
// Per-system observables of a batch: out[s * 20 + c] = column sums over system s's particles
// (rows from launch_observables' scratch), then column 18 = sum |x - c_s|^2 with centres from
// centres[3 s ..].
void launch_segmented_sums(int64_t n_systems, const int64_t *offsets, const double *scratch, double *out,
                           cudaStream_t st);
void launch_segmented_rg(int64_t n, int64_t n_systems, const int64_t *offsets, const dbl4 *x, const double *centres,
                         double *scratch, double *out, cudaStream_t st);

}  // namespace lg
