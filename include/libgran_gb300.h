/*
 * libgran_gb300.h -- C ABI of the GB300 (sm_103a) DEM pair-force + integration engine.
 *
 * This is the drop-in boundary for libgran's hot path: a granular_system stepped by a rotational
 * velocity-Verlet integrator over binary pair-force functors (frictional contact, sintered bond,
 * breaking sintered bond, Hamaker van der Waals) and unary triangular-facet surface functors.
 * libgran itself is a header-only C++ template library without any FFI; the entry points below are
 * what its templates bind to when they are re-targeted at the GPU (see the headers in include/libgran_gb300/,
 * which keep libgran's class names and constructor signatures and call into this ABI).
 *
 * Conventions
 *   - Every function returns an int status: LG_OK (0) on success, a negative LG_E* code otherwise.
 *     lg_last_error() returns a human readable description of the last failure on this thread.
 *     No C++ exception crosses this boundary.
 *   - A handle owns all of its device memory and one CUDA stream. A handle is not thread safe;
 *     distinct handles are independent. Vectors cross the ABI as AoS double[3*n] host arrays.
 *   - Host pointers are plain pages or pinned pages; nothing here keeps a host pointer after return.
 *
 * Reference citations use paths inside the libgran project (egor-demidov/libgran).
 */
#ifndef LIBGRAN_GB300_H
#define LIBGRAN_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------------- */
#define LG_OK 0
#define LG_E_INVALID (-1)   /* bad argument (null pointer, size out of range, unknown enum) */
#define LG_E_CUDA (-2)      /* a CUDA runtime call failed */
#define LG_E_NOMEM (-3)     /* device or host allocation failed, or a budget was exceeded */
#define LG_E_STATE (-4)     /* call not valid in the handle's current state */
#define LG_E_DEVICE (-5)    /* a kernel reported an error word (capacity overflow, non-finite) */

/* ---- model selectors ---------------------------------------------------------------------- */
/* Which binary functor sits in the binary_force_functor_container (binary_force_container.h:14-35).
 * SINTER and BREAKING_SINTER embed their own copy of a contact_force_functor for non-bonded pairs
 * (alt_sinter_bridge.h:36,100-101; alt_breaking_sinter_bridge.h:35,86-87). */
#define LG_BINARY_NONE 0
#define LG_BINARY_CONTACT 1          /* contact_force_functor, contact_force/contact_force.h:8-157 */
#define LG_BINARY_SINTER 2           /* alt_sinter_functor, sinter_bridge/alt_sinter_bridge.h:17-180 */
#define LG_BINARY_BREAKING_SINTER 3  /* alt_breaking_sinter_functor, alt_breaking_sinter_bridge.h:16-166 */
#define LG_BINARY_SINTER_CONNECTORS 4  /* sinter_functor + sinter_step_handler, sinter_bridge.h:14-272:
                                          five connector springs per bond, moved with the particles by
                                          the integrator's increments; FP64 precision only */

/* Which Hamaker functor (if any) is folded in after the binary functor. */
#define LG_HAMAKER_NONE 0
#define LG_HAMAKER_FULL 1        /* hamaker_functor, hamaker_force/hamaker_force.h:18-48 */
#define LG_HAMAKER_LIMITED 2     /* limited_range_hamaker_functor, limited_range_hamaker_force.h:18-52 */
#define LG_HAMAKER_SIMPLIFIED 3  /* simplified_hamaker_functor, simplified_hamaker_force.h:8-34 */

/* Neck strength lookup of the breaking sintered bond. The reference stores strengths at particle
 * indices (alt_breaking_sinter_bridge.h:71-73) and reads them at pair indices (:118), so in the
 * reference nearly every bond reads strength 0. PER_BOND gives each bond its own strength (the
 * evident intent); REFERENCE_INDEXING reproduces the reference's lookup bit for bit. */
#define LG_NECK_PER_BOND 0
#define LG_NECK_REFERENCE_INDEXING 1

/* Arithmetic of the pair kernel. */
#define LG_PRECISION_FP64 0   /* every operation in FP64 */
#define LG_PRECISION_MIXED 1  /* FP64 separation, overlap, springs, sums, integration; FP32 rest */

/* Pair enumeration. */
#define LG_PAIRS_ALL 0        /* all ordered pairs j != i (granular_system, granular_system.h:25-86) */
#define LG_PAIRS_VERLET 1     /* Verlet list of radius r_verlet (granular_system_neighbor_list.h:54-64) */

/* ---- functor parameter blocks (same order as the reference constructors) ------------------- */

/* contact_force_functor(n_part, k, gamma_n, k_t, gamma_t, mu_s, phi_d, k_r, gamma_r, mu_r, phi_r,
 *                       k_o, gamma_o, mu_o, phi_o, r_part, mass, inertia, dt, ...)
 * contact_force/contact_force.h:10-30; surface_contact_force_functor has the same list,
 * contact_force/surface_contact_force.h:10-30. */
typedef struct lg_contact_params {
    double k, gamma_n;
    double k_t, gamma_t, mu_s, phi_d;
    double k_r, gamma_r, mu_r, phi_r;
    double k_o, gamma_o, mu_o, phi_o;
    double r_part, mass, inertia, dt;
} lg_contact_params;

/* alt_sinter_functor(n_part, x0, k, gamma_n, k_t, gamma_t, k_r, gamma_r, k_o, gamma_o,
 *                    r_part, mass, inertia, dt, ..., critical_separation, contact_force)
 * sinter_bridge/alt_sinter_bridge.h:19-36 (alt_breaking_sinter_bridge.h:17-35 adds the neck
 * strength distribution, passed to lg_create as an array). */
typedef struct lg_sinter_params {
    double k, gamma_n, k_t, gamma_t, k_r, gamma_r, k_o, gamma_o;
    double r_part, mass, inertia, dt;
    double critical_separation;
} lg_sinter_params;

/* sinter_functor(n_part, k_d, gamma_d, <contact parameters>, ..., random_unit_vector_generator,
 * critical_separation), sinter_bridge.h:100-136: the connector springs' stiffness and damping and
 * the bonding distance; the contact parameters are lg_system_desc::contact. */
typedef struct lg_connector_params {
    double k_d, gamma_d;
    double critical_separation;
} lg_connector_params;

/* hamaker_functor(A, h0, r_part, mass, ...)                hamaker_force.h:20-26
 * limited_range_hamaker_functor(A, h0, r_cutoff, r_part, mass, ...) limited_range_hamaker_force.h:20-27
 * simplified_hamaker_functor(A, h0, r_part, mass, ...)     simplified_hamaker_force.h:10-16
 * surface_hamaker_functor(A, h0, r_part, mass, ...)        surface_hamaker_force.h:10-15 */
typedef struct lg_hamaker_params {
    double A, h0, r_cutoff, r_part, mass;
} lg_hamaker_params;

/* triangular_facet(v_facet, {v0, v1, v2}, surface functors...), triangular_facet.h:18-19, with an
 * optional surface_contact_force_functor and an optional surface_hamaker_functor folded in that
 * order (triangular_facet.h:32-51). */
typedef struct lg_facet_desc {
    double v_facet[3];
    double vertices[9];
    int32_t has_contact;
    int32_t has_hamaker;
    lg_contact_params contact;
    lg_hamaker_params hamaker;
} lg_facet_desc;

/* Everything the granular_system constructor and its functor list fix at compile/construct time
 * (granular_system.h:53-63; granular_system_neighbor_list.h:54-64 adds n_part and r_verlet). */
/* ---- step-handler hooks and body forces (types) ------------------------------------------- */

/* Held increments (a custom step handler that holds particles, Custom-step-handler.md:82-97, whose
 * fixed_particle_step_handler skips increment_v of one particle): mask[i] is a bit set of the
 * increments the integrator skips for particle i, in both half kicks and in the drift. With
 * connectors (LG_BINARY_SINTER_CONNECTORS) a held x or theta also keeps the particle's connectors
 * (the skipped call is sinter_step_handler's, sinter_bridge.h:24-42, 55-75). */
#define LG_HOLD_X 1
#define LG_HOLD_V 2
#define LG_HOLD_THETA 4
#define LG_HOLD_OMEGA 8

/* Unary body force appended to the unary functor container after the facets (the container folds
 * its functors as f0 + (f1 + (... + body)), unary_force_container.h:27-29).
 *   LG_BODY_CENTRAL: central_attraction_functor of Custom-unary-force-model.md:66-120,
 *     a = k_a / mass * (centre - x_i), alpha = 0; the centre is set with lg_set_body_centre (the
 *     tutorial's update_center_of_mass), one centre per system of a batch. */
#define LG_BODY_NONE 0
#define LG_BODY_CENTRAL 1
typedef struct lg_body_force {
    int32_t model;     /* LG_BODY_* */
    double k_a;        /* N/m */
    double mass;       /* kg */
    double centre[3];  /* initial centre of every system */
} lg_body_force;

/* User-defined unary functor on the device (in place of a body force): called on the host once per
 * force evaluation, or once per captured graph (replays relaunch what it launched), it launches
 * work on `stream` that writes every particle's unary terms into a_out and alpha_out. Device
 * arrays hold 4 doubles per particle (x, y, z, unused). The terms join the fold like a body force.
 * Return 0, or nonzero to fail the step. include/libgran_gb300/libgran/body_force/device_unary.cuh
 * builds such a hook from a __device__ functor. */
typedef struct lg_unary_hook_args {
    int64_t n;
    const double *x, *v, *theta, *omega; /* the evaluation's positions and half-step velocities */
    double *a_out, *alpha_out;
    const int32_t *system_of;            /* batch: system index per particle; NULL otherwise */
    double dt;
    void *stream;                        /* cudaStream_t */
} lg_unary_hook_args;
typedef int (*lg_unary_hook)(const lg_unary_hook_args *args, void *user);

typedef struct lg_system_desc {
    int64_t n_part;
    int32_t binary_model;    /* LG_BINARY_* */
    int32_t hamaker_model;   /* LG_HAMAKER_* */
    lg_contact_params contact;  /* contact functor, or the sintered functor's inner contact copy */
    lg_sinter_params sinter;    /* used by LG_BINARY_SINTER / LG_BINARY_BREAKING_SINTER */
    lg_hamaker_params hamaker;  /* used unless hamaker_model == LG_HAMAKER_NONE */
    int32_t neck_mode;       /* LG_NECK_* */
    int32_t pairs;           /* LG_PAIRS_* */
    double r_verlet;         /* list radius (centre distance) for LG_PAIRS_VERLET */
    int32_t precision;       /* LG_PRECISION_* */
    int32_t n_facets;        /* number of lg_facet_desc passed to lg_create */
    int32_t facet_auto_move; /* 1: move every facet by v_facet*dt after each step */
    int32_t max_neighbors;   /* Verlet list row capacity; 0 picks a default */
    int32_t threads_per_row; /* lanes per row group of the force kernel (see lg_set_threads_per_row);
                                0 picks automatically; used from the construction-time evaluation on */
    int32_t force_kernel;    /* LG_FORCE_KERNEL_*: which force kernel evaluates the pairs */
    /* LG_BINARY_SINTER_CONNECTORS: */
    lg_connector_params connector;
    const double *connector_axes; /* per bond in detection order (i ascending, then j > i), the unit
                                     vector that sinter_bridge.h:169-175 draws from the caller's
                                     generator for it (3 doubles); it must not be parallel to the
                                     bond axis */
    int64_t n_connector_axes;     /* must equal the number of bonds found */
    /* step-handler hook and unary terms in force from construction on (the construction-time force
     * evaluation includes them, as the reference's containers do): */
    const uint8_t *hold_mask;     /* n bytes of LG_HOLD_* bits, or NULL */
    lg_body_force body;           /* model LG_BODY_NONE (zero-initialised): none */
    lg_unary_hook unary_hook;     /* or NULL; excludes a body force */
    void *unary_hook_user;
} lg_system_desc;

/* Force kernels. Both give deterministic sums; in FP64 both add each row in ascending j, and the
 * compacted kernel and the row-group kernel with one lane per row are bit-identical to a
 * sequential evaluation of libgran's functors. */
#define LG_FORCE_KERNEL_AUTO 0       /* mixed: compacted; FP64: pair-parallel for small systems, compacted
                                       for large ones */
#define LG_FORCE_KERNEL_ROWGROUP 1   /* T lanes per row (threads_per_row), fixed butterfly combine */
#define LG_FORCE_KERNEL_COMPACT 2    /* one row per lane, warp-compacted pair queues (see csrc) */
#define LG_FORCE_KERNEL_PAIRS 3      /* FP64, small systems: one thread per pair slot spread over all SMs,
                                       then an ordered per-row fold (the reference's summation order) */
#define LG_FORCE_KERNEL_PERSISTENT 4 /* mixed: every step inside a run of steps (no facets, body terms or
                                       held particles) is one persistent launch whose warps pull contact
                                       and Hamaker work items of 32-row groups from a device queue and
                                       complete each group when its last item finishes; the same bits as
                                       the compacted kernels. Other steps use the compacted kernels. */
#define LG_FORCE_KERNEL_FP64_FAST 5  /* FP64: the compacted kernel with one reciprocal where libgran divides a
                                       vector by a scalar, and the Hamaker bracket over one common
                                       denominator (2 divisions per Hamaker pair instead of 12, 2 per
                                       contact scaling instead of 6); contact is decided by the reference's
                                       exact overlap. Per-step forces within
                                       1e-12 of the reference's, not bit-identical; chosen explicitly only
                                       (never by AUTO or the autotuner). */

/* Fields that lg_get / lg_set move. */
#define LG_FIELD_X 0       /* positions            get_x()     Granular-system.md:84-120 */
#define LG_FIELD_V 1       /* velocities           get_v() */
#define LG_FIELD_THETA 2   /* orientations         get_theta() */
#define LG_FIELD_OMEGA 3   /* angular velocities   get_omega() */
#define LG_FIELD_A 4       /* translational acceleration buffer of the last force evaluation */
#define LG_FIELD_ALPHA 5   /* angular acceleration buffer of the last force evaluation */

/* Observables of test/compute_energy.cpp:7-58 and test/mass_distribution.cpp:7-27, plus the
 * potential energy bookkeeping that the reference lacks (spring and Hamaker potentials). */
typedef struct lg_observables {
    double ke_translational, ke_rotational, ke_total;
    double linear_momentum;   /* |sum m v| */
    double angular_momentum;  /* |sum I w + x x m v| */
    double center_of_mass[3];
    double radius_of_gyration;
    double potential_energy;  /* normal springs + tangential springs + Hamaker */
    int64_t n_contacts;       /* ordered pairs with positive overlap (non-bonded) */
    int64_t n_bonds;          /* ordered bonded pairs still intact */
    int64_t n_bonds_initial;  /* ordered bonded pairs at construction */
} lg_observables;

typedef struct lg_system lg_system; /* opaque */

/* Build version string, e.g. "libgran_gb300 0.1 sm_103a". Never fails. */
const char *lg_version(void);

/* Description of the last error raised on the calling thread ("" if none). */
const char *lg_last_error(void);

/* Number of CUDA devices visible (0 without a GPU). Returns LG_OK or LG_E_CUDA. */
int lg_device_count(int *count);

/* Construct a system: granular_system ctor (granular_system.h:53-63) together with the functor
 * constructors, including the bond detection of alt_sinter_functor (alt_sinter_bridge.h:55-89,
 * cycle-free) or alt_breaking_sinter_functor (alt_breaking_sinter_bridge.h:37-77).
 * x0, v0, theta0, omega0: double[3*n]. facets: n_facets descriptors (may be NULL if 0).
 * neck_strengths: one value per bond in detection order (i ascending, then j > i ascending), as the
 * reference draws them from its distribution (alt_breaking_sinter_bridge.h:70); only read for
 * LG_BINARY_BREAKING_SINTER; n_neck_strengths must equal the number of bonds found, or be 0 to
 * mean "no strength" (+infinity). The initial accelerations are evaluated here, as the integrator's
 * first half kick needs them. */
int lg_create(const lg_system_desc *desc, const double *x0, const double *v0, const double *theta0,
              const double *omega0, const lg_facet_desc *facets, const double *neck_strengths,
              int64_t n_neck_strengths, int device, lg_system **out);

/* Release every resource of the handle. NULL is accepted. */
int lg_destroy(lg_system *sys);

/* Advance nsteps steps of size dt: nsteps x do_step(dt) (Granular-system.md:65-80), each a
 * rotational velocity-Verlet step with one force evaluation. With LG_PAIRS_VERLET and
 * rebuild_every > 0, the Verlet list is rebuilt before every step whose global step index is a
 * multiple of rebuild_every (test/hamaker_neighbor.cpp:121-122 uses 20). Asynchronous with respect
 * to the host; errors from the device surface at the next synchronising call. */
int lg_step(lg_system *sys, double dt, int64_t nsteps, int64_t rebuild_every);

/* Rebuild the Verlet list now: update_neighbor_list() (test/hamaker_neighbor.cpp:122). Spring
 * history of pairs present before and after is carried over. */
int lg_update_neighbor_list(lg_system *sys);

/* Copy a field to/from the host (double[3*n]). lg_get synchronises the handle's stream. */
int lg_get(lg_system *sys, int field, double *out);
int lg_set(lg_system *sys, int field, const double *in);

/* The whole kinematic state in one call (x, v, theta, omega; double[3*n] each, any may be NULL to
 * skip it): one copy per array, one conversion pass, one synchronisation, instead of four of each.
 * Same meaning as the lg_get / lg_set calls of the fields given. */
int lg_get_state(lg_system *sys, double *x, double *v, double *theta, double *omega);
int lg_set_state(lg_system *sys, const double *x, const double *v, const double *theta, const double *omega);

/* reset_acceleration_buffers() (Granular-system.md:228-244): zero a and alpha. */
int lg_reset_acceleration_buffers(lg_system *sys);

/* Reductions on the device: observables of test/compute_energy.cpp and test/mass_distribution.cpp. */
int lg_get_observables(lg_system *sys, lg_observables *out);

/* The same observables, restricted to the parts requested (fields of parts not requested are 0;
 * n_bonds_initial is always set): LG_OBS_STATE = kinetic energies, momenta, centre of mass,
 * radius of gyration (per-particle sums, cheap); LG_OBS_PAIRS = potential energy, contacts, bonds
 * (a pass over every pair slot). lg_get_observables is LG_OBS_STATE | LG_OBS_PAIRS. */
#define LG_OBS_STATE 1
#define LG_OBS_PAIRS 2
int lg_get_observables_select(lg_system *sys, int32_t parts, lg_observables *out);

/* Device error word (bit set of LG_DEVERR_*) accumulated since creation; synchronises. */
#define LG_DEVERR_LIST_OVERFLOW 1    /* a Verlet list row exceeded its capacity */
#define LG_DEVERR_NONFINITE 2        /* a non-finite acceleration was produced */
#define LG_DEVERR_BOND_LOST 4        /* a bonded pair fell out of the Verlet list */
int lg_get_device_errors(lg_system *sys, int32_t *errors);

/* Bond bookkeeping of the sintered functors.
 * lg_get_bonds: number of ordered bonded pairs still intact, and optionally (i, j) of each, sorted
 * (the nonzero entries of bonded_contacts, alt_sinter_bridge.h:163). out_pairs may be NULL;
 * capacity is the number of int64 pairs it can hold. */
int lg_get_bonds(lg_system *sys, int64_t *n_bonds, int64_t *out_pairs, int64_t capacity);

/* Spring state of an ordered pair (i, j): 9 doubles (xi_t, xi_r, xi_o), the tuple of
 * contact_force_functor::contact_springs[i*n+j] (contact_force.h:156) for non-bonded pairs and of
 * alt_sinter_functor::get_contact_springs()[i*n+j] (alt_sinter_bridge.h:159-161) for bonded pairs.
 * Pairs not tracked (outside the Verlet list) report zeros. */
int lg_get_pair_springs(lg_system *sys, int64_t i, int64_t j, double *out9);

/* Facet control: triangular_facet::update_positions(dt) (triangular_facet.h:62-66) and the current
 * vertices (get_vertices(), triangular_facet.h:57-59). */
int lg_facet_update_positions(lg_system *sys, int32_t facet, double dt);
int lg_facet_get_vertices(lg_system *sys, int32_t facet, double *out9);

/* ---- step-handler hooks and body forces -------------------------------------------------- */

/* Replace the hold mask (n bytes of LG_HOLD_* bits; NULL holds nothing), from the next step on. */
int lg_set_hold_mask(lg_system *sys, const uint8_t *mask);
/* Replace the body force (NULL removes it), from the next force evaluation on. */
int lg_set_body_force(lg_system *sys, const lg_body_force *force);
/* centres: 3 doubles per system (one system unless the handle is a batch); queued on the handle's
 * stream, takes effect from the next force evaluation. */
int lg_set_body_centre(lg_system *sys, const double *centres);
/* Replace the unary hook (hook NULL removes it), from the next force evaluation on. */
int lg_set_unary_hook(lg_system *sys, lg_unary_hook hook, void *user);

/* ---- state dumps (libgran's writer.cpp formats) ------------------------------------------- */

/* ASCII VTK files as libgran's writer writes them (writer.cpp:13-170): coordinates divided by
 * r_part, numbers as std::ostream prints doubles by default ("%.6g"), the same headers and
 * separators. lg_write_* take the handle's current state; lg_format_* take host arrays and need no
 * GPU. Output goes to `path` (libgran's writer numbers files in a directory itself; the drop-in
 * writer.h keeps that naming).
 *   particles:  write_particles (writer.cpp:51-118): points, and the fields thetax/thetay/thetaz
 *               (the rotated unit axes of AngleAxis(theta_x, X) AngleAxis(theta_y, Y)
 *               AngleAxis(theta_z, Z)); theta: 3n doubles
 *   necks:      write_necks (writer.cpp:120-170): midpoint and unit normal (x_i - x_j) of every
 *               intact bond i < j in (i, j) order; pairs: n_pairs (i, j) int64 pairs
 *   connectors: write_spring_connectors (writer.cpp:13-49): the 5 connector points of every bond
 *               end, particle i ascending, then partner j ascending (5-connector model)
 *   csv:        the tutorials' dump_particle_positions: "x, y, z" then one line per particle. */
int lg_write_vtk_particles(lg_system *sys, const char *path, double r_part);
int lg_write_vtk_necks(lg_system *sys, const char *path, double r_part);
int lg_write_vtk_connectors(lg_system *sys, const char *path, double r_part);
int lg_write_csv_positions(lg_system *sys, const char *path, double r_part);
int lg_format_vtk_particles(const double *x, const double *theta, int64_t n, double r_part, const char *path);
int lg_format_vtk_necks(const double *x, int64_t n, const int64_t *pairs, int64_t n_pairs, double r_part,
                        const char *path);
int lg_format_vtk_connectors(const double *points, int64_t n_points, double r_part, const char *path);
int lg_format_csv_positions(const double *x, int64_t n, double r_part, const char *path);
/* Connector points of the 5-connector model in the order of lg_write_vtk_connectors (3 doubles
 * each, 5 per bond end); n_points is set to the total; out may be NULL. */
int lg_get_connectors(lg_system *sys, int64_t *n_points, double *out, int64_t capacity);

/* Number of CUDA kernel launches issued by this handle since creation (diagnostics). */
int lg_get_launch_count(lg_system *sys, int64_t *count);

/* Pair-slot statistics of the current pair data: mean and maximum row length (all-pairs mode: n-1),
 * and the number of ordered pairs whose contact springs are live or that are intact bonds. */
typedef struct lg_pair_stats {
    double mean_row_length;
    int64_t max_row_length;
    int64_t live_contact_slots;
    int64_t bonded_slots;
} lg_pair_stats;
int lg_get_pair_stats(lg_system *sys, lg_pair_stats *out);

/* Kernel timing: while enabled, every force-kernel launch is bracketed by CUDA events on the
 * handle's stream; lg_get_force_kernel_time returns the summed device time (ms) and the number of
 * launches timed since the last reset (the call synchronises and resets the counters). */
int lg_enable_kernel_timing(lg_system *sys, int32_t enable);
int lg_get_force_kernel_time(lg_system *sys, double *ms_total, int64_t *launches);

/* Lanes per row group of the force kernel: 1 walks each row sequentially (the reference's summation
 * order), 2..32 split a row across lanes and combine the partial sums with a fixed butterfly
 * (deterministic, different rounding). 0 restores the automatic choice. */
int lg_set_threads_per_row(lg_system *sys, int32_t threads_per_row);

/* Select the force kernel (LG_FORCE_KERNEL_*) for the following steps. */
int lg_set_force_kernel(lg_system *sys, int32_t force_kernel);

/* Seeded synthetic aggregate: random sequential attachment of n spheres of radius r (each new sphere
 * touches a uniformly chosen existing one in a uniformly random direction; a candidate that overlaps
 * any other sphere by more than 1e-12 r is rejected). x: double[3n]. Host-only, no GPU needed. */
int lg_generate_rsa_aggregate(uint64_t seed, int64_t n, double r, double *x);

/* Uniform random velocity components in [-vmax, vmax] from a seeded stream. Host-only. */
int lg_generate_velocities(uint64_t seed, int64_t n, double vmax, double *v);

/* CUDA graphs: lg_step replays each whole rebuild period (or 16 steps without a Verlet list) as one
 * captured graph from the second period on (default on). 0 disables and frees the graphs. */
int lg_set_graphs(lg_system *sys, int32_t enable);

/* ---- batches: many independent aggregates in one handle ------------------------------------
 * Every system of a batch is simulated exactly as it would be alone (its own bonds, pair rows and
 * springs; rows never cross systems), with the functor parameters of `desc` shared by all. desc
 * n_part is the total particle count, sizes[n_systems] the particle count of each system, and the
 * state arrays hold the systems one after another, each in its own coordinates. Verlet pairs only.
 * Facets apply to every system in that system's coordinates. Neck strengths: per bond, system by
 * system. All single-system calls (lg_step, lg_get, ...) act on the whole batch. */
int lg_batch_create(const lg_system_desc *desc, int64_t n_systems, const int64_t *sizes, const double *x0,
                    const double *v0, const double *theta0, const double *omega0, const lg_facet_desc *facets,
                    const double *neck_strengths, int64_t n_neck_strengths, int device, lg_system **out);
/* Number of systems (0 for a single system) and, if offsets is not NULL, their prefix offsets
 * (n_systems + 1 values). */
int lg_batch_info(lg_system *sys, int64_t *n_systems, int64_t *offsets);
/* Observables of every system: out[n_systems]. */
int lg_batch_get_observables(lg_system *sys, lg_observables *out);

/* Device-state snapshot of the handle (state, springs, bonds, pair rows, facets) and its restore; one
 * snapshot slot per handle, allocated on first use (about the handle's own device footprint). */
int lg_snapshot(lg_system *sys);
int lg_restore(lg_system *sys);

/* Project autotuner (the reference's only tuning knob is the OpenMP thread count): times the
 * force-kernel variants and shapes -- compacted kernels (mixed: with two or one contact lanes per
 * row); row groups of 1..32 lanes; FP64: the pair-parallel kernel; mixed: the persistent step kernel
 * in every shape of lg_set_step_shape (register budget 4/5/6 blocks per SM x 1/2/4 Hamaker slices x
 * pulled / round-robin items / two launches side by side) -- for probe_steps steps on the live
 * system between a snapshot and its restore (the state afterwards is the state before the call),
 * graph-replayed, best of two timings each, and keeps the fastest. The choice is cached per
 * (precision, pair mode, functor set, log2 size, batch) when use_cache is 1. *threads_per_row
 * receives the pick's threads_per_row (lg_tuning). */
int lg_autotune(lg_system *sys, double dt, int64_t probe_steps, int64_t rebuild_every, int32_t *force_kernel,
                int32_t *threads_per_row, int32_t use_cache);

/* A handle's (or a cache entry's) kernel choice and shape. ms_per_step: the autotuner's timing of
 * it (0 when not timed). */
typedef struct {
    int32_t force_kernel;     /* LG_FORCE_KERNEL_* (resolved, never AUTO) */
    int32_t threads_per_row;  /* row groups: lanes per row; mixed compacted kernels: contact lanes per row (1 or 2) */
    int32_t step_min_blocks;  /* persistent step kernel: register budget (resident blocks per SM) */
    int32_t step_slices;      /* persistent step kernel: Hamaker items per 32-row group */
    int32_t step_assign;      /* persistent step kernel: 0 pulled items, 1 round robin */
    double ms_per_step;
} lg_tuning;
int lg_get_tuning(lg_system *sys, lg_tuning *out);
/* The autotuner's cache: a lookup for a descriptor, size and batch flag (LG_E_STATE when absent),
 * and a text file to keep picks across processes (one entry per line; load merges). */
int lg_autotune_cache_lookup(const lg_system_desc *desc, int64_t n, int32_t batch, lg_tuning *out);
int lg_autotune_cache_save(const char *path);
int lg_autotune_cache_load(const char *path);
int lg_autotune_cache_clear(void);

/* Observables of a particle state held in device memory that the caller owns, computed without
 * allocating any device memory. No counterpart in the reference: it serves callers that cannot
 * allocate when they need these numbers -- a serving loop that admits work against a fixed device
 * memory budget, a host framework whose own caching allocator holds the device memory, code that
 * must not stall other streams (cudaMalloc and cudaFree can synchronise the device).
 *   x, v, omega: device arrays double[3n] (AoS); out: device array of LG_NOALLOC_OBS doubles:
 *   0 translational KE, 1 rotational KE, 2 total KE, 3 |linear momentum|, 4 |angular momentum|,
 *   5..7 centre of mass, 8 radius of gyration. stream: a cudaStream_t (NULL = default stream); the
 *   call is asynchronous.
 * Limit: 1 <= n <= LG_NOALLOC_MAX_PARTICLES, else LG_E_INVALID with a message. Partial sums live in
 * one fixed 512 KiB array in device memory that every GPU loading this library holds until the
 * process exits; all calls share it, so calls that overlap on the GPU (e.g. on two streams at once)
 * race and must be serialised by the caller. The first call on each device looks up the array's
 * device address (set-up, with that device current); make that first call before any stream
 * capture. Later calls outside a capture look the address up again (a cudaDeviceReset reloads the
 * module and can move the array); a call during a capture uses the address of the last call made
 * outside one. Calls no cudaMalloc, cudaFree or allocating library routine. */
#define LG_NOALLOC_OBS 9
#define LG_NOALLOC_MAX_PARTICLES 1048320
int lg_observables_noalloc(const double *x, const double *v, const double *omega, int64_t n, double mass,
                           double inertia, double *out, void *stream);

/* Shape of the persistent step kernel (LG_FORCE_KERNEL_PERSISTENT, mixed precision; no
 * counterpart in the reference): min_blocks = register budget as resident blocks per SM (4, 5 or
 * 6; 0 = 4), slices = Hamaker items per 32-row group (1, 2 or 4; 0 = the size rule the compacted
 * kernels use, which gives their bits), assign = 0 (warps pull work items from a device counter),
 * 1 (round robin) or 2 (contact and Hamaker items as two launches side by side, each compiled for its
 * own items, each pulling from its own counter; the last of a group's items completes it, so no
 * completion kernel follows). Every shape gives the same bits for the same slices. lg_autotune
 * chooses a shape when it tries the persistent kernel. */
int lg_set_step_shape(lg_system *sys, int32_t min_blocks, int32_t slices, int32_t assign);
int lg_get_step_shape(lg_system *sys, int32_t *min_blocks, int32_t *slices, int32_t *assign);

/* Time `nsteps` steps with CUDA events on the handle's stream (no host copies inside); ms_out
 * receives the elapsed device time. Same semantics as lg_step. */
int lg_step_timed(lg_system *sys, double dt, int64_t nsteps, int64_t rebuild_every, float *ms_out);

/* ---- serving: continuous batching of aggregate-mechanics requests ---------------------------
 * No counterpart in libgran (its drivers run one system per process). A server holds a system
 * template (functors, Verlet pairs, precision; no facets, body forces or hold masks), a
 * device-memory budget and a step size, and keeps one batch of slots of fixed capacities (size
 * classes; lg_server_set_slots, or by default 8 slots each of 128 .. 8192 monomers, fewer when the
 * budget is small). Requests (an aggregate state and a step budget) may be submitted at any time;
 * a request occupies the smallest free slot that holds it, and every resident request advances in
 * the same launches, one rebuild period at a time. Each lg_server_tick waits for the period in
 * flight, retires finished requests (observables and positions copied back, slot freed), admits
 * queued requests into free slots at rebuild boundaries (first come first served, with backfill;
 * each is first built alone from the template -- bond detection, construction force evaluation --
 * and then moved into its slot on the device), launches the next period and prepares queued
 * requests while it runs. A request evolves as it would alone: bit for bit in FP64, and in mixed
 * precision when the lone run uses the server's Hamaker slicing (lg_server_stats.hamaker_slices,
 * lg_set_step_shape) and step budgets are multiples of the rebuild period. Latency = host time from
 * submission to retirement. */
#define LG_REQ_QUEUED 0
#define LG_REQ_RUNNING 1
#define LG_REQ_DONE 2
#define LG_REQ_FAILED 3
#define LG_REQ_CANCELLED 4

typedef struct lg_server lg_server;
typedef struct lg_server_stats {
    int64_t budget_bytes, used_bytes, peak_bytes;
    int64_t active, queued, completed, rejected, failed, cancelled;
    int64_t particle_steps;
    double p50_latency_ms, p99_latency_ms, max_latency_ms;
    int64_t slots, slots_busy;              /* slots of the batch, slots holding a request */
    int64_t slot_particles, resident_particles;  /* capacity of all slots, particles of the residents */
    int32_t hamaker_slices;                 /* mixed precision: Hamaker slices of the batch's kernels */
    double device_ms;                       /* device time of the periods run (CUDA events) */
    int64_t periods;                        /* periods run */
} lg_server_stats;

/* Device bytes a system of n particles (a request alone, or the slots together) is charged. */
int64_t lg_estimate_device_bytes(const lg_system_desc *tmpl, int64_t n);
int lg_server_create(const lg_system_desc *tmpl, int64_t budget_bytes, int64_t rebuild_every, double dt, int device,
                     lg_server **out);
int lg_server_destroy(lg_server *srv);
/* Slot capacities (before the first admission); LG_E_NOMEM when they do not fit the budget. */
int lg_server_set_slots(lg_server *srv, const int64_t *capacities, int64_t count);
/* Queue a request (x0, v0: double[3n]; v0 may be NULL). Malformed requests (n < 1, nsteps < 1,
 * non-finite state) fail with LG_E_INVALID; a request larger than the largest slot with LG_E_NOMEM. */
int lg_server_submit(lg_server *srv, int64_t n, const double *x0, const double *v0, int64_t nsteps,
                     int64_t *request_id);
int lg_server_cancel(lg_server *srv, int64_t request_id);
int lg_server_tick(lg_server *srv, int32_t *n_active, int32_t *n_queued, int32_t *n_retired);
/* State (LG_REQ_*) of a request; when done, its observables and final positions (double[3n], may be
 * NULL) and its latency. A failed request's reason is in lg_last_error(). */
int lg_server_poll(lg_server *srv, int64_t request_id, int32_t *state, lg_observables *obs, double *x_out,
                   double *latency_ms);
int lg_server_release(lg_server *srv, int64_t request_id);
int lg_server_get_stats(lg_server *srv, lg_server_stats *out);
/* Test hook: the next `count` admissions fail as a device allocation failure would (host side). */
int lg_server_inject_alloc_failures(lg_server *srv, int32_t count);

#ifdef __cplusplus
}
#endif

#endif /* LIBGRAN_GB300_H */
