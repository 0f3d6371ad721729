"""ctypes mirror of the C ABI declared in include/libgran_gb300.h.

The structures here have the same field order and types as the C structs; the loader finds the
in-tree shared library built by ``__graft_entry__.build()`` and fails loudly when it is missing, so
no code path silently falls back to anything else.
"""
import ctypes as C
import os

LG_OK = 0
LG_E_INVALID, LG_E_CUDA, LG_E_NOMEM, LG_E_STATE, LG_E_DEVICE = -1, -2, -3, -4, -5

LG_BINARY_NONE, LG_BINARY_CONTACT, LG_BINARY_SINTER, LG_BINARY_BREAKING_SINTER = 0, 1, 2, 3
LG_BINARY_SINTER_CONNECTORS = 4
LG_HAMAKER_NONE, LG_HAMAKER_FULL, LG_HAMAKER_LIMITED, LG_HAMAKER_SIMPLIFIED = 0, 1, 2, 3
LG_NECK_PER_BOND, LG_NECK_REFERENCE_INDEXING = 0, 1
LG_PRECISION_FP64, LG_PRECISION_MIXED = 0, 1
LG_PAIRS_ALL, LG_PAIRS_VERLET = 0, 1
LG_FORCE_KERNEL_AUTO, LG_FORCE_KERNEL_ROWGROUP, LG_FORCE_KERNEL_COMPACT, LG_FORCE_KERNEL_PAIRS = 0, 1, 2, 3
LG_FORCE_KERNEL_PERSISTENT = 4
LG_FORCE_KERNEL_FP64_FAST = 5
LG_FIELD_X, LG_FIELD_V, LG_FIELD_THETA, LG_FIELD_OMEGA, LG_FIELD_A, LG_FIELD_ALPHA = range(6)
LG_DEVERR_LIST_OVERFLOW, LG_DEVERR_NONFINITE, LG_DEVERR_BOND_LOST = 1, 2, 4
LG_NOALLOC_OBS, LG_NOALLOC_MAX_PARTICLES = 9, 1048320
LG_OBS_STATE, LG_OBS_PAIRS = 1, 2
LG_REQ_QUEUED, LG_REQ_RUNNING, LG_REQ_DONE, LG_REQ_FAILED, LG_REQ_CANCELLED = 0, 1, 2, 3, 4
LG_HOLD_X, LG_HOLD_V, LG_HOLD_THETA, LG_HOLD_OMEGA = 1, 2, 4, 8
LG_BODY_NONE, LG_BODY_CENTRAL = 0, 1


class lg_contact_params(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "k", "gamma_n", "k_t", "gamma_t", "mu_s", "phi_d", "k_r", "gamma_r", "mu_r", "phi_r",
        "k_o", "gamma_o", "mu_o", "phi_o", "r_part", "mass", "inertia", "dt")]


class lg_sinter_params(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "k", "gamma_n", "k_t", "gamma_t", "k_r", "gamma_r", "k_o", "gamma_o",
        "r_part", "mass", "inertia", "dt", "critical_separation")]


class lg_connector_params(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("k_d", "gamma_d", "critical_separation")]


class lg_hamaker_params(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("A", "h0", "r_cutoff", "r_part", "mass")]


class lg_facet_desc(C.Structure):
    _fields_ = [("v_facet", C.c_double * 3), ("vertices", C.c_double * 9),
                ("has_contact", C.c_int32), ("has_hamaker", C.c_int32),
                ("contact", lg_contact_params), ("hamaker", lg_hamaker_params)]


class lg_pair_stats(C.Structure):
    _fields_ = [("mean_row_length", C.c_double), ("max_row_length", C.c_int64),
                ("live_contact_slots", C.c_int64), ("bonded_slots", C.c_int64)]


class lg_server_stats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("budget_bytes", "used_bytes", "peak_bytes", "active", "queued", "completed",
                                         "rejected", "failed", "cancelled", "particle_steps")] + \
               [(n, C.c_double) for n in ("p50_latency_ms", "p99_latency_ms", "max_latency_ms")] + \
               [(n, C.c_int64) for n in ("slots", "slots_busy", "slot_particles", "resident_particles")] + \
               [("hamaker_slices", C.c_int32), ("device_ms", C.c_double), ("periods", C.c_int64)]


class lg_body_force(C.Structure):
    _fields_ = [("model", C.c_int32), ("k_a", C.c_double), ("mass", C.c_double), ("centre", C.c_double * 3)]


class lg_unary_hook_args(C.Structure):
    _fields_ = [("n", C.c_int64), ("x", C.c_void_p), ("v", C.c_void_p), ("theta", C.c_void_p),
                ("omega", C.c_void_p), ("a_out", C.c_void_p), ("alpha_out", C.c_void_p),
                ("system_of", C.c_void_p), ("dt", C.c_double), ("stream", C.c_void_p)]


lg_unary_hook = C.CFUNCTYPE(C.c_int, C.POINTER(lg_unary_hook_args), C.c_void_p)


class lg_system_desc(C.Structure):
    _fields_ = [("n_part", C.c_int64), ("binary_model", C.c_int32), ("hamaker_model", C.c_int32),
                ("contact", lg_contact_params), ("sinter", lg_sinter_params),
                ("hamaker", lg_hamaker_params), ("neck_mode", C.c_int32), ("pairs", C.c_int32),
                ("r_verlet", C.c_double), ("precision", C.c_int32), ("n_facets", C.c_int32),
                ("facet_auto_move", C.c_int32), ("max_neighbors", C.c_int32), ("threads_per_row", C.c_int32),
                ("force_kernel", C.c_int32), ("connector", lg_connector_params),
                ("connector_axes", C.POINTER(C.c_double)), ("n_connector_axes", C.c_int64),
                ("hold_mask", C.POINTER(C.c_uint8)), ("body", lg_body_force), ("unary_hook", lg_unary_hook),
                ("unary_hook_user", C.c_void_p)]


class lg_tuning(C.Structure):
    _fields_ = [("force_kernel", C.c_int32), ("threads_per_row", C.c_int32), ("step_min_blocks", C.c_int32),
                ("step_slices", C.c_int32), ("step_assign", C.c_int32), ("ms_per_step", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class lg_observables(C.Structure):
    _fields_ = [("ke_translational", C.c_double), ("ke_rotational", C.c_double),
                ("ke_total", C.c_double), ("linear_momentum", C.c_double),
                ("angular_momentum", C.c_double), ("center_of_mass", C.c_double * 3),
                ("radius_of_gyration", C.c_double), ("potential_energy", C.c_double),
                ("n_contacts", C.c_int64), ("n_bonds", C.c_int64), ("n_bonds_initial", C.c_int64)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["center_of_mass"] = list(self.center_of_mass)
        return d


PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "_lib", "liblg_gb300.so")

_lib = None


def lib():
    """Load the engine's shared library (built in-tree by __graft_entry__.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            "libgran_gb300: CUDA engine library %s is missing; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    _declare(L)
    _lib = L
    return L


def _declare(L):
    P = C.POINTER
    d = C.c_double
    i64 = C.c_int64
    i32 = C.c_int32
    vp = C.c_void_p
    sig = {
        "lg_version": (C.c_char_p, []),
        "lg_last_error": (C.c_char_p, []),
        "lg_device_count": (C.c_int, [P(C.c_int)]),
        "lg_create": (C.c_int, [P(lg_system_desc), P(d), P(d), P(d), P(d), P(lg_facet_desc), P(d), i64,
                                C.c_int, P(vp)]),
        "lg_destroy": (C.c_int, [vp]),
        "lg_step": (C.c_int, [vp, d, i64, i64]),
        "lg_step_timed": (C.c_int, [vp, d, i64, i64, P(C.c_float)]),
        "lg_update_neighbor_list": (C.c_int, [vp]),
        "lg_get": (C.c_int, [vp, C.c_int, P(d)]),
        "lg_set": (C.c_int, [vp, C.c_int, P(d)]),
        "lg_reset_acceleration_buffers": (C.c_int, [vp]),
        "lg_get_observables": (C.c_int, [vp, P(lg_observables)]),
        "lg_get_observables_select": (C.c_int, [vp, C.c_int32, P(lg_observables)]),
        # plain addresses: the state calls sit on the per-exchange path, where building four
        # ctypes pointer objects costs more than the transfer's own host work
        "lg_get_state": (C.c_int, [vp, vp, vp, vp, vp]),
        "lg_set_state": (C.c_int, [vp, vp, vp, vp, vp]),
        "lg_get_device_errors": (C.c_int, [vp, P(i32)]),
        "lg_get_bonds": (C.c_int, [vp, P(i64), P(i64), i64]),
        "lg_get_pair_springs": (C.c_int, [vp, i64, i64, P(d)]),
        "lg_facet_update_positions": (C.c_int, [vp, i32, d]),
        "lg_facet_get_vertices": (C.c_int, [vp, i32, P(d)]),
        "lg_get_launch_count": (C.c_int, [vp, P(i64)]),
        "lg_set_threads_per_row": (C.c_int, [vp, i32]),
        "lg_set_force_kernel": (C.c_int, [vp, i32]),
        "lg_set_graphs": (C.c_int, [vp, i32]),
        "lg_batch_create": (C.c_int, [P(lg_system_desc), i64, P(i64), P(d), P(d), P(d), P(d), P(lg_facet_desc),
                                      P(d), i64, C.c_int, P(vp)]),
        "lg_batch_info": (C.c_int, [vp, P(i64), P(i64)]),
        "lg_batch_get_observables": (C.c_int, [vp, P(lg_observables)]),
        "lg_autotune": (C.c_int, [vp, d, i64, i64, P(i32), P(i32), i32]),
        "lg_snapshot": (C.c_int, [vp]),
        "lg_estimate_device_bytes": (i64, [P(lg_system_desc), i64]),
        "lg_server_create": (C.c_int, [P(lg_system_desc), i64, i64, d, C.c_int, P(vp)]),
        "lg_server_destroy": (C.c_int, [vp]),
        "lg_server_submit": (C.c_int, [vp, i64, P(d), P(d), i64, P(i64)]),
        "lg_server_cancel": (C.c_int, [vp, i64]),
        "lg_server_tick": (C.c_int, [vp, P(i32), P(i32), P(i32)]),
        "lg_server_poll": (C.c_int, [vp, i64, P(i32), P(lg_observables), P(d), P(d)]),
        "lg_server_release": (C.c_int, [vp, i64]),
        "lg_server_get_stats": (C.c_int, [vp, P(lg_server_stats)]),
        "lg_server_inject_alloc_failures": (C.c_int, [vp, i32]),
        "lg_server_set_slots": (C.c_int, [vp, P(i64), i64]),
        "lg_observables_noalloc": (C.c_int, [vp, vp, vp, i64, d, d, vp, vp]),
        "lg_set_step_shape": (C.c_int, [vp, i32, i32, i32]),
        "lg_get_tuning": (C.c_int, [vp, P(lg_tuning)]),
        "lg_autotune_cache_lookup": (C.c_int, [P(lg_system_desc), i64, i32, P(lg_tuning)]),
        "lg_autotune_cache_save": (C.c_int, [C.c_char_p]),
        "lg_autotune_cache_load": (C.c_int, [C.c_char_p]),
        "lg_autotune_cache_clear": (C.c_int, []),
        "lg_get_step_shape": (C.c_int, [vp, P(i32), P(i32), P(i32)]),
        "lg_restore": (C.c_int, [vp]),
        "lg_get_pair_stats": (C.c_int, [vp, P(lg_pair_stats)]),
        "lg_enable_kernel_timing": (C.c_int, [vp, i32]),
        "lg_get_force_kernel_time": (C.c_int, [vp, P(d), P(i64)]),
        "lg_generate_rsa_aggregate": (C.c_int, [C.c_uint64, i64, d, P(d)]),
        "lg_generate_velocities": (C.c_int, [C.c_uint64, i64, d, P(d)]),
        "lg_set_hold_mask": (C.c_int, [vp, P(C.c_uint8)]),
        "lg_set_body_force": (C.c_int, [vp, P(lg_body_force)]),
        "lg_set_body_centre": (C.c_int, [vp, P(d)]),
        "lg_set_unary_hook": (C.c_int, [vp, lg_unary_hook, vp]),
        "lg_write_vtk_particles": (C.c_int, [vp, C.c_char_p, d]),
        "lg_write_vtk_necks": (C.c_int, [vp, C.c_char_p, d]),
        "lg_write_vtk_connectors": (C.c_int, [vp, C.c_char_p, d]),
        "lg_write_csv_positions": (C.c_int, [vp, C.c_char_p, d]),
        "lg_format_vtk_particles": (C.c_int, [P(d), P(d), i64, d, C.c_char_p]),
        "lg_format_vtk_necks": (C.c_int, [P(d), i64, P(i64), i64, d, C.c_char_p]),
        "lg_format_vtk_connectors": (C.c_int, [P(d), i64, d, C.c_char_p]),
        "lg_format_csv_positions": (C.c_int, [P(d), i64, d, C.c_char_p]),
        "lg_get_connectors": (C.c_int, [vp, P(i64), P(d), i64]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


class LgError(RuntimeError):
    pass


def check(status, what=""):
    if status != LG_OK:
        msg = lib().lg_last_error().decode(errors="replace")
        raise LgError("%s failed (status %d): %s" % (what, status, msg))
