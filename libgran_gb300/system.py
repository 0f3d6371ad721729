"""Handle-level Python wrapper of the C ABI (one lg_system).

This is plumbing for tests, benchmarks and the libgran-style classes in ``granular.py``; every
call goes straight to the CUDA engine in ``_lib/liblg_gb300.so``.
"""
import ctypes as C

import numpy as np

from . import _abi as A


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _vec(a, n):
    if a is None:
        return np.zeros((n, 3))
    if type(a) is np.ndarray and a.dtype == np.float64 and a.shape == (n, 3) and a.flags.c_contiguous:
        return a  # the common case, without conversions
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(n, 3))


class System:
    """One simulated system (or, with ``sizes``, a batch of independent systems) resident on a GPU."""

    def __init__(self, desc, x0, v0=None, th0=None, om0=None, facets=None, neck=None, device=0, sizes=None):
        L = A.lib()
        self.n = int(desc.n_part)
        self.desc = desc
        self._x0 = _vec(x0, self.n)
        v0, th0, om0 = _vec(v0, self.n), _vec(th0, self.n), _vec(om0, self.n)
        fp = None
        if facets:
            self._facets = (A.lg_facet_desc * len(facets))(*facets)
            fp = C.cast(self._facets, C.POINTER(A.lg_facet_desc))
        neck_a = None if neck is None else np.ascontiguousarray(neck, dtype=np.float64)
        h = C.c_void_p()
        if sizes is None:
            A.check(L.lg_create(C.byref(desc), _dp(self._x0), _dp(v0), _dp(th0), _dp(om0), fp,
                                None if neck_a is None else _dp(neck_a), 0 if neck_a is None else len(neck_a),
                                int(device), C.byref(h)), "lg_create")
            self.sizes = None
        else:
            sz = np.ascontiguousarray(sizes, dtype=np.int64)
            A.check(L.lg_batch_create(C.byref(desc), len(sz), sz.ctypes.data_as(C.POINTER(C.c_int64)), _dp(self._x0),
                                      _dp(v0), _dp(th0), _dp(om0), fp, None if neck_a is None else _dp(neck_a),
                                      0 if neck_a is None else len(neck_a), int(device), C.byref(h)),
                    "lg_batch_create")
            self.sizes = sz
        self.h = h

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            A.lib().lg_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, dt, nsteps=1, rebuild_every=0):
        A.check(A.lib().lg_step(self.h, float(dt), int(nsteps), int(rebuild_every)), "lg_step")

    def step_timed(self, dt, nsteps=1, rebuild_every=0):
        ms = C.c_float()
        A.check(A.lib().lg_step_timed(self.h, float(dt), int(nsteps), int(rebuild_every), C.byref(ms)),
                "lg_step_timed")
        return ms.value

    def update_neighbor_list(self):
        A.check(A.lib().lg_update_neighbor_list(self.h), "lg_update_neighbor_list")

    def get(self, field, out=None):
        """Copy one per-particle field to the host: a new (n, 3) float64 array, or into `out` (a
        C-contiguous (n, 3) float64 array, e.g. a view of pinned memory)."""
        if out is None:
            out = np.empty((self.n, 3))
        elif out.dtype != np.float64 or out.shape != (self.n, 3) or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a C-contiguous (n, 3) float64 array")
        A.check(A.lib().lg_get(self.h, int(field), _dp(out)), "lg_get")
        return out

    def set(self, field, arr):
        a = _vec(arr, self.n)
        A.check(A.lib().lg_set(self.h, int(field), _dp(a)), "lg_set")

    def get_state(self, out=None):
        """(x, v, theta, omega) in one call: new (n, 3) arrays, or into the four C-contiguous (n, 3)
        float64 arrays of `out` (e.g. views of pinned memory)."""
        if out is None:
            out = tuple(np.empty((self.n, 3)) for _ in range(4))
        addrs = []
        for a in out:
            if a.dtype != np.float64 or a.shape != (self.n, 3) or not a.flags.c_contiguous:
                raise ValueError("state arrays must be C-contiguous (n, 3) float64")
            addrs.append(a.__array_interface__["data"][0])
        A.check(A.lib().lg_get_state(self.h, *addrs), "lg_get_state")
        return out

    def set_state(self, x=None, v=None, theta=None, omega=None):
        """Upload any of (x, v, theta, omega) in one call (None leaves a field unchanged)."""
        arrs = [None if a is None else _vec(a, self.n) for a in (x, v, theta, omega)]
        addrs = [None if a is None else a.__array_interface__["data"][0] for a in arrs]
        A.check(A.lib().lg_set_state(self.h, *addrs), "lg_set_state")  # arrs stay alive until it returns

    def set_threads_per_row(self, T):
        A.check(A.lib().lg_set_threads_per_row(self.h, int(T)), "lg_set_threads_per_row")

    def set_step_shape(self, min_blocks=0, slices=0, assign=0):
        """Shape of the persistent step kernel (register budget, Hamaker slices, item assignment)."""
        A.check(A.lib().lg_set_step_shape(self.h, int(min_blocks), int(slices), int(assign)), "lg_set_step_shape")

    def step_shape(self):
        mb, sl, asg = C.c_int32(), C.c_int32(), C.c_int32()
        A.check(A.lib().lg_get_step_shape(self.h, C.byref(mb), C.byref(sl), C.byref(asg)), "lg_get_step_shape")
        return {"min_blocks": mb.value, "slices": sl.value, "assign": asg.value}

    def set_force_kernel(self, variant):
        A.check(A.lib().lg_set_force_kernel(self.h, int(variant)), "lg_set_force_kernel")

    def set_hold_mask(self, mask):
        """Per-particle LG_HOLD_* bits of the increments the integrator skips (None: hold nothing)."""
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        if m is not None and m.shape != (self.n,):
            raise ValueError("hold mask needs one byte per particle")
        A.check(A.lib().lg_set_hold_mask(self.h, None if m is None else m.ctypes.data_as(C.POINTER(C.c_uint8))),
                "lg_set_hold_mask")

    def set_body_force(self, body):
        """An lg_body_force (None removes it)."""
        A.check(A.lib().lg_set_body_force(self.h, None if body is None else C.byref(body)), "lg_set_body_force")

    def set_body_centre(self, centres):
        """Centre of the central body force: 3 values, or 3 per system of a batch."""
        c = np.ascontiguousarray(centres, dtype=np.float64).reshape(-1)
        if c.size != 3 * (1 if self.sizes is None else len(self.sizes)):
            raise ValueError("one centre (3 values) per system")
        A.check(A.lib().lg_set_body_centre(self.h, _dp(c)), "lg_set_body_centre")

    def write_vtk(self, kind, path, r_part):
        """Dump the current state in libgran's writer format: kind "particles", "necks",
        "connectors", or "csv" (the tutorials' position dump)."""
        fn = {"particles": "lg_write_vtk_particles", "necks": "lg_write_vtk_necks",
              "connectors": "lg_write_vtk_connectors", "csv": "lg_write_csv_positions"}[kind]
        A.check(getattr(A.lib(), fn)(self.h, str(path).encode(), float(r_part)), fn)

    def connectors(self):
        """Connector points of the 5-connector model (bond ends by particle, then partner; 5 each)."""
        k = C.c_int64()
        A.check(A.lib().lg_get_connectors(self.h, C.byref(k), None, 0), "lg_get_connectors")
        out = np.zeros((max(k.value, 1), 3))
        A.check(A.lib().lg_get_connectors(self.h, C.byref(k), _dp(out), k.value), "lg_get_connectors")
        return out[:k.value]

    def reset_acceleration_buffers(self):
        A.check(A.lib().lg_reset_acceleration_buffers(self.h), "lg_reset_acceleration_buffers")

    def observables(self, parts=None):
        """Observables of the current state; `parts` (LG_OBS_STATE | LG_OBS_PAIRS bits) restricts
        them, e.g. LG_OBS_STATE skips the pass over the pair slots (potential energy, contacts)."""
        o = A.lg_observables()
        if parts is None:
            A.check(A.lib().lg_get_observables(self.h, C.byref(o)), "lg_get_observables")
        else:
            A.check(A.lib().lg_get_observables_select(self.h, int(parts), C.byref(o)), "lg_get_observables_select")
        return o.as_dict()

    def batch_observables(self):
        """Per-system observables of a batch (list of dicts)."""
        ns = len(self.sizes)
        arr = (A.lg_observables * ns)()
        A.check(A.lib().lg_batch_get_observables(self.h, C.cast(arr, C.POINTER(A.lg_observables))),
                "lg_batch_get_observables")
        return [arr[q].as_dict() for q in range(ns)]

    def snapshot(self):
        A.check(A.lib().lg_snapshot(self.h), "lg_snapshot")

    def restore(self):
        A.check(A.lib().lg_restore(self.h), "lg_restore")

    def set_graphs(self, on):
        A.check(A.lib().lg_set_graphs(self.h, 1 if on else 0), "lg_set_graphs")

    def autotune(self, dt, probe_steps=20, rebuild_every=20, use_cache=True):
        """Time the kernel variants and shapes on this system and keep the fastest; returns
        (force kernel, threads_per_row of the pick: row-group lanes, or contact lanes per row for the
        mixed compacted kernels)."""
        k, t = C.c_int32(), C.c_int32()
        A.check(A.lib().lg_autotune(self.h, float(dt), int(probe_steps), int(rebuild_every), C.byref(k), C.byref(t),
                                    1 if use_cache else 0), "lg_autotune")
        return k.value, t.value

    def tuning(self):
        """The handle's kernel choice and shape (lg_tuning as a dict)."""
        t = A.lg_tuning()
        A.check(A.lib().lg_get_tuning(self.h, C.byref(t)), "lg_get_tuning")
        return t.as_dict()

    def device_errors(self):
        e = C.c_int32()
        A.check(A.lib().lg_get_device_errors(self.h, C.byref(e)), "lg_get_device_errors")
        return e.value

    def bonds(self):
        L = A.lib()
        nb = C.c_int64()
        A.check(L.lg_get_bonds(self.h, C.byref(nb), None, 0), "lg_get_bonds")
        arr = np.zeros(2 * max(nb.value, 1), dtype=np.int64)
        A.check(L.lg_get_bonds(self.h, C.byref(nb), arr.ctypes.data_as(C.POINTER(C.c_int64)), nb.value),
                "lg_get_bonds")
        return arr[:2 * nb.value].reshape(nb.value, 2)

    def springs(self, i, j):
        out = np.zeros(9)
        A.check(A.lib().lg_get_pair_springs(self.h, int(i), int(j), _dp(out)), "lg_get_pair_springs")
        return out

    def facet_vertices(self, f):
        out = np.zeros(9)
        A.check(A.lib().lg_facet_get_vertices(self.h, int(f), _dp(out)), "lg_facet_get_vertices")
        return out

    def facet_update_positions(self, f, dt):
        A.check(A.lib().lg_facet_update_positions(self.h, int(f), float(dt)), "lg_facet_update_positions")

    def pair_stats(self):
        st = A.lg_pair_stats()
        A.check(A.lib().lg_get_pair_stats(self.h, C.byref(st)), "lg_get_pair_stats")
        return {k: getattr(st, k) for k, _ in st._fields_}

    def enable_kernel_timing(self, on=True):
        A.check(A.lib().lg_enable_kernel_timing(self.h, 1 if on else 0), "lg_enable_kernel_timing")

    def force_kernel_time(self):
        ms = C.c_double()
        cnt = C.c_int64()
        A.check(A.lib().lg_get_force_kernel_time(self.h, C.byref(ms), C.byref(cnt)), "lg_get_force_kernel_time")
        return ms.value, cnt.value

    def launch_count(self):
        c = C.c_int64()
        A.check(A.lib().lg_get_launch_count(self.h, C.byref(c)), "lg_get_launch_count")
        return c.value


def generate_aggregate(seed, n, r):
    """Seeded random-sequential-attachment aggregate of n spheres of radius r (host code)."""
    x = np.zeros((int(n), 3))
    A.check(A.lib().lg_generate_rsa_aggregate(C.c_uint64(seed), int(n), float(r), _dp(x)),
            "lg_generate_rsa_aggregate")
    return x


def generate_velocities(seed, n, vmax):
    v = np.zeros((int(n), 3))
    A.check(A.lib().lg_generate_velocities(C.c_uint64(seed), int(n), float(vmax), _dp(v)), "lg_generate_velocities")
    return v
