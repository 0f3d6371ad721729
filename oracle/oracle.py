"""Python access to the CPU oracle (liblg_oracle.so) and, where it was built, to the reference
harness (oracle/_ref/liblgref.so: libgran's own functor headers on the same system loop).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg as the checker. The product package never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from libgran_gb300 import _abi as A

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liblg_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "liblgref.so")
# where the harness recipe looks for the libgran source tree unless LIBGRAN_ROOT names another
DEFAULT_LIBGRAN_ROOT = "/root/reference"


def libgran_root():
    """The libgran source tree the reference harness compiles from: $LIBGRAN_ROOT, else the
    default location; None when neither holds libgran's include tree (the GPU machine)."""
    root = os.environ.get("LIBGRAN_ROOT") or DEFAULT_LIBGRAN_ROOT
    return root if os.path.isdir(os.path.join(root, "include", "libgran")) else None


def build_oracle(force=False):
    """Compile the C restatement (gcc, -ffp-contract=off so no multiply-add is fused)."""
    src = os.path.join(HERE, "lg_oracle.c")
    if not force and os.path.exists(ORACLE_SO) and os.path.getmtime(ORACLE_SO) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "lg_oracle.h"))):
        return ORACLE_SO
    cmd = ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", "-o", ORACLE_SO, src, "-lm"]
    subprocess.check_call(cmd)
    return ORACLE_SO


def build_ref(root=None):
    """Compile the reference harness from the libgran source tree when it is present."""
    root = root or libgran_root()
    if not root or not os.path.isdir(os.path.join(root, "include", "libgran")):
        return None
    subprocess.check_call(["make", "-s", "-C", os.path.join(HERE, "ref_harness"), "LIBGRAN=" + root,
                           "-j4"])
    return REF_SO


_olib = None
_rlib = None


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def olib():
    global _olib
    if _olib is None:
        build_oracle()
        L = C.CDLL(ORACLE_SO)
        P = C.POINTER
        d, i64, vp = C.c_double, C.c_int64, C.c_void_p
        L.lgo_create.restype = vp
        L.lgo_create.argtypes = [P(A.lg_system_desc), P(d), P(d), P(d), P(d), P(A.lg_facet_desc), P(d), i64,
                                 C.c_int]
        L.lgo_destroy.argtypes = [vp]
        L.lgo_step.argtypes = [vp, d, i64, i64]
        L.lgo_update_neighbor_list.argtypes = [vp]
        L.lgo_get.argtypes = [vp, C.c_int, P(d)]
        L.lgo_set.argtypes = [vp, C.c_int, P(d)]
        L.lgo_get_pair_springs.argtypes = [vp, i64, i64, P(d)]
        L.lgo_count_bonds.restype = i64
        L.lgo_count_bonds.argtypes = [vp, P(i64), i64]
        L.lgo_row_length.restype = i64
        L.lgo_row_length.argtypes = [vp, i64]
        L.lgo_row.restype = i64
        L.lgo_row.argtypes = [vp, i64, P(C.c_int32), i64]
        L.lgo_observables.argtypes = [vp, P(A.lg_observables)]
        L.lgo_facet_update_positions.argtypes = [vp, C.c_int32, d]
        L.lgo_facet_get_vertices.argtypes = [vp, C.c_int32, P(d)]
        L.lgo_step_index.restype = i64
        L.lgo_step_index.argtypes = [vp]
        L.lgo_run_many.argtypes = [P(vp), P(d), P(i64), P(i64), C.c_int]
        L.lgo_set_hold_mask.argtypes = [vp, P(C.c_uint8)]
        L.lgo_set_body_force.argtypes = [vp, P(A.lg_body_force)]
        L.lgo_set_body_centre.argtypes = [vp, P(d)]
        L.lgo_get_connectors.restype = i64
        L.lgo_get_connectors.argtypes = [vp, P(d), i64]
        L.lgo_generate_rsa_aggregate.argtypes = [C.c_uint64, i64, d, P(d)]
        L.lgo_generate_velocities.argtypes = [C.c_uint64, i64, d, P(d)]
        _olib = L
    return _olib


def rlib():
    """The reference harness library, or None when it is not built (no libgran tree here)."""
    global _rlib
    if _rlib is None:
        if not os.path.exists(REF_SO):
            if build_ref() is None:
                return None
        L = C.CDLL(REF_SO)
        P = C.POINTER
        d, i64, vp = C.c_double, C.c_int64, C.c_void_p
        L.lgref_create.restype = vp
        L.lgref_create.argtypes = [P(A.lg_system_desc), P(d), P(d), P(d), P(d), P(A.lg_facet_desc), P(d), i64]
        L.lgref_destroy.argtypes = [vp]
        L.lgref_step.argtypes = [vp, d, i64, i64]
        L.lgref_update_neighbor_list.argtypes = [vp]
        L.lgref_get.argtypes = [vp, C.c_int, P(d)]
        L.lgref_pair_springs.argtypes = [vp, i64, i64, P(d)]
        L.lgref_bonds.restype = i64
        L.lgref_bonds.argtypes = [vp, P(i64), i64]
        L.lgref_facet_get_vertices.argtypes = [vp, C.c_int32, P(d)]
        L.lgref_facet_update_positions.argtypes = [vp, C.c_int32, d]
        L.lgref_set_body_centre.argtypes = [vp, P(d)]
        _rlib = L
    return _rlib


def generate_aggregate(seed, n, r):
    """Seeded random-sequential-attachment aggregate of n spheres of radius r ([n, 3] positions),
    bit-identical to the engine's lg_generate_rsa_aggregate."""
    x = np.zeros((int(n), 3))
    if olib().lgo_generate_rsa_aggregate(C.c_uint64(seed), int(n), float(r), _dp(x)) != 0:
        raise RuntimeError("lgo_generate_rsa_aggregate failed")
    return x


def generate_velocities(seed, n, vmax):
    """Seeded velocity components uniform in [-vmax, vmax], bit-identical to lg_generate_velocities."""
    v = np.zeros((int(n), 3))
    if olib().lgo_generate_velocities(C.c_uint64(seed), int(n), float(vmax), _dp(v)) != 0:
        raise RuntimeError("lgo_generate_velocities failed")
    return v


def _facet_array(facets):
    if not facets:
        return None, None
    arr = (A.lg_facet_desc * len(facets))(*facets)
    return arr, C.cast(arr, C.POINTER(A.lg_facet_desc))


def _state(n, x0, v0, th0, om0):
    z = np.zeros((n, 3))
    cv = lambda a: np.ascontiguousarray(z if a is None else np.asarray(a, dtype=np.float64).reshape(n, 3))
    return cv(x0), cv(v0), cv(th0), cv(om0)


class OracleSystem:
    """The CPU oracle on one system (see lg_oracle.c for the loop it restates)."""

    def __init__(self, desc, x0, v0=None, th0=None, om0=None, facets=None, neck=None, threads=1):
        L = olib()
        self.n = int(desc.n_part)
        self.desc = desc
        x0, v0, th0, om0 = _state(self.n, x0, v0, th0, om0)
        self._facets, fp = _facet_array(facets)
        neck_a = None if neck is None else np.ascontiguousarray(neck, dtype=np.float64)
        self.h = L.lgo_create(C.byref(desc), _dp(x0), _dp(v0), _dp(th0), _dp(om0), fp,
                              None if neck_a is None else _dp(neck_a),
                              0 if neck_a is None else len(neck_a), int(threads))
        if not self.h:
            raise RuntimeError("lgo_create failed")

    def __del__(self):
        if getattr(self, "h", None):
            olib().lgo_destroy(self.h)
            self.h = None

    def step(self, dt, nsteps=1, rebuild_every=0):
        olib().lgo_step(self.h, dt, int(nsteps), int(rebuild_every))

    def update_neighbor_list(self):
        olib().lgo_update_neighbor_list(self.h)

    def get(self, field):
        out = np.empty((self.n, 3))
        olib().lgo_get(self.h, field, _dp(out))
        return out

    def set(self, field, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(self.n, 3)
        olib().lgo_set(self.h, field, _dp(a))

    def springs(self, i, j):
        out = np.zeros(9)
        olib().lgo_get_pair_springs(self.h, i, j, _dp(out))
        return out

    def bonds(self):
        L = olib()
        n = L.lgo_count_bonds(self.h, None, 0)
        arr = np.zeros(2 * max(n, 1), dtype=np.int64)
        L.lgo_count_bonds(self.h, arr.ctypes.data_as(C.POINTER(C.c_int64)), n)
        return arr[:2 * n].reshape(n, 2)

    def row(self, i):
        L = olib()
        m = L.lgo_row_length(self.h, i)
        out = np.zeros(max(m, 1), dtype=np.int32)
        L.lgo_row(self.h, i, out.ctypes.data_as(C.POINTER(C.c_int32)), m)
        return out[:m]

    def observables(self):
        o = A.lg_observables()
        olib().lgo_observables(self.h, C.byref(o))
        return o.as_dict()

    def facet_vertices(self, f):
        out = np.zeros(9)
        olib().lgo_facet_get_vertices(self.h, f, _dp(out))
        return out

    def facet_update_positions(self, f, dt):
        olib().lgo_facet_update_positions(self.h, f, dt)

    def set_hold_mask(self, mask):
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        olib().lgo_set_hold_mask(self.h, None if m is None else m.ctypes.data_as(C.POINTER(C.c_uint8)))

    def set_body_force(self, body):
        olib().lgo_set_body_force(self.h, None if body is None else C.byref(body))

    def set_body_centre(self, c):
        olib().lgo_set_body_centre(self.h, _dp(np.ascontiguousarray(c, dtype=np.float64)))

    def connectors(self):
        L = olib()
        k = L.lgo_get_connectors(self.h, None, 0)
        out = np.zeros((max(k, 1), 3))
        L.lgo_get_connectors(self.h, _dp(out), k)
        return out[:k]


def run_many(systems, dts, nsteps, rebuild):
    """Step several oracle systems concurrently (one thread each)."""
    k = len(systems)
    hs = (C.c_void_p * k)(*[s.h for s in systems])
    d = (C.c_double * k)(*dts)
    ns = (C.c_int64 * k)(*nsteps)
    rb = (C.c_int64 * k)(*rebuild)
    olib().lgo_run_many(hs, d, ns, rb, k)


class RefHarnessSystem:
    """libgran's own functors (compiled from its source tree) on the oracle's system loop."""

    def __init__(self, desc, x0, v0=None, th0=None, om0=None, facets=None, neck=None):
        L = rlib()
        if L is None:
            raise RuntimeError("reference harness unavailable (libgran source tree not present)")
        self.n = int(desc.n_part)
        x0, v0, th0, om0 = _state(self.n, x0, v0, th0, om0)
        self._facets, fp = _facet_array(facets)
        neck_a = None if neck is None else np.ascontiguousarray(neck, dtype=np.float64)
        self.h = L.lgref_create(C.byref(desc), _dp(x0), _dp(v0), _dp(th0), _dp(om0), fp,
                                None if neck_a is None else _dp(neck_a),
                                0 if neck_a is None else len(neck_a))
        if not self.h:
            raise RuntimeError("lgref_create failed")

    def __del__(self):
        if getattr(self, "h", None):
            rlib().lgref_destroy(self.h)
            self.h = None

    def step(self, dt, nsteps=1, rebuild_every=0):
        rlib().lgref_step(self.h, dt, int(nsteps), int(rebuild_every))

    def update_neighbor_list(self):
        rlib().lgref_update_neighbor_list(self.h)

    def get(self, field):
        out = np.empty((self.n, 3))
        rlib().lgref_get(self.h, field, _dp(out))
        return out

    def springs(self, i, j):
        out = np.zeros(9)
        rlib().lgref_pair_springs(self.h, i, j, _dp(out))
        return out

    def bonds(self):
        L = rlib()
        n = L.lgref_bonds(self.h, None, 0)
        arr = np.zeros(2 * max(n, 1), dtype=np.int64)
        L.lgref_bonds(self.h, arr.ctypes.data_as(C.POINTER(C.c_int64)), n)
        return arr[:2 * n].reshape(n, 2)

    def facet_vertices(self, f):
        out = np.zeros(9)
        rlib().lgref_facet_get_vertices(self.h, f, _dp(out))
        return out

    def set_body_centre(self, c):
        if rlib().lgref_set_body_centre(self.h, _dp(np.ascontiguousarray(c, dtype=np.float64))) != 0:
            raise RuntimeError("no central body force in this harness system")
