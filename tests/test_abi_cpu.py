"""The C-ABI library: loads without a GPU, exports every declared entry point, rejects bad input."""
import ctypes as C
import os
import re

import numpy as np

from libgran_gb300 import _abi as A
from libgran_gb300 import configs as K
from libgran_gb300.system import generate_aggregate, generate_velocities

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(lg_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    L = A.lib()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_version_and_device_count():
    L = A.lib()
    assert b"sm_103a" in L.lg_version()
    c = C.c_int(-1)
    assert L.lg_device_count(C.byref(c)) == A.LG_OK
    assert c.value >= 0


def _create(desc, n):
    x = np.zeros((n, 3))
    h = C.c_void_p()
    p = x.ctypes.data_as(C.POINTER(C.c_double))
    return A.lib().lg_create(C.byref(desc), p, p, p, p, None, None, 0, 0, C.byref(h)), h


def test_create_rejects_bad_descriptors_before_touching_a_gpu():
    mat = K.Material()
    bad = [
        K.make_desc(0, A.LG_BINARY_CONTACT, contact=mat.contact()),
        K.make_desc(4, 9, contact=mat.contact()),
        K.make_desc(4, A.LG_BINARY_NONE, A.LG_HAMAKER_NONE),
        K.make_desc(4, A.LG_BINARY_CONTACT, contact=mat.contact(), pairs=A.LG_PAIRS_VERLET, r_verlet=0.0),
        K.make_desc(10000, A.LG_BINARY_CONTACT, contact=mat.contact(), pairs=A.LG_PAIRS_ALL),
        K.make_desc(4, A.LG_BINARY_CONTACT, contact=mat.contact(), n_facets=9),
        K.make_desc(4, A.LG_BINARY_CONTACT, contact=mat.contact(), precision=A.LG_PRECISION_MIXED,
                    force_kernel=A.LG_FORCE_KERNEL_PAIRS),
        K.make_desc(4, A.LG_BINARY_CONTACT, contact=mat.contact(), force_kernel=A.LG_FORCE_KERNEL_PERSISTENT),
        K.make_desc(4, A.LG_BINARY_CONTACT, contact=mat.contact(), precision=A.LG_PRECISION_MIXED,
                    force_kernel=A.LG_FORCE_KERNEL_FP64_FAST),
        K.make_desc(4, A.LG_BINARY_CONTACT, contact=mat.contact(), force_kernel=6),
    ]
    d = K.make_desc(4, A.LG_BINARY_CONTACT, contact=mat.contact())
    K.set_hold(d, np.array([0, 16, 0, 0], dtype=np.uint8))  # unknown bit
    bad.append(d)
    for body in (K.central_body(1e-6, 0.0, (0.0, 0.0, 0.0)), K.central_body(1e-6, 1e-20, (np.inf, 0.0, 0.0)),
                 A.lg_body_force(7, 1e-6, 1e-20, (C.c_double * 3)())):
        d = K.make_desc(4, A.LG_BINARY_CONTACT, contact=mat.contact())
        d.body = body
        bad.append(d)
    hook = A.lg_unary_hook(lambda args, user: 0)
    d = K.make_desc(4, A.LG_BINARY_CONTACT, contact=mat.contact())
    d.body = K.central_body(1e-6, 1e-20, (0.0, 0.0, 0.0))
    d.unary_hook = hook
    bad.append(d)
    for d in bad:
        rc, h = _create(d, max(int(d.n_part), 1))
        assert rc == A.LG_E_INVALID
        assert not h.value
        assert len(A.lib().lg_last_error()) > 0


def test_generator_is_seeded_and_overlap_free():
    r = 1.4e-8
    a = generate_aggregate(3, 400, r)
    b = generate_aggregate(3, 400, r)
    c = generate_aggregate(4, 400, r)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, c)
    d = np.sqrt(((a[:, None] - a[None]) ** 2).sum(-1))
    np.fill_diagonal(d, np.inf)
    assert d.min() > 2 * r * (1 - 1e-9)
    # every sphere after the first touches at least one earlier sphere
    for k in range(1, 400):
        assert np.isclose(d[k, :k].min(), 2 * r, rtol=1e-12)
    v = generate_velocities(3, 400, 0.1)
    assert np.abs(v).max() <= 0.1 and v.std() > 0.03


def test_oracle_generator_gives_the_engine_generators_bits():
    """The reference arm of bench.py builds its inputs with the oracle's generator (so that it loads
    no engine library); it must produce the engine's aggregate and velocities bit for bit."""
    from oracle import oracle as O
    r = 1.4e-8
    for seed, n in ((1 << 32, 32768), (7, 64), ((2 << 32) + 5, 2048), (3, 1)):
        assert np.array_equal(O.generate_aggregate(seed, n, r), generate_aggregate(seed, n, r)), (seed, n)
        assert np.array_equal(O.generate_velocities(seed, n, 0.1), generate_velocities(seed, n, 0.1)), (seed, n)


def test_noalloc_refuses_bad_arguments_before_any_cuda_call():
    """lg_observables_noalloc checks its arguments before it touches a device: sizes beyond its
    fixed scratch, n = 0 and null pointers are refused with LG_E_INVALID and a message."""
    L = A.lib()
    rc = L.lg_observables_noalloc(1, 1, 1, A.LG_NOALLOC_MAX_PARTICLES + 1, 1.0, 1.0, 1, None)
    assert rc == A.LG_E_INVALID
    assert b"outside" in L.lg_last_error()
    assert L.lg_observables_noalloc(1, 1, 1, 0, 1.0, 1.0, 1, None) == A.LG_E_INVALID
    assert L.lg_observables_noalloc(None, 1, 1, 10, 1.0, 1.0, 1, None) == A.LG_E_INVALID
    assert L.lg_observables_noalloc(1, 1, 1, 10, 1.0, 1.0, None, None) == A.LG_E_INVALID
    assert b"null" in L.lg_last_error()


def test_autotune_cache_round_trip(tmp_path):
    """The autotuner's cache on the host: entries loaded from a file are found for descriptors of
    the same precision, pair mode, functor set, log2 size and batch flag (and only for those), saved
    entries read back identically, and a malformed file is refused without changing the cache."""
    L = A.lib()
    mat = K.Material()
    assert L.lg_autotune_cache_clear() == A.LG_OK
    d = K.make_desc(32768, A.LG_BINARY_CONTACT, A.LG_HAMAKER_LIMITED, contact=mat.contact(), hamaker=mat.hamaker(),
                    pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r, precision=A.LG_PRECISION_MIXED)
    t = A.lg_tuning()
    assert L.lg_autotune_cache_lookup(C.byref(d), 32768, 0, C.byref(t)) == A.LG_E_STATE
    f = tmp_path / "tune.txt"
    # precision pairs binary hamaker log2n batch : kernel T min_blocks slices assign ms_per_step
    f.write_text("# a comment\n%d %d %d %d 15 0 : 4 1 5 2 0 0.0405\n%d %d %d %d 15 1 : 2 1 4 4 0 0.5\n"
                 % (A.LG_PRECISION_MIXED, A.LG_PAIRS_VERLET, A.LG_BINARY_CONTACT, A.LG_HAMAKER_LIMITED,
                    A.LG_PRECISION_MIXED, A.LG_PAIRS_VERLET, A.LG_BINARY_CONTACT, A.LG_HAMAKER_LIMITED))
    assert L.lg_autotune_cache_load(str(f).encode()) == A.LG_OK
    for n in (32768, 40000, 65535):  # same power-of-two bucket
        assert L.lg_autotune_cache_lookup(C.byref(d), n, 0, C.byref(t)) == A.LG_OK
        assert t.as_dict() == {"force_kernel": A.LG_FORCE_KERNEL_PERSISTENT, "threads_per_row": 1,
                               "step_min_blocks": 5, "step_slices": 2, "step_assign": 0, "ms_per_step": 0.0405}
    assert L.lg_autotune_cache_lookup(C.byref(d), 32768, 1, C.byref(t)) == A.LG_OK
    assert t.force_kernel == A.LG_FORCE_KERNEL_COMPACT and t.step_slices == 4
    assert L.lg_autotune_cache_lookup(C.byref(d), 16384, 0, C.byref(t)) == A.LG_E_STATE
    d64 = K.make_desc(32768, A.LG_BINARY_CONTACT, A.LG_HAMAKER_LIMITED, contact=mat.contact(), hamaker=mat.hamaker(),
                      pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r)
    assert L.lg_autotune_cache_lookup(C.byref(d64), 32768, 0, C.byref(t)) == A.LG_E_STATE
    g = tmp_path / "saved.txt"
    assert L.lg_autotune_cache_save(str(g).encode()) == A.LG_OK
    assert L.lg_autotune_cache_clear() == A.LG_OK
    assert L.lg_autotune_cache_lookup(C.byref(d), 32768, 0, C.byref(t)) == A.LG_E_STATE
    assert L.lg_autotune_cache_load(str(g).encode()) == A.LG_OK
    assert L.lg_autotune_cache_lookup(C.byref(d), 32768, 0, C.byref(t)) == A.LG_OK and t.step_min_blocks == 5
    bad = tmp_path / "bad.txt"
    bad.write_text("1 1 1 2 15 0 : 9 1 4 1 0 1.0\n")
    assert L.lg_autotune_cache_load(str(bad).encode()) == A.LG_E_INVALID
    assert L.lg_autotune_cache_lookup(C.byref(d), 32768, 0, C.byref(t)) == A.LG_OK and t.step_min_blocks == 5
    assert L.lg_autotune_cache_clear() == A.LG_OK
