"""Body forces, unary hooks and held increments on the GPU (the custom unary force and custom step
handler patterns of libgran's tutorials), through the C ABI and the C++ drop-in headers.

FP64: bit-exact with the oracle (whose unary fold and held increments are pinned against libgran's
own unary container through the reference harness). Mixed precision: per-step forces within 1e-6
relative (normwise) of FP64 at identical states."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from libgran_gb300 import _abi as A
from libgran_gb300 import configs as K
from libgran_gb300.system import System, generate_aggregate, generate_velocities
from oracle import oracle as O

import helpers as H

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "libgran_gb300", "_lib")
INC = os.path.join(ROOT, "include", "libgran_gb300")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _state_file(path, x, v):
    with open(path, "wb") as f:
        f.write(np.int64(len(x)).tobytes())
        f.write(np.ascontiguousarray(x, dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(v, dtype=np.float64).tobytes())


def test_dropin_tutorial_driver_matches_golden(tmp_path):
    """libgran's custom step-handler tutorial composition (central_attraction_functor in the unary
    container, fixed_particle_step_handler over rotational_step_handler) on the drop-in headers
    reproduces the fixture made by libgran's own containers, bit for bit."""
    g = np.load(os.path.join(ROOT, "tests", "golden", "tutorial_central_fixed.npz"))
    exe = str(tmp_path / "dropin_tutorial")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I" + INC, "-I" + os.path.join(CUDA, "include"),
                           "-o", exe, os.path.join(ROOT, "tests", "cpp", "dropin_tutorial.cpp"), "-L" + LIB,
                           "-llg_gb300", "-Wl,-rpath," + LIB])
    sin, sout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    _state_file(sin, g["x0"], g["v0"])
    r = subprocess.run([exe, sin, sout, "400", "10"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = np.fromfile(sout, dtype=np.float64).reshape(4, -1, 3)
    for k, f in enumerate((A.LG_FIELD_X, A.LG_FIELD_V, A.LG_FIELD_THETA, A.LG_FIELD_OMEGA)):
        assert np.array_equal(out[k], g["f%d_s400" % f]), H.FIELD_NAMES[f]
    assert np.array_equal(out[1][10], g["v0"][10])  # the fixed particle kept its velocity


def test_device_functor_hook_matches_builtin_body_force(tmp_path):
    """A __device__ functor attached with libgran_gb300::device_unary gives the built-in central
    body force's bits, eagerly and from CUDA graphs."""
    exe = str(tmp_path / "device_unary_central")
    subprocess.check_call([os.path.join(CUDA, "bin", "nvcc"), "-gencode", "arch=compute_103a,code=sm_103a",
                           "-std=c++17", "-O2", "--fmad=false", "-I" + INC, "-I" + os.path.join(ROOT, "include"),
                           "-o", exe, os.path.join(ROOT, "tests", "cpp", "device_unary_central.cu"), "-L" + LIB,
                           "-llg_gb300", "-Xlinker", "-rpath=" + LIB])
    mat = K.Material()
    x0 = generate_aggregate(21, 80, mat.r)
    sin = str(tmp_path / "in.bin")
    _state_file(sin, x0, generate_velocities(21, 80, 0.3))
    r = subprocess.run([exe, sin], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "IDENTICAL" in r.stdout, r.stdout + r.stderr


def _body_hold_desc(mat, n, x0, kernel, precision=A.LG_PRECISION_FP64):
    d = K.make_desc(n, A.LG_BINARY_CONTACT, A.LG_HAMAKER_LIMITED, contact=mat.contact(), hamaker=mat.hamaker(),
                    pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r, precision=precision, force_kernel=kernel)
    d.body = K.central_body(3.0e-6, mat.m, x0.mean(0))
    rng = np.random.default_rng(5)
    hold = np.zeros(n, dtype=np.uint8)
    pick = rng.choice(n, size=n // 10, replace=False)
    hold[pick] = rng.integers(1, 16, size=len(pick)).astype(np.uint8)
    K.set_hold(d, hold)
    return d, hold


@pytest.mark.parametrize("kernel", [A.LG_FORCE_KERNEL_ROWGROUP, A.LG_FORCE_KERNEL_COMPACT, A.LG_FORCE_KERNEL_PAIRS],
                         ids=["rowgroup1", "compact", "pairs"])
def test_body_force_and_hold_bit_exact_verlet(kernel):
    mat = K.Material()
    n = 600
    x0 = generate_aggregate(31, n, mat.r)
    v0 = generate_velocities(31, n, 0.5) + 1.0e7 * (x0 - x0.mean(0))
    d, hold = _body_hold_desc(mat, n, x0, kernel)
    d.threads_per_row = 1
    s = System(d, x0, v0)
    o = O.OracleSystem(d, x0, v0, threads=4)
    for nst in (1, 19, 40):
        s.step(mat.dt, nst, 20)
        o.step(mat.dt, nst, 20)
        for f in H.FIELDS:
            assert np.array_equal(s.get(f), o.get(f)), "%s after %d steps" % (H.FIELD_NAMES[f], nst)
    # the tutorial's per-step centre update and a new mask, between calls
    c = o.get(A.LG_FIELD_X).mean(0) + np.array([1.0, -2.0, 0.5]) * mat.r
    s.set_body_centre(c)
    o.set_body_centre(c)
    hold2 = np.roll(hold, 7)
    s.set_hold_mask(hold2)
    o.set_hold_mask(hold2)
    s.step(mat.dt, 40, 20)
    o.step(mat.dt, 40, 20)
    for f in H.FIELDS:
        assert np.array_equal(s.get(f), o.get(f)), H.FIELD_NAMES[f]
    held = (hold2 & A.LG_HOLD_X) > 0
    before = o.get(A.LG_FIELD_X)[held]
    s.step(mat.dt, 20, 20)
    assert np.array_equal(s.get(A.LG_FIELD_X)[held], before)
    assert s.device_errors() == 0


def test_batch_body_centres_per_system():
    mat = K.Material()
    sizes = [50, 90, 40]
    xs = [generate_aggregate(40 + q, n, mat.r) + q * 30 * mat.r for q, n in enumerate(sizes)]
    vs = [generate_velocities(40 + q, n, 0.3) for q, n in enumerate(sizes)]
    centres = np.array([x.mean(0) + np.array([0.0, 0.0, 2.0 * mat.r]) for x in xs])

    def desc(n):
        d = K.make_desc(n, A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, contact=mat.contact(), sinter=mat.sinter(),
                        hamaker=mat.hamaker(), pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r,
                        force_kernel=A.LG_FORCE_KERNEL_COMPACT)
        d.body = K.central_body(5.0e-6, mat.m, (0.0, 0.0, 0.0))
        return d

    b = System(desc(sum(sizes)), np.concatenate(xs), np.concatenate(vs), sizes=sizes)
    b.set_body_centre(centres)
    b.step(mat.dt, 60, 20)
    off = np.concatenate([[0], np.cumsum(sizes)])
    for q, n in enumerate(sizes):
        a = System(desc(n), xs[q], vs[q])
        a.set_body_centre(centres[q])
        a.step(mat.dt, 60, 20)
        for f in H.FIELDS:
            assert np.array_equal(a.get(f), b.get(f)[off[q]:off[q + 1]]), (q, H.FIELD_NAMES[f])


def test_mixed_body_force_and_hold_within_tolerance():
    mat = K.Material()
    n = 3000
    x0 = generate_aggregate(51, n, mat.r)
    # compressed by 0.2 %: the RSA monomers touch at 2r to within rounding, where "in contact" is a
    # rounding coin flip that FP64 and float-float separations settle differently
    x0 = x0.mean(0) + 0.998 * (x0 - x0.mean(0))
    v0 = generate_velocities(51, n, 0.5)
    d64, hold = _body_hold_desc(mat, n, x0, A.LG_FORCE_KERNEL_COMPACT)
    dmx, _ = _body_hold_desc(mat, n, x0, A.LG_FORCE_KERNEL_COMPACT, A.LG_PRECISION_MIXED)
    s64, smx = System(d64, x0, v0), System(dmx, x0, v0)
    for f in (A.LG_FIELD_A, A.LG_FIELD_ALPHA):
        assert H.rel_err(smx.get(f), s64.get(f)) <= 1e-6
    s64.step(mat.dt, 40, 20)
    smx.step(mat.dt, 40, 20)
    held_v = (hold & A.LG_HOLD_V) > 0
    assert np.array_equal(smx.get(A.LG_FIELD_V)[held_v], v0[held_v])
    held_x = (hold & A.LG_HOLD_X) > 0
    assert np.array_equal(smx.get(A.LG_FIELD_X)[held_x], x0[held_x])
    assert H.rel_err(smx.get(A.LG_FIELD_X) - x0, s64.get(A.LG_FIELD_X) - x0) <= 1e-4


def _cudart():
    for name in (os.path.join(CUDA, "lib64", "libcudart.so"), "libcudart.so"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    pytest.skip("libcudart not loadable")


def test_python_unary_hook_zero_terms_and_failure():
    """A hook written in Python (ctypes) that clears the unary terms on the engine's stream leaves
    the trajectory of a system without unary terms; a hook that reports failure fails the step."""
    rt = _cudart()
    rt.cudaMemsetAsync.argtypes = [C.c_void_p, C.c_int, C.c_size_t, C.c_void_p]
    calls = []

    @A.lg_unary_hook
    def zero_hook(args, user):
        a = args.contents
        calls.append(a.n)
        for p in (a.a_out, a.alpha_out):
            if rt.cudaMemsetAsync(p, 0, 32 * a.n, a.stream) != 0:
                return 1
        return 0

    @A.lg_unary_hook
    def failing_hook(args, user):
        return 7

    mat = K.Material()
    n = 120
    x0 = generate_aggregate(61, n, mat.r)
    v0 = generate_velocities(61, n, 0.3)
    d0 = K.make_desc(n, A.LG_BINARY_CONTACT, A.LG_HAMAKER_LIMITED, contact=mat.contact(), hamaker=mat.hamaker())
    dh = K.make_desc(n, A.LG_BINARY_CONTACT, A.LG_HAMAKER_LIMITED, contact=mat.contact(), hamaker=mat.hamaker())
    dh.unary_hook = zero_hook
    plain, hooked = System(d0, x0, v0), System(dh, x0, v0)
    plain.step(mat.dt, 50)
    hooked.step(mat.dt, 50)
    assert calls, "the hook was not called"
    for f in H.FIELDS:
        assert np.array_equal(plain.get(f), hooked.get(f)), H.FIELD_NAMES[f]
    A.check(A.lib().lg_set_unary_hook(hooked.h, failing_hook, None), "lg_set_unary_hook")
    with pytest.raises(RuntimeError, match="unary hook returned 7"):
        hooked.step(mat.dt, 1)
    with pytest.raises(RuntimeError, match="exclude each other"):
        dx = K.make_desc(n, A.LG_BINARY_CONTACT, A.LG_HAMAKER_NONE, contact=mat.contact())
        dx.unary_hook = zero_hook
        dx.body = K.central_body(1e-6, mat.m, (0.0, 0.0, 0.0))
        System(dx, x0, v0)
    with pytest.raises(RuntimeError, match="no central body force"):
        plain.set_body_centre((0.0, 0.0, 0.0))
