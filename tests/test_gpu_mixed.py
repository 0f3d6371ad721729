"""Mixed-precision path (FP32 pair arithmetic; FP64 separation, overlap, springs, sums and
integration) against the FP64 path at identical states. Tolerance: per-step forces and torques
within 1e-6 relative (normwise over the system)."""
import numpy as np
import pytest

from libgran_gb300 import _abi as A
from libgran_gb300 import configs as K
from libgran_gb300.system import System, generate_aggregate, generate_velocities

import helpers as H

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6
STATE_FIELDS = (A.LG_FIELD_X, A.LG_FIELD_V, A.LG_FIELD_THETA, A.LG_FIELD_OMEGA)


def _desc(n, bm, hm, pairs, precision, mat, kernel=A.LG_FORCE_KERNEL_AUTO):
    return K.make_desc(n, bm, hm, contact=mat.contact(), sinter=mat.sinter(), hamaker=mat.hamaker(), pairs=pairs,
                       r_verlet=4.5 * mat.r if pairs == A.LG_PAIRS_VERLET else 0.0, precision=precision,
                       force_kernel=kernel)


@pytest.mark.parametrize("kernel", [A.LG_FORCE_KERNEL_ROWGROUP, A.LG_FORCE_KERNEL_COMPACT], ids=["rowgroup", "compact"])
@pytest.mark.parametrize("pairs,n", [(A.LG_PAIRS_ALL, 300), (A.LG_PAIRS_VERLET, 4000)])
@pytest.mark.parametrize("bm,hm", [(A.LG_BINARY_CONTACT, A.LG_HAMAKER_LIMITED), (A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED),
                                   (A.LG_BINARY_CONTACT, A.LG_HAMAKER_FULL), (A.LG_BINARY_SINTER, A.LG_HAMAKER_NONE)])
def test_mixed_forces_within_1e6_of_fp64(pairs, n, bm, hm, kernel):
    mat = K.Material()
    x0 = generate_aggregate(77, n, mat.r)
    v0 = generate_velocities(77, n, 0.1) - 2e7 * (x0 - x0.mean(0))
    ref = System(_desc(n, bm, hm, pairs, A.LG_PRECISION_FP64, mat), x0, v0)
    ref.step(mat.dt, 100, 20)  # develop overlaps, springs and contacts
    state = [ref.get(f) for f in STATE_FIELDS]
    a64 = System(_desc(n, bm, hm, pairs, A.LG_PRECISION_FP64, mat), *state)
    amx = System(_desc(n, bm, hm, pairs, A.LG_PRECISION_MIXED, mat, kernel), *state)
    assert H.rel_err(amx.get(A.LG_FIELD_A), a64.get(A.LG_FIELD_A)) <= MIXED_TOL
    assert H.rel_err(amx.get(A.LG_FIELD_ALPHA), a64.get(A.LG_FIELD_ALPHA)) <= MIXED_TOL
    # both continue from the same state; the 1e-7-level per-step differences are amplified by the
    # stiff, history-dependent contacts, so trajectories are compared loosely and then re-synced
    for _ in range(3):
        a64.step(mat.dt, 10, 20)
        amx.step(mat.dt, 10, 20)
        assert H.rel_err(amx.get(A.LG_FIELD_A), a64.get(A.LG_FIELD_A)) <= 1e-2
    assert H.rel_err(amx.get(A.LG_FIELD_X) - state[0], a64.get(A.LG_FIELD_X) - state[0]) <= 1e-4
    assert amx.device_errors() == 0


@pytest.mark.parametrize("kernel", [A.LG_FORCE_KERNEL_ROWGROUP, A.LG_FORCE_KERNEL_COMPACT], ids=["rowgroup", "compact"])
@pytest.mark.parametrize("bm", [A.LG_BINARY_CONTACT, A.LG_BINARY_SINTER], ids=["contact", "sinter"])
def test_mixed_forces_at_the_contact_threshold(bm, kernel):
    """A freshly generated aggregate holds thousands of monomer pairs at the contact distance to
    within rounding (unbonded for the contact model, beside the bonds for the sinter model): whether
    such a pair touches, and so feels damping and friction, is decided by the last bits of its
    separation. The mixed path lets the FP64 overlap decide those pairs, so its forces stay within
    1e-6 of the FP64 path's at the generated state (32768 monomers, velocities +-0.1 m/s)."""
    mat = K.Material()
    n = 32768
    x0 = generate_aggregate(1 << 32, n, mat.r)
    v0 = generate_velocities(1 << 32, n, 0.1)
    a64 = System(_desc(n, bm, A.LG_HAMAKER_LIMITED, A.LG_PAIRS_VERLET, A.LG_PRECISION_FP64, mat), x0, v0)
    amx = System(_desc(n, bm, A.LG_HAMAKER_LIMITED, A.LG_PAIRS_VERLET, A.LG_PRECISION_MIXED, mat, kernel), x0, v0)
    assert H.rel_err(amx.get(A.LG_FIELD_A), a64.get(A.LG_FIELD_A)) <= MIXED_TOL
    assert H.rel_err(amx.get(A.LG_FIELD_ALPHA), a64.get(A.LG_FIELD_ALPHA)) <= MIXED_TOL
    assert a64.observables()["n_contacts"] == amx.observables()["n_contacts"]


def test_mixed_energy_drift_tracks_fp64():
    """Energy balance over 2000 steps: total energy (kinetic + spring + Hamaker potential) of the
    mixed path follows the FP64 path."""
    mat = K.Material()
    n = 2000
    x0 = generate_aggregate(5, n, mat.r)
    v0 = generate_velocities(5, n, 0.1)
    runs = {}
    for prec in (A.LG_PRECISION_FP64, A.LG_PRECISION_MIXED):
        s = System(_desc(n, A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, A.LG_PAIRS_VERLET, prec, mat), x0, v0)
        e = []
        for _ in range(10):
            s.step(mat.dt, 200, 20)
            o = s.observables()
            e.append(o["ke_total"] + o["potential_energy"])
        runs[prec] = np.array(e)
    e64, emx = runs[A.LG_PRECISION_FP64], runs[A.LG_PRECISION_MIXED]
    scale = np.abs(e64).max()
    assert np.abs(emx - e64).max() <= 2e-3 * scale


def test_mixed_breaking_bonds_match_fp64_count():
    mat = K.Material()
    n = 600
    x0 = generate_aggregate(8, n, mat.r)
    v0 = -4e7 * (x0 - x0.mean(0))
    res = {}
    for prec in (A.LG_PRECISION_FP64, A.LG_PRECISION_MIXED):
        d = _desc(n, A.LG_BINARY_BREAKING_SINTER, A.LG_HAMAKER_LIMITED, A.LG_PAIRS_ALL, prec, mat)
        probe = System(d, x0, v0)
        nb = len(probe.bonds()) // 2
        s = System(d, x0, v0, neck=np.full(nb, 1e-8))
        s.step(mat.dt, 300)
        res[prec] = len(s.bonds())
    assert abs(res[A.LG_PRECISION_MIXED] - res[A.LG_PRECISION_FP64]) <= max(2, 0.01 * res[A.LG_PRECISION_FP64])


@pytest.mark.parametrize("shift_r", [0.5, 1e4], ids=["nearby", "far"])
def test_mixed_set_positions_translation(shift_r):
    """lg_set of translated positions: a small shift keeps the float-float origins (and captured
    graphs), a large one re-derives them; either way the translated system follows the original
    (the physics is translation invariant) to FP64 rounding of the shifted coordinates."""
    mat = K.Material()
    n = 3000
    x0 = generate_aggregate(21, n, mat.r)
    v0 = generate_velocities(21, n, 0.1)
    d = _desc(n, A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, A.LG_PAIRS_VERLET, A.LG_PRECISION_MIXED, mat,
              A.LG_FORCE_KERNEL_COMPACT)
    a = System(d, x0, v0)
    b = System(d, x0, v0)
    a.step(mat.dt, 40, 20)
    b.step(mat.dt, 40, 20)  # graphs captured for both
    shift = np.array([shift_r, -0.5 * shift_r, 0.25 * shift_r]) * mat.r
    b.set(A.LG_FIELD_X, b.get(A.LG_FIELD_X) + shift)
    b.update_neighbor_list()
    a.update_neighbor_list()
    a.step(mat.dt, 40, 20)
    b.step(mat.dt, 40, 20)
    dx = (b.get(A.LG_FIELD_X) - shift) - a.get(A.LG_FIELD_X)
    assert np.abs(dx).max() <= 1e-6 * mat.r
    assert H.rel_err(b.get(A.LG_FIELD_A), a.get(A.LG_FIELD_A)) <= 1e-4
    assert a.device_errors() == 0 and b.device_errors() == 0


def test_mixed_runs_of_steps_track_single_steps():
    """Inside a run of steps the mixed completion kernel integrates in float-float (the FP64 state is
    brought up to date by the run's last step); one step per call keeps the FP64 integration. The
    pair terms are FP32 arithmetic on the high parts of the state, so states that differ by rounding
    can give pair terms that differ by an FP32 rounding (1e-7 of a term): after two steps the two
    agree to that; over 20 steps of a bonded aggregate the difference grows with the dynamics'
    sensitivity (about tenfold every ten steps), as any perturbation does. The integrator itself is
    checked exactly in free flight (next test). The 20-step bound on velocities and spins (3e-5)
    also covers the pairs of the generated aggregate that sit at the contact distance to within
    rounding: single steps let the FP64 overlap decide whether they touch (FP64 positions are
    current), steps inside a run decide it in float-float, and at that distance either decision is
    a rounding accident whose consequence grows with the dynamics like any other."""
    mat = K.Material()
    n = 2500
    x0 = generate_aggregate(31, n, mat.r)
    v0 = generate_velocities(31, n, 0.1)
    d = _desc(n, A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, A.LG_PAIRS_VERLET, A.LG_PRECISION_MIXED, mat,
              A.LG_FORCE_KERNEL_COMPACT)
    for nst, tol_x, tol_v, tol_a in ((2, 1e-10, 1e-8, 1e-6), (20, 1e-8, 3e-5, 1e-4)):
        a, b, c = System(d, x0, v0), System(d, x0, v0), System(d, x0, v0)
        a.step(mat.dt, nst, 20)
        for _ in range(nst):
            b.step(mat.dt, 1, 20)
            c.step(mat.dt, 1, 20)
        for f in STATE_FIELDS + (A.LG_FIELD_A, A.LG_FIELD_ALPHA):  # single steps are deterministic
            assert np.array_equal(b.get(f), c.get(f)), f
        assert H.rel_err(a.get(A.LG_FIELD_X) - x0, b.get(A.LG_FIELD_X) - x0) <= tol_x
        for f in (A.LG_FIELD_V, A.LG_FIELD_OMEGA, A.LG_FIELD_THETA):
            assert H.rel_err(a.get(f), b.get(f)) <= tol_v, (nst, f)
        for f in (A.LG_FIELD_A, A.LG_FIELD_ALPHA):
            assert H.rel_err(a.get(f), b.get(f)) <= tol_a, (nst, f)
        assert a.device_errors() == 0


def test_mixed_run_free_flight_is_exact():
    """Free flight (no contacts, no Hamaker force) through a run of float-float steps: positions
    follow x0 + v0 t and rotations omega0 t to better than the FP64 step-by-step integration (the
    run's displacement accumulates from zero and joins the FP64 position once)."""
    mat = K.Material()
    n = 2000
    x0 = generate_aggregate(31, n, mat.r) * 3.0
    v0 = generate_velocities(31, n, 0.1)
    om0 = generate_velocities(32, n, 1e8)
    d = _desc(n, A.LG_BINARY_CONTACT, A.LG_HAMAKER_LIMITED, A.LG_PAIRS_VERLET, A.LG_PRECISION_MIXED, mat,
              A.LG_FORCE_KERNEL_COMPACT)
    d.hamaker.A = 0.0
    s = System(d, x0, v0, om0=om0)
    s.step(mat.dt, 60, 20)
    t = 60 * mat.dt
    assert H.rel_err(s.get(A.LG_FIELD_X) - x0, v0 * t) <= 2e-8
    assert H.rel_err(s.get(A.LG_FIELD_V), v0) <= 4e-15  # the float-float round trip: 2^-49
    assert H.rel_err(s.get(A.LG_FIELD_THETA), om0 * t) <= 1e-13
    assert H.rel_err(s.get(A.LG_FIELD_OMEGA), om0) <= 4e-15


def test_mixed_runs_with_held_particles():
    """Held increments inside runs of float-float steps: held particles keep the FP64 path, so a
    held velocity or position stays exactly as it was."""
    mat = K.Material()
    n = 2000
    x0 = generate_aggregate(32, n, mat.r)
    v0 = generate_velocities(32, n, 0.3)
    hold = np.zeros(n, dtype=np.uint8)
    hold[::7] = A.LG_HOLD_V
    hold[3::7] = A.LG_HOLD_X | A.LG_HOLD_THETA
    descs = []
    for prec in (A.LG_PRECISION_FP64, A.LG_PRECISION_MIXED):
        d = _desc(n, A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, A.LG_PAIRS_VERLET, prec, mat, A.LG_FORCE_KERNEL_COMPACT)
        K.set_hold(d, hold)
        descs.append(d)
    s64, smx = System(descs[0], x0, v0), System(descs[1], x0, v0)
    s64.step(mat.dt, 80, 20)
    smx.step(mat.dt, 80, 20)
    hv, hx = hold == A.LG_HOLD_V, (hold & A.LG_HOLD_X) > 0
    assert np.array_equal(smx.get(A.LG_FIELD_V)[hv], v0[hv])
    assert np.array_equal(smx.get(A.LG_FIELD_X)[hx], x0[hx])
    assert np.array_equal(smx.get(A.LG_FIELD_THETA)[hx], np.zeros((hx.sum(), 3)))
    assert H.rel_err(smx.get(A.LG_FIELD_X) - x0, s64.get(A.LG_FIELD_X) - x0) <= 1e-4
    assert smx.device_errors() == 0


@pytest.mark.parametrize("precision", [A.LG_PRECISION_FP64, A.LG_PRECISION_MIXED], ids=["fp64", "mixed"])
def test_state_calls_match_field_calls(precision):
    """lg_set_state / lg_get_state move the same numbers as four lg_set / lg_get calls, skip the
    fields given as NULL, and leave the system stepping as after the per-field calls."""
    mat = K.Material()
    n = 1500
    x0 = generate_aggregate(41, n, mat.r)
    v0 = generate_velocities(41, n, 0.1)
    d = _desc(n, A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, A.LG_PAIRS_VERLET, precision, mat)
    a = System(d, x0, v0)
    b = System(d, x0, v0)
    a.step(mat.dt, 30, 20)
    st = a.get_state()
    for f, arr in zip(STATE_FIELDS, st):
        assert np.array_equal(arr, a.get(f))
    rng = np.random.default_rng(3)
    th = rng.normal(size=(n, 3))
    b.set_state(st[0], st[1], th, st[3])
    b.set_state(theta=st[2])  # only theta; the others stay
    for f, arr in zip(STATE_FIELDS, b.get_state()):
        assert np.array_equal(arr, a.get(f))
    c = System(d, x0, v0)
    for f, arr in zip(STATE_FIELDS, st):
        c.set(f, arr)
    b.update_neighbor_list()
    c.update_neighbor_list()
    b.step(mat.dt, 20, 20)
    c.step(mat.dt, 20, 20)
    for f in STATE_FIELDS:
        assert np.array_equal(b.get(f), c.get(f)), f


@pytest.mark.parametrize("precision", [A.LG_PRECISION_FP64, A.LG_PRECISION_MIXED], ids=["fp64", "mixed"])
def test_state_calls_pinned_and_pageable_agree(precision):
    """Pinned host buffers are read and written by the GPU directly, pageable ones are staged; both
    move the same numbers, and a system set from either steps identically."""
    import torch
    mat = K.Material()
    n = 3000
    x0 = generate_aggregate(41, n, mat.r)
    v0 = generate_velocities(41, n, 0.2)
    d = _desc(n, A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, A.LG_PAIRS_VERLET, precision, mat,
              A.LG_FORCE_KERNEL_COMPACT)
    a, b = System(d, x0, v0), System(d, x0, v0)
    a.step(mat.dt, 30, 20)
    b.step(mat.dt, 30, 20)
    pinned = [torch.empty((n, 3), dtype=torch.float64).pin_memory() for _ in range(4)]
    a.get_state(out=tuple(p.numpy() for p in pinned))
    pageable = a.get_state()
    for p, q in zip(pinned, pageable):
        assert np.array_equal(p.numpy(), q)
    shifted = [p.numpy() + 0.0 for p in pinned]
    shifted[0] += 3.0 * mat.r
    for p, q in zip(pinned, shifted):
        p.numpy()[:] = q
    a.set_state(*(p.numpy() for p in pinned))
    b.set_state(*shifted)
    for f, q in zip(STATE_FIELDS, shifted):
        assert np.array_equal(a.get(f), q) and np.array_equal(b.get(f), q)
    a.step(mat.dt, 25, 20)
    b.step(mat.dt, 25, 20)
    for f in STATE_FIELDS + (A.LG_FIELD_A, A.LG_FIELD_ALPHA):
        assert np.array_equal(a.get(f), b.get(f)), f


@pytest.mark.parametrize("n", [1, 45, 129, 1001])
def test_state_transfer_tails_and_alignment(n):
    """lg_set_state / lg_get_state with particle counts that leave a partial block and an odd number
    of doubles in the last tile, and with caller buffers that start 8 bytes past a 16-byte boundary
    (the 8-byte path), pinned and pageable: the same numbers as the per-field calls."""
    import torch
    mat = K.Material()
    x0 = generate_aggregate(5 + n, n, mat.r)
    v0 = generate_velocities(5 + n, n, 0.1)
    d = _desc(n, A.LG_BINARY_CONTACT, A.LG_HAMAKER_LIMITED, A.LG_PAIRS_VERLET, A.LG_PRECISION_MIXED, mat)
    s = System(d, x0, v0)
    s.step(mat.dt, 7, 20)
    ref = [s.get(f) for f in STATE_FIELDS]
    rng = np.random.default_rng(n)
    new = [r + rng.normal(scale=1e-12, size=r.shape) for r in ref]

    def buffers(kind, shift):
        out = []
        for _ in range(4):
            if kind == "pinned":
                flat = torch.empty(3 * n + 1, dtype=torch.float64).pin_memory().numpy()
            else:
                flat = np.empty(3 * n + 1)
            base = flat.__array_interface__["data"][0]
            off = (shift - base % 16) % 16 // 8  # doubles to skip so that the start is base + shift mod 16
            out.append(flat[off:off + 3 * n].reshape(n, 3))
        return out

    for kind in ("pinned", "pageable"):
        for shift in (0, 8):
            bufs = buffers(kind, shift)
            assert all(b.__array_interface__["data"][0] % 16 == shift for b in bufs)
            s.get_state(out=tuple(bufs))
            for b, r in zip(bufs, ref):
                assert np.array_equal(b, r)
            for b, v in zip(bufs, new):
                b[...] = v
            s.set_state(*bufs)
            for f, v in zip(STATE_FIELDS, new):
                assert np.array_equal(s.get(f), v)
            for f, r in zip(STATE_FIELDS, ref):  # back to the reference state for the next round
                s.set(f, r)
    assert s.device_errors() == 0
