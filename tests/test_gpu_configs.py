"""The benchmark configurations at their own sizes, GPU (through the C ABI) against the oracle.

  C0  256 monomers (seed 0), sintered bonds + Luding contact + full Hamaker, all pairs,
      velocities +-0.1 m/s, 10^4 velocity-Verlet steps (alt_sinter_bridge.h:92-129 with
      hamaker_force.h:28-43, driven as main.cpp:147-161 drives them).
  C1  32768 monomers (seed 2^32), contact + limited Hamaker, Verlet rows of 4.5 r rebuilt every 20
      steps with spring carry (test/hamaker_neighbor.cpp:119-124), 200 steps in FP64.
  C2  a batch with aggregates at both clip sizes (32 and 2048 monomers), sintered bonds + Hamaker.
  C3  a batch with aggregates at both clip sizes (128 and 4096 monomers), breaking bonds at 10 nN,
      contact + Hamaker, pushed by a plane wall at 1 m/s.

Tolerances (FP64): per-step forces and torques within 1e-12 relative (normwise over the system),
positions within 1e-9 relative after 100 steps. The kernels that walk a row in the reference's
order (compacted, pair-parallel, row groups of one lane) are held to bit equality. Row groups of
T > 1 lanes combine a row's partial sums in a different order, so their forces are compared with
the oracle's at identical states: the bit-exact run is snapshotted, one step is taken with the
T-lane kernel from the same positions, velocities and springs as the oracle's step, and the run is
then restored."""
import os

import numpy as np
import pytest

from libgran_gb300 import _abi as A
from libgran_gb300 import configs as K
from libgran_gb300.system import System, generate_aggregate, generate_velocities
from oracle import oracle as O

import helpers as H

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-12
POS_TOL = 1e-9
STATE = (A.LG_FIELD_X, A.LG_FIELD_V, A.LG_FIELD_THETA, A.LG_FIELD_OMEGA, A.LG_FIELD_A, A.LG_FIELD_ALPHA)
THREADS = os.cpu_count() or 1


def _bit_equal(s, o, where):
    for f in STATE:
        a, b = s.get(f), o.get(f)
        assert np.array_equal(a, b), "%s: %s differs (rel %g)" % (where, H.FIELD_NAMES[f], H.rel_err(a, b))


def _rowgroup_forces_at_identical_state(s, o, dt, rebuild, lanes, kernel=A.LG_FORCE_KERNEL_ROWGROUP):
    """s and o hold bit-identical states (positions, velocities, springs). For each lane count, one
    step of s with the T-lane row-group kernel (or another kernel) is compared with one step of o; s
    is then restored and stepped with its own kernel, which brings it level with o again."""
    kernel0 = s.desc.force_kernel
    T0 = max(int(s.desc.threads_per_row), 1)
    o_next = None
    worst = 0.0
    for T in lanes:
        s.snapshot()
        s.set_force_kernel(kernel)
        s.set_threads_per_row(T)
        s.step(dt, 1, rebuild)
        if o_next is None:
            o.step(dt, 1, rebuild)
            o_next = (o.get(A.LG_FIELD_A), o.get(A.LG_FIELD_ALPHA), o.get(A.LG_FIELD_X))
        ea = H.rel_err(s.get(A.LG_FIELD_A), o_next[0])
        et = H.rel_err(s.get(A.LG_FIELD_ALPHA), o_next[1])
        assert ea <= FORCE_TOL and et <= FORCE_TOL, (T, ea, et)
        # the step's drift used the previous step's (identical) accelerations
        assert np.array_equal(s.get(A.LG_FIELD_X), o_next[2]), T
        worst = max(worst, ea, et)
        s.restore()
        s.set_force_kernel(kernel0)
        s.set_threads_per_row(T0)
    s.step(dt, 1, rebuild)
    return worst


def test_c0_exact_configuration_ten_thousand_steps():
    """C0 as configured: every FP64 kernel that walks rows in order stays bit-identical to the
    oracle for 10^4 steps; row groups of 4 and 32 lanes give the oracle's forces within 1e-12 at
    identical states along the run."""
    mat = K.Material()
    n = 256
    x0 = generate_aggregate(0, n, mat.r)
    v0 = generate_velocities(0, n, 0.1)
    d = K.make_desc(n, A.LG_BINARY_SINTER, A.LG_HAMAKER_FULL, contact=mat.contact(), sinter=mat.sinter(),
                    hamaker=mat.hamaker(), pairs=A.LG_PAIRS_ALL)
    o = O.OracleSystem(d, x0, v0, threads=THREADS)
    assert len(o.bonds()) == 2 * (n - 1)  # the aggregate's tree (ordered pairs): every touching pair bonded
    systems = {}
    for name, kern in (("auto", A.LG_FORCE_KERNEL_AUTO), ("pairs", A.LG_FORCE_KERNEL_PAIRS),
                       ("compact", A.LG_FORCE_KERNEL_COMPACT), ("rowgroup1", A.LG_FORCE_KERNEL_ROWGROUP)):
        dk = K.make_desc(n, A.LG_BINARY_SINTER, A.LG_HAMAKER_FULL, contact=mat.contact(), sinter=mat.sinter(),
                         hamaker=mat.hamaker(), pairs=A.LG_PAIRS_ALL, force_kernel=kern, threads_per_row=1)
        systems[name] = System(dk, x0, v0)
    for name, s in systems.items():
        _bit_equal(s, o, "construction, " + name)
    done = 0
    for cp in (1, 100, 5000, 10000):
        o.step(mat.dt, cp - done)
        for name, s in systems.items():
            s.step(mat.dt, cp - done)
            _bit_equal(s, o, "step %d, %s" % (cp, name))
        if cp == 100:
            assert H.rel_err(systems["auto"].get(A.LG_FIELD_X), o.get(A.LG_FIELD_X)) <= POS_TOL
        done = cp
    s = systems["compact"]
    for cp in (10000, 10001):  # identical states at the end of the run (the helper steps both by one)
        _rowgroup_forces_at_identical_state(s, o, mat.dt, 0, (4, 32))
        _bit_equal(s, o, "after the row-group check at step %d" % (cp + 1))
    # the fast FP64 kernel (reciprocals, one Hamaker denominator) at the same identical states
    assert _rowgroup_forces_at_identical_state(s, o, mat.dt, 0, (1,), kernel=A.LG_FORCE_KERNEL_FP64_FAST) <= FORCE_TOL
    _bit_equal(s, o, "after the fast-kernel check")
    for s in systems.values():
        assert np.array_equal(s.bonds(), o.bonds())
        assert s.device_errors() == 0
        s.close()


def test_c1_fp64_32768_against_oracle():
    """C1 in FP64 at 32768 monomers: bit-identical to the oracle (all host cores) over 200 steps
    and 10 list rebuilds with spring carry; row groups of 4 and 32 lanes within 1e-12 of the
    oracle's forces at identical states after contacts have formed."""
    mat = K.Material()
    n = 32768
    x0 = generate_aggregate(1 << 32, n, mat.r)
    v0 = generate_velocities(1 << 32, n, 0.1)
    d = K.make_desc(n, A.LG_BINARY_CONTACT, A.LG_HAMAKER_LIMITED, contact=mat.contact(), hamaker=mat.hamaker(),
                    pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r, max_neighbors=96,
                    force_kernel=A.LG_FORCE_KERNEL_COMPACT, threads_per_row=1)
    s = System(d, x0, v0)
    o = O.OracleSystem(d, x0, v0, threads=THREADS)
    _bit_equal(s, o, "construction")
    done = 0
    for cp in (1, 20, 100, 200):
        s.step(mat.dt, cp - done, 20)
        o.step(mat.dt, cp - done, 20)
        _bit_equal(s, o, "step %d" % cp)
        done = cp
    assert o.observables()["n_contacts"] > 1000  # contacts formed and are carried
    worst = _rowgroup_forces_at_identical_state(s, o, mat.dt, 20, (4, 32))
    _bit_equal(s, o, "after the row-group check")
    assert worst <= FORCE_TOL
    worst = _rowgroup_forces_at_identical_state(s, o, mat.dt, 20, (1,), kernel=A.LG_FORCE_KERNEL_FP64_FAST)
    _bit_equal(s, o, "after the fast-kernel check")
    assert worst <= FORCE_TOL
    # springs of contacting pairs agree after the rebuilds
    checked = 0
    for i in range(0, n, 1021):
        for j in o.row(i)[:8]:
            so = o.springs(i, j)
            if np.abs(so).max() > 0:
                assert np.array_equal(s.springs(i, j), so), (i, j)
                checked += 1
    assert checked > 0
    assert s.device_errors() == 0
    s.close()


def _batch_against_oracle(sizes, seed_config, desc_of, steps, facets=None, neck_of=None, prep=None):
    mat = K.Material()
    sizes = np.asarray(sizes, dtype=np.int64)
    x0, v0 = K.seeded_aggregates(sizes, seed_config, mat.r)
    if prep is not None:
        x0 = prep(x0, sizes, mat.r)
    off = np.concatenate([[0], np.cumsum(sizes)])
    d = desc_of(mat, int(sizes.sum()), A.LG_PRECISION_FP64)
    neck = None
    if neck_of is not None:
        probe = System(d, x0, v0, facets=facets, sizes=sizes)
        neck = neck_of(len(probe.bonds()) // 2)
        probe.close()
    s = System(d, x0, v0, facets=facets, neck=neck, sizes=sizes)
    s.step(mat.dt, steps, 20)
    got = {f: s.get(f) for f in STATE}
    assert s.device_errors() == 0
    s.close()
    oracles = []
    for q in range(len(sizes)):
        dq = desc_of(mat, int(sizes[q]), A.LG_PRECISION_FP64)
        xq, vq = x0[off[q]:off[q + 1]], v0[off[q]:off[q + 1]]
        nq = None
        if neck_of is not None:
            nq = neck_of(len(O.OracleSystem(dq, xq, vq, facets=facets).bonds()) // 2)
        oracles.append(O.OracleSystem(dq, xq, vq, facets=facets, neck=nq))
    O.run_many(oracles, [mat.dt] * len(oracles), [steps] * len(oracles), [20] * len(oracles))
    for q, o in enumerate(oracles):
        for f in STATE:
            assert np.array_equal(o.get(f), got[f][off[q]:off[q + 1]]), (q, int(sizes[q]), H.FIELD_NAMES[f])
    return x0, v0, sizes


def test_c2_batch_at_the_clip_sizes_matches_oracle():
    """C2's composition (sintered bonds + limited Hamaker + contact for non-bonded pairs, Verlet
    rows): a batch holding aggregates of 2048 and 32 monomers (the clip sizes) and the median size
    is bit-identical to the oracle system by system over 100 steps."""
    def desc_of(mat, n, prec):
        return K.make_desc(n, A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, contact=mat.contact(), sinter=mat.sinter(),
                           hamaker=mat.hamaker(), pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r, precision=prec,
                           force_kernel=A.LG_FORCE_KERNEL_COMPACT)
    _batch_against_oracle([2048, 32, 256, 2048, 33, 700], 2, desc_of, 100)


def test_c3_batch_at_the_clip_sizes_matches_oracle():
    """C3's composition (bonds breaking at 10 nN, contact + limited Hamaker, a plane wall moving
    at 1 m/s): a batch holding aggregates of 4096 and 128 monomers is bit-identical to the oracle
    system by system over 200 steps."""
    mat = K.Material()
    wall = K.wall_facet(mat, extent=50 * mat.r)

    def desc_of(m, n, prec):
        return K.make_desc(n, A.LG_BINARY_BREAKING_SINTER, A.LG_HAMAKER_LIMITED, contact=m.contact(),
                           sinter=m.sinter(), hamaker=m.hamaker(), pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * m.r,
                           precision=prec, n_facets=1, facet_auto_move=1, force_kernel=A.LG_FORCE_KERNEL_COMPACT)
    _batch_against_oracle([4096, 128, 1000, 4096, 130], 3, desc_of, 200, facets=[wall],
                          neck_of=lambda nb: np.full(nb, 1e-8), prep=K.rest_on_wall)


@pytest.mark.parametrize("case", ["c0", "c1"])
def test_fast_fp64_kernel_follows_the_oracle(case):
    """LG_FORCE_KERNEL_FP64_FAST on its own for 100 steps: forces within 1e-12 of the oracle's at the
    start (identical state), positions within 1e-9 after 100 steps (2 and 5 list rebuilds)."""
    mat = K.Material()
    if case == "c0":
        n, seed = 256, 0
        d = K.make_desc(n, A.LG_BINARY_SINTER, A.LG_HAMAKER_FULL, contact=mat.contact(), sinter=mat.sinter(),
                        hamaker=mat.hamaker(), pairs=A.LG_PAIRS_ALL, force_kernel=A.LG_FORCE_KERNEL_FP64_FAST)
        rb = 0
    else:
        n, seed = 32768, 1 << 32
        d = K.make_desc(n, A.LG_BINARY_CONTACT, A.LG_HAMAKER_LIMITED, contact=mat.contact(), hamaker=mat.hamaker(),
                        pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r, max_neighbors=96,
                        force_kernel=A.LG_FORCE_KERNEL_FP64_FAST)
        rb = 20
    x0, v0 = generate_aggregate(seed, n, mat.r), generate_velocities(seed, n, 0.1)
    s = System(d, x0, v0)
    o = O.OracleSystem(d, x0, v0, threads=THREADS)
    for f in (A.LG_FIELD_A, A.LG_FIELD_ALPHA):
        assert H.rel_err(s.get(f), o.get(f)) <= FORCE_TOL, H.FIELD_NAMES[f]
    s.step(mat.dt, 100, rb)
    o.step(mat.dt, 100, rb)
    assert H.rel_err(s.get(A.LG_FIELD_X), o.get(A.LG_FIELD_X)) <= POS_TOL
    assert H.rel_err(s.get(A.LG_FIELD_X) - x0, o.get(A.LG_FIELD_X) - x0) <= POS_TOL
    assert s.device_errors() == 0
