"""GPU engine against the golden fixtures (libgran's functors) and the oracle, through the C ABI.

Tolerances (FP64 path): per-step forces and torques within 1e-12 relative (normwise over the
system), positions within 1e-9 relative after 100 steps. With one lane per row the engine walks
each row in the reference's order and is expected to agree bit for bit; the checks below still use
the stated tolerances, and report the bit-exact cases separately."""
import os

import numpy as np
import pytest

from libgran_gb300 import _abi as A
from libgran_gb300 import configs as K
from libgran_gb300.system import System, generate_aggregate, generate_velocities
from oracle import oracle as O

import helpers as H
import known_answer as KA

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-12
POS_TOL = 1e-9


@pytest.mark.parametrize("path", H.golden_files(), ids=lambda p: os.path.basename(p)[:-4])
def test_gpu_reproduces_golden_sequential_rows(path):
    g = np.load(path)
    case = H.golden_case(os.path.basename(path)[:-4])
    case["desc"].threads_per_row = 1
    s = System(case["desc"], g["x0"], g["v0"], facets=case.get("facets"), neck=case.get("neck"))
    worst = {}

    def check(f, cp, got, want):
        e = H.rel_err(got, want)
        worst[H.FIELD_NAMES[f]] = max(worst.get(H.FIELD_NAMES[f], 0.0), e)
        tol = FORCE_TOL if cp <= 1 or f in (A.LG_FIELD_A, A.LG_FIELD_ALPHA) and cp <= 10 else POS_TOL
        assert e <= tol, "%s step %d: rel err %g" % (H.FIELD_NAMES[f], cp, e)

    H.run_checkpoints(s, case, g, check)
    for (i, j), sp in zip(g["spring_pairs"], g["springs"]):
        assert H.rel_err(s.springs(i, j), sp) <= POS_TOL or np.abs(sp).max() == 0.0
    assert np.array_equal(s.bonds(), g["bonds"])
    assert s.device_errors() == 0


@pytest.mark.parametrize("kernel", [A.LG_FORCE_KERNEL_ROWGROUP, A.LG_FORCE_KERNEL_COMPACT, A.LG_FORCE_KERNEL_PAIRS],
                         ids=["rowgroup1", "compact", "pairs"])
@pytest.mark.parametrize("path", H.golden_files(), ids=lambda p: os.path.basename(p)[:-4])
def test_gpu_sequential_rows_are_bit_exact_with_oracle(path, kernel):
    g = np.load(path)
    case = H.golden_case(os.path.basename(path)[:-4])
    case["desc"].threads_per_row = 1
    case["desc"].force_kernel = kernel
    s = System(case["desc"], g["x0"], g["v0"], facets=case.get("facets"), neck=case.get("neck"))
    o = O.OracleSystem(case["desc"], g["x0"], g["v0"], facets=case.get("facets"), neck=case.get("neck"))
    for nst in (1, 9, 90):
        s.step(case["dt"], nst, case.get("rebuild", 0))
        o.step(case["dt"], nst, case.get("rebuild", 0))
        for f in H.FIELDS:
            assert np.array_equal(s.get(f), o.get(f)), "%s differs after %d steps" % (H.FIELD_NAMES[f], nst)


def _aggregate_system(n, seed, bm, hm, pairs, neck_mode=A.LG_NECK_PER_BOND, vscale=0.1, squeeze=0.0):
    mat = K.Material()
    x0 = generate_aggregate(seed, n, mat.r)
    v0 = generate_velocities(seed, n, vscale) - squeeze * (x0 - x0.mean(0))
    d = K.make_desc(n, bm, hm, contact=mat.contact(), sinter=mat.sinter(), hamaker=mat.hamaker(), neck_mode=neck_mode,
                    pairs=pairs, r_verlet=4.5 * mat.r if pairs == A.LG_PAIRS_VERLET else 0.0)
    return mat, d, x0, v0


@pytest.mark.parametrize("T", [1, 4, 32, 0, -1])  # 0: compacted kernel, -1: pair-parallel kernel
@pytest.mark.parametrize("bm,hm", [(A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED), (A.LG_BINARY_CONTACT, A.LG_HAMAKER_FULL),
                                   (A.LG_BINARY_BREAKING_SINTER, A.LG_HAMAKER_LIMITED)])
def test_all_pairs_forces_and_positions(T, bm, hm):
    mat, d, x0, v0 = _aggregate_system(256, 21, bm, hm, A.LG_PAIRS_ALL, squeeze=2e7)
    if T <= 0:
        d.force_kernel = A.LG_FORCE_KERNEL_COMPACT if T == 0 else A.LG_FORCE_KERNEL_PAIRS
        T = 1
    nb = None
    if bm == A.LG_BINARY_BREAKING_SINTER:
        probe = O.OracleSystem(d, x0, v0)
        nb = np.full(len(probe.bonds()) // 2, 2e-9)
    d.threads_per_row = T
    s = System(d, x0, v0, neck=nb)
    o = O.OracleSystem(d, x0, v0, neck=nb, threads=4)
    for step in range(1, 101):
        s.step(mat.dt, 1)
        o.step(mat.dt, 1)
        if step <= 5 or step % 25 == 0:
            assert H.rel_err(s.get(A.LG_FIELD_A), o.get(A.LG_FIELD_A)) <= FORCE_TOL * (1 if step <= 1 else 1e3)
            assert H.rel_err(s.get(A.LG_FIELD_ALPHA), o.get(A.LG_FIELD_ALPHA)) <= FORCE_TOL * (1 if step <= 1 else 1e3)
    assert H.rel_err(s.get(A.LG_FIELD_X) - x0, o.get(A.LG_FIELD_X) - x0) <= POS_TOL
    assert H.rel_err(s.get(A.LG_FIELD_X), o.get(A.LG_FIELD_X)) <= POS_TOL
    if T == 1:
        assert np.array_equal(s.get(A.LG_FIELD_X), o.get(A.LG_FIELD_X))
    assert np.array_equal(s.bonds(), o.bonds())


@pytest.mark.parametrize("T", [1, 8, 0, -1])
def test_verlet_list_with_spring_carry(T):
    mat, d, x0, v0 = _aggregate_system(2000, 33, A.LG_BINARY_CONTACT, A.LG_HAMAKER_LIMITED, A.LG_PAIRS_VERLET,
                                       squeeze=3e7)
    if T <= 0:  # compacted / pair-parallel kernel: sequential order per row, bit-exact
        d.force_kernel = A.LG_FORCE_KERNEL_COMPACT if T == 0 else A.LG_FORCE_KERNEL_PAIRS
        T = 1
    else:
        d.force_kernel = A.LG_FORCE_KERNEL_ROWGROUP
    d.threads_per_row = T
    s = System(d, x0, v0)
    o = O.OracleSystem(d, x0, v0, threads=8)
    for k in range(5):
        s.step(mat.dt, 20, 20)
        o.step(mat.dt, 20, 20)
        assert H.rel_err(s.get(A.LG_FIELD_A), o.get(A.LG_FIELD_A)) <= (FORCE_TOL if T == 1 else 1e-9)
    assert H.rel_err(s.get(A.LG_FIELD_X), o.get(A.LG_FIELD_X)) <= POS_TOL
    # springs of contacting pairs were carried across the rebuilds
    xs = o.get(A.LG_FIELD_X)
    checked = 0
    for i in range(0, 2000, 97):
        for j in o.row(i)[:6]:
            sw, so = s.springs(i, j), o.springs(i, j)
            if np.abs(so).max() > 0:
                assert H.rel_err(sw, so) <= 1e-6
                checked += 1
    assert s.device_errors() == 0
    assert o.observables()["n_contacts"] > 0


def test_observables_match_oracle():
    mat, d, x0, v0 = _aggregate_system(512, 9, A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, A.LG_PAIRS_ALL)
    s = System(d, x0, v0)
    o = O.OracleSystem(d, x0, v0)
    s.step(mat.dt, 50)
    o.step(mat.dt, 50)
    a, b = s.observables(), o.observables()
    for k in ("ke_translational", "ke_rotational", "ke_total", "linear_momentum", "angular_momentum",
              "radius_of_gyration", "potential_energy"):
        assert abs(a[k] - b[k]) <= 1e-10 * max(abs(b[k]), 1e-300), (k, a[k], b[k])
    assert a["n_bonds"] == b["n_bonds"] and a["n_contacts"] == b["n_contacts"]
    assert np.allclose(a["center_of_mass"], b["center_of_mass"], rtol=1e-12, atol=1e-22)
    # the selectable parts give the same numbers as the full call, and zeros for what was not asked
    st, pr = s.observables(A.LG_OBS_STATE), s.observables(A.LG_OBS_PAIRS)
    for k in ("ke_translational", "ke_rotational", "ke_total", "linear_momentum", "angular_momentum",
              "radius_of_gyration"):
        assert st[k] == a[k] and pr[k] == 0.0, k
    assert list(st["center_of_mass"]) == list(a["center_of_mass"])
    assert pr["potential_energy"] == a["potential_energy"] and st["potential_energy"] == 0.0
    assert pr["n_contacts"] == a["n_contacts"] and pr["n_bonds"] == a["n_bonds"] and st["n_bonds"] == 0
    assert st["n_bonds_initial"] == pr["n_bonds_initial"] == a["n_bonds_initial"]


def test_results_are_deterministic():
    mat, d, x0, v0 = _aggregate_system(3000, 4, A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, A.LG_PAIRS_VERLET)
    outs = []
    for _ in range(2):
        d.threads_per_row = 4
        s = System(d, x0, v0)
        s.step(mat.dt, 60, 20)
        outs.append([s.get(f) for f in H.FIELDS])
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


def test_list_overflow_is_reported_not_faulted():
    mat, d, x0, v0 = _aggregate_system(500, 2, A.LG_BINARY_CONTACT, A.LG_HAMAKER_LIMITED, A.LG_PAIRS_VERLET)
    d.max_neighbors = 2
    s = System(d, x0, v0)
    assert s.device_errors() & A.LG_DEVERR_LIST_OVERFLOW


def test_facet_auto_move_and_manual_move():
    c = KA.surface_case()
    f = KA.surface_facet(c["dt"], A_h=1e-20)
    f.v_facet[2] = 0.5
    d = c["desc"]
    d.facet_auto_move = 1
    s = System(d, c["x0"], c["v0"], facets=[f])
    o = O.OracleSystem(d, c["x0"], c["v0"], facets=[f])
    s.step(c["dt"], 1000)
    o.step(c["dt"], 1000)
    assert np.array_equal(s.facet_vertices(0), o.facet_vertices(0))
    s.facet_update_positions(0, 1e-9)
    o.facet_update_positions(0, 1e-9)
    assert np.array_equal(s.facet_vertices(0), o.facet_vertices(0))
    s.step(c["dt"], 100)
    o.step(c["dt"], 100)
    assert H.rel_err(s.get(A.LG_FIELD_X), o.get(A.LG_FIELD_X)) <= 1e-12
