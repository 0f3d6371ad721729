"""Batches of independent aggregates in one handle, CUDA-graph replay and the autotuner.

A system inside a batch must give the same result as the same system alone (its rows, springs and
bonds never involve other systems): for the compacted kernels this holds bit for bit."""
import numpy as np
import pytest

from libgran_gb300 import _abi as A
from libgran_gb300 import configs as K
from libgran_gb300.system import System, generate_aggregate, generate_velocities
from oracle import oracle as O

import helpers as H

pytestmark = pytest.mark.gpu

FIELDS = (A.LG_FIELD_X, A.LG_FIELD_V, A.LG_FIELD_OMEGA, A.LG_FIELD_A, A.LG_FIELD_ALPHA)


def _systems(sizes, seed0=1000, squeeze=2e7):
    mat = K.Material()
    xs, vs = [], []
    for q, n in enumerate(sizes):
        x = generate_aggregate(seed0 + q, n, mat.r)
        v = generate_velocities(seed0 + q, n, 0.1) - squeeze * (x - x.mean(0))
        xs.append(x)
        vs.append(v)
    return mat, xs, vs


def _desc(mat, n, bm, precision, kernel=A.LG_FORCE_KERNEL_COMPACT):
    return K.make_desc(n, bm, A.LG_HAMAKER_LIMITED, contact=mat.contact(), sinter=mat.sinter(), hamaker=mat.hamaker(),
                       pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r, precision=precision, force_kernel=kernel,
                       max_neighbors=160)


@pytest.mark.parametrize("precision", [A.LG_PRECISION_FP64, A.LG_PRECISION_MIXED], ids=["fp64", "mixed"])
@pytest.mark.parametrize("bm", [A.LG_BINARY_SINTER, A.LG_BINARY_CONTACT], ids=["sinter", "contact"])
def test_batch_matches_systems_alone_bit_for_bit(precision, bm):
    sizes = [37, 256, 90, 600, 33]
    mat, xs, vs = _systems(sizes)
    batch = System(_desc(mat, sum(sizes), bm, precision), np.concatenate(xs), np.concatenate(vs), sizes=sizes)
    batch.step(mat.dt, 100, 20)
    bx = batch.get(A.LG_FIELD_X)
    bobs = batch.batch_observables()
    off = np.concatenate([[0], np.cumsum(sizes)])
    for q, n in enumerate(sizes):
        alone = System(_desc(mat, n, bm, precision), xs[q], vs[q])
        alone.step(mat.dt, 100, 20)
        for f in FIELDS:
            assert np.array_equal(alone.get(f), batch.get(f)[off[q]:off[q + 1]]), (q, H.FIELD_NAMES[f])
        ao = alone.observables()
        for k in ("ke_total", "radius_of_gyration", "potential_energy", "linear_momentum"):
            assert abs(ao[k] - bobs[q][k]) <= 1e-12 * max(abs(ao[k]), 1e-300), (q, k)
        assert ao["n_bonds"] == bobs[q]["n_bonds"]
    assert batch.device_errors() == 0


@pytest.mark.parametrize("kernel", [A.LG_FORCE_KERNEL_COMPACT, A.LG_FORCE_KERNEL_PAIRS], ids=["compact", "pairs"])
def test_batch_fp64_matches_oracle(kernel):
    sizes = [64, 200, 48]
    mat, xs, vs = _systems(sizes, seed0=55)
    batch = System(_desc(mat, sum(sizes), A.LG_BINARY_SINTER, A.LG_PRECISION_FP64, kernel), np.concatenate(xs),
                   np.concatenate(vs), sizes=sizes)
    batch.step(mat.dt, 60, 20)
    off = np.concatenate([[0], np.cumsum(sizes)])
    for q, n in enumerate(sizes):
        o = O.OracleSystem(_desc(mat, n, A.LG_BINARY_SINTER, A.LG_PRECISION_FP64), xs[q], vs[q])
        o.step(mat.dt, 60, 20)
        for f in FIELDS:
            assert np.array_equal(o.get(f), batch.get(f)[off[q]:off[q + 1]]), (q, H.FIELD_NAMES[f])
    assert batch.device_errors() == 0


@pytest.mark.parametrize("precision,kernel", [(A.LG_PRECISION_FP64, A.LG_FORCE_KERNEL_COMPACT),
                                              (A.LG_PRECISION_MIXED, A.LG_FORCE_KERNEL_COMPACT),
                                              (A.LG_PRECISION_FP64, A.LG_FORCE_KERNEL_PAIRS)],
                         ids=["fp64", "mixed", "fp64-pairs"])
def test_graph_replay_equals_eager_launches(precision, kernel):
    sizes = [300, 500, 120]
    mat, xs, vs = _systems(sizes, seed0=7)
    outs = []
    for graphs in (False, True):
        s = System(_desc(mat, sum(sizes), A.LG_BINARY_SINTER, precision, kernel), np.concatenate(xs),
                   np.concatenate(vs), sizes=sizes)
        s.set_graphs(graphs)
        s.step(mat.dt, 100, 20)
        s.step(mat.dt, 7, 20)   # unaligned tail
        s.step(mat.dt, 53, 20)  # realigns and replays again
        outs.append([s.get(f) for f in FIELDS])
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


def test_autotuner_picks_a_valid_variant():
    sizes = [256] * 64
    mat, xs, vs = _systems(sizes, seed0=99)
    s = System(_desc(mat, sum(sizes), A.LG_BINARY_SINTER, A.LG_PRECISION_MIXED, kernel=A.LG_FORCE_KERNEL_AUTO),
               np.concatenate(xs), np.concatenate(vs), sizes=sizes)
    before = [s.get(f) for f in FIELDS]
    k, T = s.autotune(mat.dt, probe_steps=20, rebuild_every=20, use_cache=False)
    assert k in (A.LG_FORCE_KERNEL_COMPACT, A.LG_FORCE_KERNEL_ROWGROUP, A.LG_FORCE_KERNEL_PERSISTENT)
    assert T in (1, 2, 4, 8, 16, 32)
    t = s.tuning()
    assert t["force_kernel"] == k and t["ms_per_step"] > 0
    assert t["step_min_blocks"] in (4, 5, 6) and t["step_slices"] in (1, 2, 4) and t["step_assign"] in (0, 1, 2)
    for f, b in zip(FIELDS, before):  # tuning leaves the state as it was
        assert np.array_equal(s.get(f), b)
    s.step(mat.dt, 40, 20)
    assert s.device_errors() == 0
    # a second handle of the same kind takes the cached pick without timing anything
    s2 = System(_desc(mat, sum(sizes), A.LG_BINARY_SINTER, A.LG_PRECISION_MIXED, kernel=A.LG_FORCE_KERNEL_AUTO),
                np.concatenate(xs), np.concatenate(vs), sizes=sizes)
    s2.autotune(mat.dt, probe_steps=20, rebuild_every=20, use_cache=True)
    t2 = s2.tuning()
    for key in ("force_kernel", "threads_per_row", "step_min_blocks", "step_slices", "step_assign"):
        assert t2[key] == t[key], key
    s2.step(mat.dt, 40, 20)
    assert s2.device_errors() == 0


def test_snapshot_restore_replays_identically():
    sizes = [200, 300]
    mat, xs, vs = _systems(sizes, seed0=3)
    s = System(_desc(mat, sum(sizes), A.LG_BINARY_SINTER, A.LG_PRECISION_FP64), np.concatenate(xs), np.concatenate(vs),
               sizes=sizes)
    s.step(mat.dt, 20, 20)
    s.snapshot()
    s.step(mat.dt, 60, 20)
    first = [s.get(f) for f in FIELDS]
    s.restore()
    s.step(mat.dt, 60, 20)
    for a, f in zip(first, FIELDS):
        assert np.array_equal(a, s.get(f))


def test_restructuring_batch_with_wall_and_breaking_bonds_matches_oracle():
    """Batched aggregates pushed by a moving wall, bonds breaking at 10 nN: the FP64 batch is
    bit-identical to the oracle system by system; mixed precision gives the broken-bond fraction
    and radius of gyration within 1e-3 relative."""
    from libgran_gb300 import configs as K2
    mat = K.Material()
    sizes = np.array([128, 300, 200, 160])
    x0, v0 = K2.seeded_aggregates(sizes, 77, mat.r)
    x0 = K2.rest_on_wall(x0, sizes, mat.r)
    v0 = v0 * 20.0  # livelier than the workload so that bonds load within a short test
    wall = K2.wall_facet(mat, extent=50 * mat.r)
    off = np.concatenate([[0], np.cumsum(sizes)])
    res = {}
    for prec in (A.LG_PRECISION_FP64, A.LG_PRECISION_MIXED):
        d = K.make_desc(int(sizes.sum()), A.LG_BINARY_BREAKING_SINTER, A.LG_HAMAKER_LIMITED, contact=mat.contact(),
                        sinter=mat.sinter(), hamaker=mat.hamaker(), pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r,
                        precision=prec, n_facets=1, facet_auto_move=1, force_kernel=A.LG_FORCE_KERNEL_COMPACT,
                        max_neighbors=128)
        probe = System(d, x0, v0, facets=[wall], sizes=sizes)
        nb = len(probe.bonds()) // 2
        s = System(d, x0, v0, facets=[wall], neck=np.full(nb, 1e-8), sizes=sizes)
        b0 = len(s.bonds())
        s.step(mat.dt, 400, 20)
        res[prec] = (s, b0, len(s.bonds()), np.array([o["radius_of_gyration"] for o in s.batch_observables()]))
        assert s.device_errors() == 0
    s64, b0, b1, rg64 = res[A.LG_PRECISION_FP64]
    assert b1 < b0  # some bonds broke
    # FP64 batch == oracle, system by system
    for q in range(len(sizes)):
        n = int(sizes[q])
        dq = K.make_desc(n, A.LG_BINARY_BREAKING_SINTER, A.LG_HAMAKER_LIMITED, contact=mat.contact(),
                         sinter=mat.sinter(), hamaker=mat.hamaker(), pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r,
                         n_facets=1, facet_auto_move=1)
        xq, vq = x0[off[q]:off[q + 1]], v0[off[q]:off[q + 1]]
        probe = O.OracleSystem(dq, xq, vq, facets=[wall])
        nbq = len(probe.bonds()) // 2
        o = O.OracleSystem(dq, xq, vq, facets=[wall], neck=np.full(nbq, 1e-8))
        o.step(mat.dt, 400, 20)
        assert np.array_equal(o.get(A.LG_FIELD_X), s64.get(A.LG_FIELD_X)[off[q]:off[q + 1]]), q
    smx, c0, c1, rgmx = res[A.LG_PRECISION_MIXED]
    assert c0 == b0
    assert abs((c0 - c1) - (b0 - b1)) <= max(2, 1e-3 * (b0 - b1))  # 2 ordered pairs = one bond
    assert np.max(np.abs(rgmx - rg64) / rg64) <= 1e-3


def test_pair_parallel_kernel_limits():
    """The pair-parallel kernel is FP64 only and refuses systems beyond its scratch limit."""
    sizes = [64, 80]
    mat, xs, vs = _systems(sizes, seed0=3)
    with pytest.raises(RuntimeError, match="FP64 only"):
        System(_desc(mat, sum(sizes), A.LG_BINARY_SINTER, A.LG_PRECISION_MIXED, A.LG_FORCE_KERNEL_PAIRS),
               np.concatenate(xs), np.concatenate(vs), sizes=sizes)
    s = System(_desc(mat, sum(sizes), A.LG_BINARY_SINTER, A.LG_PRECISION_MIXED), np.concatenate(xs),
               np.concatenate(vs), sizes=sizes)
    with pytest.raises(RuntimeError, match="FP64 only"):
        s.set_force_kernel(A.LG_FORCE_KERNEL_PAIRS)


def test_one_contact_lane_per_row_from_a_tuning_record(tmp_path):
    """The mixed compacted kernels with one contact lane per row (a tuning choice for large batches,
    applied here from a cache record): eager and graph-replayed give the same bits, and the result
    stays within the mixed path's tolerance of the default two lanes."""
    L = A.lib()
    sizes = [300] * 40
    n = sum(sizes)
    mat, xs, vs = _systems(sizes, seed0=17)
    x0, v0 = np.concatenate(xs), np.concatenate(vs)
    lg2 = int(np.floor(np.log2(n)))
    f = tmp_path / "tune.txt"
    f.write_text("%d %d %d %d %d 1 : %d 1 4 4 0 1.0\n" % (A.LG_PRECISION_MIXED, A.LG_PAIRS_VERLET, A.LG_BINARY_SINTER,
                                                        A.LG_HAMAKER_LIMITED, lg2, A.LG_FORCE_KERNEL_COMPACT))
    assert L.lg_autotune_cache_clear() == A.LG_OK
    assert L.lg_autotune_cache_load(str(f).encode()) == A.LG_OK
    try:
        runs = []
        for graphs in (True, False):
            s = System(_desc(mat, n, A.LG_BINARY_SINTER, A.LG_PRECISION_MIXED, kernel=A.LG_FORCE_KERNEL_AUTO), x0, v0,
                       sizes=sizes)
            k, T = s.autotune(mat.dt, probe_steps=20, rebuild_every=20, use_cache=True)
            assert k == A.LG_FORCE_KERNEL_COMPACT and T == 1 and s.tuning()["threads_per_row"] == 1
            s.set_graphs(graphs)
            s.step(mat.dt, 60, 20)
            assert s.device_errors() == 0
            runs.append([s.get(f_) for f_ in FIELDS])
        for a, b in zip(*runs):
            assert np.array_equal(a, b)
        two = System(_desc(mat, n, A.LG_BINARY_SINTER, A.LG_PRECISION_MIXED, kernel=A.LG_FORCE_KERNEL_COMPACT), x0, v0,
                     sizes=sizes)
        assert two.tuning()["threads_per_row"] == 2
        two.step(mat.dt, 60, 20)
        x1, x2 = runs[0][0], two.get(A.LG_FIELD_X)
        assert np.abs(x1 - x2).max() <= 1e-5 * np.abs(x2 - x0).max()
    finally:
        L.lg_autotune_cache_clear()
