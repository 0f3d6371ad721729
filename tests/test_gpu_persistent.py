"""The persistent step kernel of the mixed path (LG_FORCE_KERNEL_PERSISTENT): every step inside a
run of steps is one launch whose warps pull contact and Hamaker work items from a device queue and
complete each 32-row group when its last item finishes. Each row's arithmetic and order of terms are
those of the compacted two-stream kernels with the same slicing, so both must give the same bits,
eagerly and graph-replayed, for single systems, batches and all-pairs mode."""
import numpy as np
import pytest

from libgran_gb300 import _abi as A
from libgran_gb300 import configs as K
from libgran_gb300.system import System, generate_aggregate, generate_velocities

import helpers as H

pytestmark = pytest.mark.gpu

FIELDS = (A.LG_FIELD_X, A.LG_FIELD_V, A.LG_FIELD_THETA, A.LG_FIELD_OMEGA, A.LG_FIELD_A, A.LG_FIELD_ALPHA)


def _run(desc, x0, v0, kernel, schedule, sizes=None, graphs=True):
    desc.force_kernel = kernel
    s = System(desc, x0, v0, sizes=sizes)
    s.set_graphs(graphs)
    for nst, rb in schedule:
        s.step(K.Material().dt, nst, rb)
    out = [s.get(f) for f in FIELDS]
    assert s.device_errors() == 0
    s.close()
    return out


def _same(a, b):
    for f, x, y in zip(FIELDS, a, b):
        assert np.array_equal(x, y), "%s differs (rel %g)" % (H.FIELD_NAMES[f], H.rel_err(x, y))


@pytest.mark.parametrize("bm,hm", [(A.LG_BINARY_CONTACT, A.LG_HAMAKER_LIMITED), (A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED),
                                   (A.LG_BINARY_NONE, A.LG_HAMAKER_LIMITED), (A.LG_BINARY_SINTER, A.LG_HAMAKER_NONE)],
                         ids=["contact+ham", "sinter+ham", "ham", "sinter"])
@pytest.mark.parametrize("n", [32768, 1000, 45])
def test_persistent_matches_compact_verlet(n, bm, hm):
    mat = K.Material()
    x0 = generate_aggregate(1 << 32, n, mat.r)
    v0 = generate_velocities(1 << 32, n, 0.1) - 1e7 * (x0 - x0.mean(0))
    d = K.make_desc(n, bm, hm, contact=mat.contact(), sinter=mat.sinter(), hamaker=mat.hamaker(),
                    pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r, precision=A.LG_PRECISION_MIXED, max_neighbors=96)
    sched = [(60, 20), (7, 20), (33, 20), (1, 20), (19, 20)]  # whole periods, a tail, realignment, a single step
    ref = _run(d, x0, v0, A.LG_FORCE_KERNEL_COMPACT, sched)
    _same(_run(d, x0, v0, A.LG_FORCE_KERNEL_PERSISTENT, sched), ref)
    _same(_run(d, x0, v0, A.LG_FORCE_KERNEL_PERSISTENT, sched, graphs=False), ref)


def test_persistent_matches_compact_all_pairs():
    """All pairs: the persistent kernel defers to the compacted kernels (a warp per contact row)."""
    mat = K.Material()
    n = 300
    x0 = generate_aggregate(5, n, mat.r)
    v0 = generate_velocities(5, n, 0.1) - 2e7 * (x0 - x0.mean(0))
    d = K.make_desc(n, A.LG_BINARY_SINTER, A.LG_HAMAKER_FULL, contact=mat.contact(), sinter=mat.sinter(),
                    hamaker=mat.hamaker(), precision=A.LG_PRECISION_MIXED)
    sched = [(50, 0), (3, 0), (16, 0)]
    _same(_run(d, x0, v0, A.LG_FORCE_KERNEL_PERSISTENT, sched), _run(d, x0, v0, A.LG_FORCE_KERNEL_COMPACT, sched))


def test_persistent_matches_compact_in_a_batch():
    """C2-like batch (sintered bonds + Hamaker, sizes from 32 to 2048): the persistent kernel pulls
    items of every system from one queue."""
    mat = K.Material()
    sizes = np.array([2048, 32, 256, 700, 33, 2048, 90])
    x0, v0 = K.seeded_aggregates(sizes, 2, mat.r)
    d = K.make_desc(int(sizes.sum()), A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, contact=mat.contact(),
                    sinter=mat.sinter(), hamaker=mat.hamaker(), pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r,
                    precision=A.LG_PRECISION_MIXED)
    sched = [(100, 20), (11, 20)]
    _same(_run(d, x0, v0, A.LG_FORCE_KERNEL_PERSISTENT, sched, sizes=sizes),
          _run(d, x0, v0, A.LG_FORCE_KERNEL_COMPACT, sched, sizes=sizes))


def test_persistent_falls_back_where_it_does_not_apply():
    """Held particles and facets take the compacted kernels (their completion needs FP64 state);
    the results are those of the compacted kernels."""
    mat = K.Material()
    n = 500
    x0 = generate_aggregate(9, n, mat.r)
    v0 = generate_velocities(9, n, 0.1)
    mask = np.zeros(n, dtype=np.uint8)
    mask[::7] = A.LG_HOLD_X | A.LG_HOLD_V
    outs = []
    for kern in (A.LG_FORCE_KERNEL_COMPACT, A.LG_FORCE_KERNEL_PERSISTENT):
        d = K.make_desc(n, A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, contact=mat.contact(), sinter=mat.sinter(),
                        hamaker=mat.hamaker(), pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r,
                        precision=A.LG_PRECISION_MIXED, force_kernel=kern)
        K.set_hold(d, mask)
        s = System(d, x0, v0)
        s.step(mat.dt, 40, 20)
        outs.append([s.get(f) for f in FIELDS])
    _same(outs[1], outs[0])


def _run_shape(desc, x0, v0, kernel, shape, schedule, sizes=None):
    desc.force_kernel = kernel
    s = System(desc, x0, v0, sizes=sizes)
    s.set_step_shape(*shape)
    for nst, rb in schedule:
        s.step(K.Material().dt, nst, rb)
    out = [s.get(f) for f in FIELDS]
    assert s.device_errors() == 0
    s.close()
    return out


@pytest.mark.parametrize("assign", [0, 1, 2])
@pytest.mark.parametrize("mb,sl", [(4, 1), (4, 4), (5, 2), (6, 4)])
def test_persistent_shapes_give_the_compact_bits(mb, sl, assign):
    """Every shape (register budget, Hamaker slices, one launch pulling or round-robin, or the two
    launches side by side) gives the bits of the compacted kernels with the same slices."""
    mat = K.Material()
    n = 6000
    x0 = generate_aggregate(77, n, mat.r)
    v0 = generate_velocities(77, n, 0.1) - 1e7 * (x0 - x0.mean(0))
    d = K.make_desc(n, A.LG_BINARY_CONTACT, A.LG_HAMAKER_LIMITED, contact=mat.contact(), hamaker=mat.hamaker(),
                    pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r, precision=A.LG_PRECISION_MIXED)
    sched = [(40, 20), (13, 20)]
    ref = _run_shape(d, x0, v0, A.LG_FORCE_KERNEL_COMPACT, (0, sl, 0), sched)
    _same(_run_shape(d, x0, v0, A.LG_FORCE_KERNEL_PERSISTENT, (mb, sl, assign), sched), ref)


def test_split_launches_in_a_batch_with_bonds():
    """The two side-by-side launches on a batch of sintered aggregates of uneven sizes."""
    mat = K.Material()
    sizes = np.array([1500, 40, 333, 2048, 7])
    x0, v0 = K.seeded_aggregates(sizes, 4, mat.r)
    d = K.make_desc(int(sizes.sum()), A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, contact=mat.contact(),
                    sinter=mat.sinter(), hamaker=mat.hamaker(), pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r,
                    precision=A.LG_PRECISION_MIXED)
    sched = [(60, 20), (5, 20)]
    ref = _run_shape(d, x0, v0, A.LG_FORCE_KERNEL_COMPACT, (0, 2, 0), sched, sizes=sizes)
    _same(_run_shape(d, x0, v0, A.LG_FORCE_KERNEL_PERSISTENT, (4, 2, 2), sched, sizes=sizes), ref)
