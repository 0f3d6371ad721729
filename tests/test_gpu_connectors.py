"""The 5-connector sinter model (sinter_bridge.h: sinter_functor + sinter_step_handler) on the GPU,
through the C ABI: bit-exact with the oracle (which is bit-exact with libgran's own functor and
step handler, tests/test_oracle_cpu.py), inside batches, and libgran's sintered_test known answer."""
import numpy as np
import pytest

from libgran_gb300 import _abi as A
from libgran_gb300 import configs as K
from libgran_gb300.system import System, generate_aggregate, generate_velocities
from oracle import oracle as O

import helpers as H
import known_answer as KA

pytestmark = pytest.mark.gpu


def _connector_desc(mat, x0, pairs, hm, seed, kernel=A.LG_FORCE_KERNEL_AUTO, precision=A.LG_PRECISION_FP64):
    d = K.make_desc(len(x0), A.LG_BINARY_SINTER_CONNECTORS, hm, contact=mat.contact(), hamaker=mat.hamaker(),
                    pairs=pairs, r_verlet=4.5 * mat.r if pairs == A.LG_PAIRS_VERLET else 0.0, precision=precision,
                    force_kernel=kernel)
    nb = len(K.connector_bonds(x0, mat.r, mat.d_crit))
    K.set_connectors(d, 0.5 * mat.k_n, 0.3 * mat.g_n, mat.d_crit, K.random_unit_axes(nb, seed))
    return d


@pytest.mark.parametrize("kernel", [A.LG_FORCE_KERNEL_ROWGROUP, A.LG_FORCE_KERNEL_COMPACT, A.LG_FORCE_KERNEL_PAIRS],
                         ids=["rowgroup1", "compact", "pairs"])
@pytest.mark.parametrize("pairs,n", [(A.LG_PAIRS_ALL, 200), (A.LG_PAIRS_VERLET, 3000)], ids=["all", "verlet"])
def test_connectors_bit_exact_with_oracle(pairs, n, kernel):
    mat = K.Material()
    x0 = generate_aggregate(61, n, mat.r)
    v0 = generate_velocities(61, n, 0.3) - 1.5e7 * (x0 - x0.mean(0))
    d = _connector_desc(mat, x0, pairs, A.LG_HAMAKER_LIMITED, 61, kernel)
    d.threads_per_row = 1
    s = System(d, x0, v0)
    o = O.OracleSystem(d, x0, v0)
    for nst in (1, 19, 40):
        s.step(mat.dt, nst, 20)
        o.step(mat.dt, nst, 20)
        for f in H.FIELDS:
            assert np.array_equal(s.get(f), o.get(f)), "%s after %d steps" % (H.FIELD_NAMES[f], nst)
    ao, oo = s.observables(), o.observables()
    assert ao["n_bonds"] == oo["n_bonds"] == d.n_connector_axes * 2
    assert abs(ao["potential_energy"] - oo["potential_energy"]) <= 1e-10 * abs(oo["potential_energy"])
    assert s.device_errors() == 0


def test_connectors_batch_matches_systems_alone():
    mat = K.Material()
    sizes = [40, 150, 64]
    xs = [generate_aggregate(70 + q, n, mat.r) for q, n in enumerate(sizes)]
    vs = [generate_velocities(70 + q, n, 0.2) for q, n in enumerate(sizes)]
    axes = [K.random_unit_axes(len(K.connector_bonds(x, mat.r, mat.d_crit)), 80 + q) for q, x in enumerate(xs)]
    def desc(n, ax):
        d = K.make_desc(n, A.LG_BINARY_SINTER_CONNECTORS, A.LG_HAMAKER_LIMITED, contact=mat.contact(),
                        hamaker=mat.hamaker(), pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r, max_neighbors=160)
        return K.set_connectors(d, 0.5 * mat.k_n, 0.3 * mat.g_n, mat.d_crit, ax)
    batch = System(desc(sum(sizes), np.concatenate(axes)), np.concatenate(xs), np.concatenate(vs), sizes=sizes)
    batch.step(mat.dt, 60, 20)
    off = np.concatenate([[0], np.cumsum(sizes)])
    for q, n in enumerate(sizes):
        alone = System(desc(n, axes[q]), xs[q], vs[q])
        alone.step(mat.dt, 60, 20)
        for f in H.FIELDS:
            assert np.array_equal(alone.get(f), batch.get(f)[off[q]:off[q + 1]]), (q, H.FIELD_NAMES[f])
    assert batch.device_errors() == 0


def test_connectors_snapshot_restore_repeats_steps():
    mat = K.Material()
    x0 = generate_aggregate(90, 500, mat.r)
    v0 = generate_velocities(90, 500, 0.3)
    s = System(_connector_desc(mat, x0, A.LG_PAIRS_VERLET, A.LG_HAMAKER_LIMITED, 90), x0, v0)
    s.step(mat.dt, 20, 20)
    s.snapshot()
    s.step(mat.dt, 40, 20)
    first = [s.get(f) for f in H.FIELDS]
    s.restore()
    s.step(mat.dt, 40, 20)
    for f, a in zip(H.FIELDS, first):
        assert np.array_equal(s.get(f), a), H.FIELD_NAMES[f]


def test_connectors_need_fp64_and_axes():
    mat = K.Material()
    x0 = generate_aggregate(91, 50, mat.r)
    with pytest.raises(Exception):
        System(_connector_desc(mat, x0, A.LG_PAIRS_ALL, A.LG_HAMAKER_NONE, 1, precision=A.LG_PRECISION_MIXED), x0)
    d = _connector_desc(mat, x0, A.LG_PAIRS_ALL, A.LG_HAMAKER_NONE, 1)
    d.n_connector_axes -= 1
    with pytest.raises(Exception):
        System(d, x0)


def test_sintered_known_answer_on_gpu():
    """test/sintered.cpp: a bonded 3x3x3 cube thrown into rigid motion; after 1e6 steps of 1e-13 s
    its radius of gyration and centre displacement match the reference's targets (1 %)."""
    c = KA.sintered_case()
    s = System(c["desc"], c["x0"], c["v0"])
    o0 = s.observables()
    s.step(c["dt"], c["nsteps"])
    m = KA.measured(c, o0, s.observables())
    for k, tv in c["targets"].items():
        assert abs(m[k] - tv) / tv < 0.01, (k, m[k], tv)
    assert s.device_errors() == 0
