"""Serving loop on the GPU: requests of different sizes arrive while others run, occupy slots of one
batch and advance in the same launches, and each result is the same as the request run alone."""
import numpy as np
import pytest

from libgran_gb300 import _abi as A
from libgran_gb300 import configs as K
from libgran_gb300.serving import Server
from libgran_gb300.system import System, generate_aggregate, generate_velocities

pytestmark = pytest.mark.gpu


def _tmpl(prec=A.LG_PRECISION_MIXED):
    mat = K.Material()
    return mat, K.make_desc(1, A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, contact=mat.contact(), sinter=mat.sinter(),
                            hamaker=mat.hamaker(), pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r, precision=prec,
                            max_neighbors=96)


def _req(seed, n):
    mat = K.Material()
    return generate_aggregate(seed, n, mat.r), generate_velocities(seed, n, 0.1)


@pytest.mark.parametrize("prec", [A.LG_PRECISION_MIXED, A.LG_PRECISION_FP64], ids=["mixed", "fp64"])
def test_results_in_the_mix_equal_results_alone(prec):
    mat, d = _tmpl(prec)
    sizes = [64, 700, 150, 2000, 90, 333]
    steps = [200, 60, 140, 100, 40, 80]
    s = Server(d, budget_bytes=8 << 30, dt=mat.dt)
    reqs = []
    arrivals = {0: [0, 1, 2, 3], 1: [4], 2: [5]}  # tick -> requests submitted before that tick
    tick = 0
    busy = 0
    while True:
        for q in arrivals.get(tick, []):
            x0, v0 = _req(500 + q, sizes[q])
            reqs.append((q, s.submit(x0, v0, steps[q])))
        a, qd, _ = s.tick()
        busy = max(busy, s.stats()["slots_busy"])
        tick += 1
        if tick > 5 and a == 0 and qd == 0:
            break
        assert tick < 1000
    assert busy >= 4  # requests shared the batch's launches
    for q, rid in reqs:
        p = s.poll(rid, want_x=True)
        assert p["state"] == A.LG_REQ_DONE, p["error"]
        x0, v0 = _req(500 + q, sizes[q])
        dd = K.make_desc(sizes[q], d.binary_model, d.hamaker_model, contact=d.contact, sinter=d.sinter,
                         hamaker=d.hamaker, pairs=d.pairs, r_verlet=d.r_verlet, precision=prec, max_neighbors=96)
        alone = System(dd, x0, v0)
        if prec == A.LG_PRECISION_MIXED:  # the server's Hamaker slicing gives the batch's bits
            alone.set_step_shape(0, s.stats()["hamaker_slices"], 0)
        alone.step(mat.dt, steps[q], 20)
        assert np.array_equal(p["x"], alone.get(A.LG_FIELD_X)), q
        ao = alone.observables()
        assert abs(ao["ke_total"] - p["obs"]["ke_total"]) <= 1e-12 * ao["ke_total"]
    st = s.stats()
    assert st["completed"] == len(sizes) and st["failed"] == 0
    assert st["p99_latency_ms"] >= st["p50_latency_ms"] > 0


def test_slots_bound_resident_requests():
    """Two slots: six requests of 1500 monomers run two at a time and all complete; the slots and
    the standalone handles being prepared stay within the budget."""
    mat, d = _tmpl()
    s = Server(d, budget_bytes=16 << 30, dt=mat.dt)
    s.set_slots([2048, 2048])
    ids = [s.submit(*_req(900 + q, 1500), 100) for q in range(6)]
    peak_active = 0
    while True:
        a, qd, _ = s.tick()
        st = s.stats()
        assert st["used_bytes"] <= st["budget_bytes"]
        assert st["slots_busy"] <= 2
        peak_active = max(peak_active, a)
        if a == 0 and qd == 0:
            break
    assert peak_active == 2
    assert all(s.poll(r)["state"] == A.LG_REQ_DONE for r in ids)
    assert s.stats()["completed"] == 6


def test_cancel_running_request_frees_its_slot():
    mat, d = _tmpl()
    s = Server(d, budget_bytes=4 << 30, dt=mat.dt)
    s.set_slots([1024])
    r1 = s.submit(*_req(1, 500), 10000)
    s.tick()
    assert s.stats()["slots_busy"] == 1
    r2 = s.submit(*_req(2, 600), 40)
    s.tick()
    assert s.poll(r2)["state"] == A.LG_REQ_QUEUED  # the only slot is taken
    s.cancel(r1)
    assert s.poll(r1)["state"] == A.LG_REQ_CANCELLED
    assert s.stats()["slots_busy"] == 0
    for _ in range(20):
        a, qd, _ = s.tick()
        if a == 0 and qd == 0:
            break
    p = s.poll(r2, want_x=True)
    assert p["state"] == A.LG_REQ_DONE, p["error"]
    # the slot's previous occupant left nothing behind: the result equals the request alone
    x0, v0 = _req(2, 600)
    dd = K.make_desc(600, d.binary_model, d.hamaker_model, contact=d.contact, sinter=d.sinter, hamaker=d.hamaker,
                     pairs=d.pairs, r_verlet=d.r_verlet, precision=d.precision, max_neighbors=96)
    alone = System(dd, x0, v0)
    alone.set_step_shape(0, s.stats()["hamaker_slices"], 0)
    alone.step(mat.dt, 40, 20)
    assert np.array_equal(p["x"], alone.get(A.LG_FIELD_X))
