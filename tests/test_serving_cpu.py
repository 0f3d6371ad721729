"""Serving loop host logic without a GPU: request validation, slot configuration against the budget,
injected allocation failure, cancellation (no request here ever reaches a device)."""
import numpy as np

from libgran_gb300 import _abi as A
from libgran_gb300 import configs as K
from libgran_gb300.serving import Server


def _tmpl():
    mat = K.Material()
    return mat, K.make_desc(1, A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, contact=mat.contact(), sinter=mat.sinter(),
                            hamaker=mat.hamaker(), pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r,
                            precision=A.LG_PRECISION_MIXED)


def test_malformed_and_oversized_requests_are_rejected():
    mat, d = _tmpl()
    s = Server(d, budget_bytes=64 << 20, dt=mat.dt)
    L = A.lib()
    x = np.zeros((10, 3))
    for n, steps, arr in ((0, 10, x), (10, 0, x), (10, 10, np.full((10, 3), np.nan))):
        rid = A.C.c_int64()
        rc = L.lg_server_submit(s.h, n, arr.ctypes.data_as(A.C.POINTER(A.C.c_double)), None, steps, A.C.byref(rid))
        assert rc == A.LG_E_INVALID and b"malformed" in L.lg_last_error()
    big = s.estimate_bytes(10 ** 7)
    assert big > 64 << 20
    rid = A.C.c_int64()
    xb = np.zeros((10 ** 6, 3))
    rc = L.lg_server_submit(s.h, 10 ** 6, xb.ctypes.data_as(A.C.POINTER(A.C.c_double)), None, 10, A.C.byref(rid))
    assert rc == A.LG_E_NOMEM
    assert s.stats()["rejected"] == 1


def test_injected_allocation_failure_marks_request_failed():
    mat, d = _tmpl()
    s = Server(d, budget_bytes=1 << 30, dt=mat.dt)
    s.inject_alloc_failures(1)
    rid = s.submit(np.zeros((8, 3)), None, 40)
    s.tick()
    p = s.poll(rid)
    assert p["state"] == A.LG_REQ_FAILED
    assert "injected" in p["error"]
    st = s.stats()
    assert st["failed"] == 1 and st["used_bytes"] == 0


def test_cancel_queued_request_and_estimates():
    mat, d = _tmpl()
    s = Server(d, budget_bytes=1 << 30, dt=mat.dt)
    rid = s.submit(np.zeros((8, 3)), None, 40)
    s.cancel(rid)
    assert s.poll(rid)["state"] == A.LG_REQ_CANCELLED
    assert s.stats()["queued"] == 0 and s.stats()["cancelled"] == 1
    e = [s.estimate_bytes(n) for n in (64, 512, 8192)]
    assert e[0] < e[1] < e[2]


def test_slot_configuration():
    """Default slots shrink to fit the budget; explicit slots must fit it; a request larger than the
    largest slot is refused at submission."""
    mat, d = _tmpl()
    big = Server(d, budget_bytes=150 * 10 ** 9, dt=mat.dt).stats()
    small = Server(d, budget_bytes=256 << 20, dt=mat.dt).stats()
    assert big["slots"] == 56 and big["slot_particles"] == 8 * (128 + 256 + 512 + 1024 + 2048 + 4096 + 8192)
    assert 1 <= small["slots"] < big["slots"] and small["slot_particles"] < big["slot_particles"]
    s = Server(d, budget_bytes=1 << 30, dt=mat.dt)
    try:
        s.set_slots([10 ** 7])
        assert False, "slots beyond the budget were accepted"
    except A.LgError as e:
        assert "budget" in str(e)
    s.set_slots([300, 100])
    st = s.stats()
    assert st["slots"] == 2 and st["slot_particles"] == 400 and st["slots_busy"] == 0
    rid = A.C.c_int64()
    x = np.zeros((301, 3))
    rc = A.lib().lg_server_submit(s.h, 301, x.ctypes.data_as(A.C.POINTER(A.C.c_double)), None, 20, A.C.byref(rid))
    assert rc == A.LG_E_NOMEM and b"largest slot" in A.lib().lg_last_error()
