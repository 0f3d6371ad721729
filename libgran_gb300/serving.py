"""Python wrapper of the serving loop (lg_server_* in include/libgran_gb300.h)."""
import ctypes as C

import numpy as np

from . import _abi as A


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Server:
    """Continuous-batching server: submit requests at any time, call tick() to make progress; resident
    requests share slots of one batch and advance in the same launches."""

    def __init__(self, template_desc, budget_bytes, dt, rebuild_every=20, device=0):
        self.tmpl = template_desc
        h = C.c_void_p()
        A.check(A.lib().lg_server_create(C.byref(template_desc), int(budget_bytes), int(rebuild_every), float(dt),
                                         int(device), C.byref(h)), "lg_server_create")
        self.h = h
        self.sizes = {}

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            A.lib().lg_server_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_slots(self, capacities):
        """Slot capacities of the server's batch (before the first admission)."""
        c = np.ascontiguousarray(capacities, dtype=np.int64)
        A.check(A.lib().lg_server_set_slots(self.h, c.ctypes.data_as(C.POINTER(C.c_int64)), len(c)),
                "lg_server_set_slots")

    def estimate_bytes(self, n):
        return A.lib().lg_estimate_device_bytes(C.byref(self.tmpl), int(n))

    def submit(self, x0, v0, nsteps):
        x0 = np.ascontiguousarray(x0, dtype=np.float64).reshape(-1, 3)
        v0 = None if v0 is None else np.ascontiguousarray(v0, dtype=np.float64).reshape(-1, 3)
        rid = C.c_int64()
        A.check(A.lib().lg_server_submit(self.h, len(x0), _dp(x0), None if v0 is None else _dp(v0), int(nsteps),
                                         C.byref(rid)), "lg_server_submit")
        self.sizes[rid.value] = len(x0)
        return rid.value

    def cancel(self, rid):
        A.check(A.lib().lg_server_cancel(self.h, int(rid)), "lg_server_cancel")

    def tick(self):
        a, q, r = C.c_int32(), C.c_int32(), C.c_int32()
        A.check(A.lib().lg_server_tick(self.h, C.byref(a), C.byref(q), C.byref(r)), "lg_server_tick")
        return a.value, q.value, r.value

    def poll(self, rid, want_x=False):
        st = C.c_int32()
        o = A.lg_observables()
        lat = C.c_double()
        x = np.zeros((self.sizes[rid], 3)) if want_x else None
        A.check(A.lib().lg_server_poll(self.h, int(rid), C.byref(st), C.byref(o), None if x is None else _dp(x),
                                       C.byref(lat)), "lg_server_poll")
        err = A.lib().lg_last_error().decode(errors="replace") if st.value == A.LG_REQ_FAILED else ""
        return {"state": st.value, "obs": o.as_dict() if st.value == A.LG_REQ_DONE else None, "x": x,
                "latency_ms": lat.value, "error": err}

    def release(self, rid):
        A.check(A.lib().lg_server_release(self.h, int(rid)), "lg_server_release")
        self.sizes.pop(rid, None)

    def stats(self):
        st = A.lg_server_stats()
        A.check(A.lib().lg_server_get_stats(self.h, C.byref(st)), "lg_server_get_stats")
        return {k: getattr(st, k) for k, _ in st._fields_}

    def inject_alloc_failures(self, count):
        A.check(A.lib().lg_server_inject_alloc_failures(self.h, int(count)), "lg_server_inject_alloc_failures")
