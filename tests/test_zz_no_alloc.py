"""lg_observables_noalloc: observables of a state in caller-owned device memory, computed without
allocating device memory (for callers that cannot allocate when they need them: a serving loop
working inside a fixed device-memory budget, a framework whose allocator owns the device memory,
code that must not stall other streams). It is checked against the handle's own
lg_get_observables on the same state, within the tolerance of the other observable tests, on two
calls in a row (its fixed scratch keeps the previous call's contents). This file sorts last so that
a run stopping at the first failure has run every other test before it."""

import numpy as np
import pytest

from libgran_gb300 import _abi as A
from libgran_gb300 import configs as K
from libgran_gb300.system import System, generate_aggregate, generate_velocities

pytestmark = pytest.mark.gpu

TOL = 1e-10
KEYS = ("ke_translational", "ke_rotational", "ke_total", "linear_momentum", "angular_momentum")


def _noalloc(x, v, w, mass, inertia):
    import torch
    dev = torch.device("cuda", 0)
    xt = torch.from_numpy(np.ascontiguousarray(x)).to(dev)
    vt = torch.from_numpy(np.ascontiguousarray(v)).to(dev)
    wt = torch.from_numpy(np.ascontiguousarray(w)).to(dev)
    out = torch.full((A.LG_NOALLOC_OBS,), float("nan"), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    rc = A.lib().lg_observables_noalloc(xt.data_ptr(), vt.data_ptr(), wt.data_ptr(), len(x), mass, inertia,
                                        out.data_ptr(), stream)
    A.check(rc, "lg_observables_noalloc")
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _check(o, ref):
    got = dict(zip(("ke_translational", "ke_rotational", "ke_total", "linear_momentum", "angular_momentum"), o[:5]))
    for k in KEYS:
        assert abs(got[k] - ref[k]) <= TOL * max(abs(ref[k]), 1e-300), (k, got[k], ref[k])
    assert np.allclose(o[5:8], ref["center_of_mass"], rtol=TOL, atol=1e-30)
    assert abs(o[8] - ref["radius_of_gyration"]) <= TOL * ref["radius_of_gyration"]


@pytest.mark.parametrize("n", [1, 1000, 70000])
def test_noalloc_observables_match_handle_observables_twice(n):
    mat = K.Material()
    x0 = generate_aggregate(31, n, mat.r)
    v0 = generate_velocities(31, n, 0.1)
    w0 = generate_velocities(32, n, 1e6)
    d = K.make_desc(n, A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, contact=mat.contact(), sinter=mat.sinter(),
                    hamaker=mat.hamaker(), pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r)
    s = System(d, x0, v0, om0=w0)
    for _ in range(2):  # two calls in a row, the state moving in between
        s.step(mat.dt, 20, 20)
        x, v, w = s.get(A.LG_FIELD_X), s.get(A.LG_FIELD_V), s.get(A.LG_FIELD_OMEGA)
        _check(_noalloc(x, v, w, mat.m, mat.I), s.observables())
