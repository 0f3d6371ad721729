"""Shared helpers of the parity tests."""
import glob
import os

import numpy as np

from libgran_gb300 import _abi as A

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIELDS = [A.LG_FIELD_X, A.LG_FIELD_V, A.LG_FIELD_THETA, A.LG_FIELD_OMEGA, A.LG_FIELD_A, A.LG_FIELD_ALPHA]
FIELD_NAMES = {A.LG_FIELD_X: "x", A.LG_FIELD_V: "v", A.LG_FIELD_THETA: "theta", A.LG_FIELD_OMEGA: "omega",
               A.LG_FIELD_A: "a", A.LG_FIELD_ALPHA: "alpha"}


def golden_files():
    return sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


def golden_case(name):
    import golden_cases
    for c in golden_cases.cases():
        if c["name"] == name:
            return c
    raise KeyError(name)


def rel_err(a, b):
    """Normwise relative error: max |a - b| over the field divided by max |b| over the field."""
    scale = np.abs(b).max()
    if scale == 0.0:
        return float(np.abs(a - b).max())
    return float(np.abs(a - b).max() / scale)


def run_checkpoints(sysobj, case, golden, check, rebuild=None):
    """Step sysobj through the golden checkpoints and call check(field, step, got, want)."""
    done = 0
    rb = case.get("rebuild", 0) if rebuild is None else rebuild
    for cp in golden["checkpoints"]:
        if cp > done:
            sysobj.step(case["dt"], int(cp - done), rb)
            done = int(cp)
        for f in FIELDS:
            check(f, int(cp), sysobj.get(f), golden["f%d_s%d" % (f, cp)])
