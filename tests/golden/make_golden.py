"""Generate the golden fixtures of tests/golden/ from the reference harness.

The harness compiles libgran's own functor headers (unmodified, from the libgran source tree) on
the system loop of the oracle; running it needs that tree and is done on the development machine.
The fixtures (initial state, states after a few step counts, springs and bonds) travel with the
repository so that the GPU test machine can check the engine against values produced by
libgran's code. Usage: python tests/golden/make_golden.py [libgran_root] (default: $LIBGRAN_ROOT,
else the tree oracle.libgran_root() finds)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from libgran_gb300 import _abi as A  # noqa: E402
from libgran_gb300 import configs as K  # noqa: E402
from libgran_gb300.system import generate_aggregate, generate_velocities  # noqa: E402
from oracle import oracle as O  # noqa: E402
import golden_cases  # noqa: E402

FIELDS = [A.LG_FIELD_X, A.LG_FIELD_V, A.LG_FIELD_THETA, A.LG_FIELD_OMEGA, A.LG_FIELD_A, A.LG_FIELD_ALPHA]


def run_case(c):
    r = O.RefHarnessSystem(c["desc"], c["x0"], c["v0"], facets=c.get("facets"), neck=c.get("neck"))
    out = {"x0": c["x0"], "v0": c["v0"], "checkpoints": np.array(c["checkpoints"], dtype=np.int64)}
    done = 0
    for cp in c["checkpoints"]:
        r.step(c["dt"], cp - done, c.get("rebuild", 0)) if cp > done else None
        done = cp
        for f in FIELDS:
            out["f%d_s%d" % (f, cp)] = r.get(f)
    pairs = np.array(c.get("spring_pairs", []), dtype=np.int64).reshape(-1, 2)
    out["spring_pairs"] = pairs
    out["springs"] = np.array([r.springs(i, j) for i, j in pairs]).reshape(-1, 9)
    out["bonds"] = r.bonds()
    if c.get("facets"):
        out["facet_vertices"] = np.array([r.facet_vertices(f) for f in range(len(c["facets"]))])
    return out


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else O.libgran_root()
    if not root or O.build_ref(root) is None:
        sys.exit("make_golden: no libgran source tree (pass its path or set LIBGRAN_ROOT)")
    for c in golden_cases.cases():
        out = run_case(c)
        path = os.path.join(HERE, c["name"] + ".npz")
        np.savez_compressed(path, **out)
        print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
