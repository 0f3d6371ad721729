"""bench.py's inputs that come from committed files: the DRAM traffic of the roofline's kernels is
read from the ncu summaries in profiles/, and each summary names the command that produced it."""
import os
import re
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_roofline_traffic_comes_from_the_profile_summaries():
    for tag in ("forces_mixed_c1", "forces_compact_fp64_c1"):
        t = bench.read_profile_traffic(tag)
        assert t is not None and t > 1e6, tag
    assert bench.read_profile_traffic("no_such_kernel") is None


def test_profile_summaries_give_their_commands():
    d = os.path.join(ROOT, "profiles")
    names = sorted(f for f in os.listdir(d) if f.endswith(".md"))
    assert names
    for f in names:
        text = open(os.path.join(d, f)).read()
        assert "ncu " in text and "--clock-control none" in text, f
        for cmd in re.findall(r"^\s+ncu .*$", text, flags=re.M):
            assert "--clock-control none" in cmd, (f, cmd)


def test_reference_arm_inputs_load_no_engine_library():
    """The reference arm's inputs come from the oracle alone: in a fresh process, building them maps
    the oracle's library and no library of the engine."""
    import subprocess
    code = ("import sys; sys.path.insert(0, %r); import bench; bench.N_PART = 512; "
            "from oracle import oracle as O; bench.workload_state(O); print(bench.repo_native_libraries())" % ROOT)
    out = subprocess.check_output([sys.executable, "-c", code], cwd=ROOT, text=True).strip().splitlines()[-1]
    libs = eval(out)
    assert libs == ["oracle/liblg_oracle.so"], libs
