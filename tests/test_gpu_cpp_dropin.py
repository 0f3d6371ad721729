"""The C++ drop-in headers (include/libgran_gb300/libgran/...): a libgran-style driver with the
template composition of libgran's test/hamaker.cpp and test/hamaker_neighbor.cpp, compiled against
the drop-in headers and the engine library. A 20000-step run must match the oracle's end state; the
full 3e6-step run (libgran's own 1 % targets; about 2 minutes per mode on a GB300, where FP64 on a
19-particle system is latency-bound at about 37 us a step) runs when LG_LONG_TESTS=1."""
import os
import subprocess

import pytest

import known_answer as KA
from oracle import oracle as O

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("dropin") / "dropin_hamaker")
    lib = os.path.join(ROOT, "libgran_gb300", "_lib")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include", "libgran_gb300"),
           "-I/usr/local/cuda/include", "-o", out, os.path.join(ROOT, "tests", "cpp", "dropin_hamaker.cpp"),
           "-L" + lib, "-llg_gb300", "-Wl,-rpath," + lib]
    subprocess.check_call(cmd)
    return out


@pytest.mark.parametrize("mode", ["all", "neighbor"])
def test_dropin_driver_matches_oracle(driver, mode):
    steps = 20000
    r = subprocess.run([driver, mode, "1000", str(steps)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    vals = dict(zip(("momentum", "ke", "rg"), [float(t) for t in r.stdout.split()[1::2]]))
    c = KA.hamaker_case(mode == "neighbor")
    o = O.OracleSystem(c["desc"], c["x0"], c["v0"])
    o.step(c["dt"], steps, c["rebuild"])
    ob = o.observables()
    assert abs(vals["ke"] - ob["ke_total"]) <= 1e-6 * ob["ke_total"]
    assert abs(vals["momentum"] - ob["linear_momentum"]) <= 1e-6 * ob["linear_momentum"]
    assert abs(vals["rg"] - ob["radius_of_gyration"]) <= 1e-6 * ob["radius_of_gyration"]


@pytest.mark.skipif(os.environ.get("LG_LONG_TESTS") != "1", reason="full-length known-answer run (LG_LONG_TESTS=1)")
@pytest.mark.parametrize("mode", ["all", "neighbor"])
def test_dropin_driver_hits_libgran_targets(driver, mode):
    r = subprocess.run([driver, mode, "1000"], capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.fixture(scope="module")
def sintered_driver(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("dropin") / "dropin_sintered")
    lib = os.path.join(ROOT, "libgran_gb300", "_lib")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include", "libgran_gb300"),
           "-I/usr/local/cuda/include", "-o", out, os.path.join(ROOT, "tests", "cpp", "dropin_sintered.cpp"),
           "-L" + lib, "-llg_gb300", "-Wl,-rpath," + lib]
    subprocess.check_call(cmd)
    return out


def test_dropin_sintered_driver_hits_libgran_targets(sintered_driver):
    """libgran's test/sintered.cpp composition (sinter_functor, sinter_step_handler alias, the
    reference's own generator of connector axes) on the drop-in headers, full 1e6-step run."""
    r = subprocess.run([sintered_driver], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout + r.stderr
    vals = dict(zip(("rg", "cd"), [float(t) for t in r.stdout.split()[1::2]]))
    c = KA.sintered_case()
    assert abs(vals["rg"] - c["targets"]["radius_of_gyration"]) / c["targets"]["radius_of_gyration"] < 0.01
    assert abs(vals["cd"] - c["targets"]["center_displacement"]) / c["targets"]["center_displacement"] < 0.01
