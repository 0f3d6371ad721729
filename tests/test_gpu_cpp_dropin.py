"""The C++ drop-in headers (include/libgran_gb300/libgran/...): a libgran-style driver with the
template composition of libgran's test/hamaker.cpp and test/hamaker_neighbor.cpp, compiled against
the drop-in headers and the engine library, must hit libgran's own 1 % targets."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("dropin") / "dropin_hamaker")
    lib = os.path.join(ROOT, "libgran_gb300", "_lib")
    cmd = ["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include", "libgran_gb300"),
           "-I/usr/local/cuda/include", "-o", out, os.path.join(ROOT, "tests", "cpp", "dropin_hamaker.cpp"),
           "-L" + lib, "-llg_gb300", "-Wl,-rpath," + lib]
    subprocess.check_call(cmd)
    return out


@pytest.mark.parametrize("mode", ["all_pairs", "neighbor"])
def test_dropin_driver_hits_libgran_targets(driver, mode):
    args = [driver] + (["neighbor"] if mode == "neighbor" else ["all", "1000"])
    r = subprocess.run(args, capture_output=True, text=True, timeout=600)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stdout + r.stderr
