import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TESTS = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running known-answer simulation")


def _ensure_built():
    so = os.path.join(ROOT, "libgran_gb300", "_lib", "liblg_gb300.so")
    oso = os.path.join(ROOT, "oracle", "liblg_oracle.so")
    if not (os.path.exists(so) and os.path.exists(oso)):
        import __graft_entry__
        __graft_entry__.build()


_ensure_built()


@pytest.fixture(scope="session")
def gpu_available():
    from libgran_gb300 import _abi as A
    import ctypes as C
    c = C.c_int()
    A.lib().lg_device_count(C.byref(c))
    return c.value > 0
