"""libgran_gb300: a GB300-native (sm_103a) engine for libgran's DEM pair-force + integration path.

The CUDA engine lives in ``_lib/liblg_gb300.so`` (built by ``__graft_entry__.build()``); its C ABI
is declared in ``include/libgran_gb300.h``. ``granular`` mirrors libgran's class names and
constructor signatures on top of it; ``system.System`` is the handle-level wrapper.
"""
from . import _abi  # noqa: F401
from .system import System, generate_aggregate, generate_velocities  # noqa: F401

__version__ = "0.1"
