"""mdsctk_gb300 -- GB300 (sm_103a) implementation of the MDSCTK hot path.

The compute lives in libmdsgpu (CUDA kernels behind the C ABI of
include/mdsgpu.h); this package holds its ctypes binding, the Python mirror
of the tools (``Context``), the build recipe and the seeded synthetic
workload generators.
"""
from ._lib import LIB_PATH, MdsError, lib  # noqa: F401
from .api import Context  # noqa: F401

__all__ = ["Context", "MdsError", "lib", "LIB_PATH"]
