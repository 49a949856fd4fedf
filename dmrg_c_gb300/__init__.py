"""GB300-native eigensolver hot path of dmrg_C.

The product is the C-ABI library ``libdmrg_gb300.so`` (CUDA kernels for sm_103a + host
orchestration in C++), exporting the reference's own entry points.  This package holds
its sources (``csrc/``), the build recipe, and Python bindings used by tests and the
benchmark.
"""
from . import abi  # noqa: F401

__all__ = ["abi", "lib", "build"]
