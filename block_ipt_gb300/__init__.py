"""GB300-native block IPT + Davidson eigensolver.

The solver is libipt_gb300.so (CUDA for sm_103a behind the C ABI of
include/ipt_cuda.h and include/ipt_block.h); this package builds it, binds it
through ctypes and provides the seeded workload generators.
"""
from . import _lib  # noqa: F401
from ._lib import IPTError, load  # noqa: F401

__all__ = ["IPTError", "load", "api", "workloads", "build"]
