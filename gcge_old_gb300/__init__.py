"""GB300-native GCG eigensolver (the GCGE iteration on one GPU).

The product is the C-ABI shared library ``_build/libgcge_cuda.so`` (declared
in ``include/gcge_cuda.h``); this package loads it with ctypes and mirrors
the reference's solver interface (GCGE_SOLVER_Create/Setup/Solve/...,
src/gcge_solver.h:42-60) for Python callers, tests and the benchmark.  There
is no CPU fallback: importing :mod:`gcge_old_gb300.lib` raises if the CUDA
library has not been built.
"""
from .matrices import CSRMatrix  # noqa: F401

__all__ = ["CSRMatrix"]
