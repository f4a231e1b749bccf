"""portblas_gb300 — GB300-native (sm_103a) drop-in for portBLAS's hot path.

``blas`` mirrors portBLAS's ``blas::`` functions for GEMM, GEMV, the BLAS-1
reductions and ``extension::_reduction`` over device pointers; every call
runs hand-written CUDA kernels in ``lib/libgbblas.so`` through its C ABI.
"""
from . import blas
from .blas import SB_Handle, extension

__all__ = ["blas", "SB_Handle", "extension"]
