"""GB300-native ILU0-preconditioned BiCGSTAB for 3x3-block BSR systems.

The solver runs in libgbilu.so (C ABI in include/gbilu.h, CUDA kernels for
sm_103a in fpga_gb300/csrc/). This package holds its build script, the ctypes
binding used by tests and the benchmark, the seeded matrix generator and a
torch.autograd wrapper around the adjoint.
"""
from .native import GbIlu, GbIluError, load, status_string  # noqa: F401
from . import synth  # noqa: F401

__all__ = ["GbIlu", "GbIluError", "load", "status_string", "synth"]
