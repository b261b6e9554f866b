"""GB300-native implementation of PLUTO 4.3's unsplit ideal-MHD step.

The compute path is libpluto_gb300.so (hand-written sm_103a CUDA kernels
behind the C ABI declared in include/pluto_gb300.h); this package is the
thin host-side mirror of PLUTO's AdvanceStep interface over that ABI.
"""
from .solver import Solver, make_config  # noqa: F401
from . import _lib  # noqa: F401

__all__ = ["Solver", "make_config"]
