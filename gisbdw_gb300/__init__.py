"""gisbdw_gb300 — GB300-native exact treedepth solvers.

The compute path is the native library libgtd.so (hand-written sm_103a
kernels behind the C ABI in include/gtd.h). This package holds its ctypes
binding (``_lib``), the reference-shaped solver classes (``treedepth``), the
seeded graph generators and text IO (``graphs``) and the build script
(``build``).
"""
from . import graphs
from ._lib import GtdError, InvalidArgument, DeadlineExceeded, Handle
from .treedepth import BnBGPU, DynamicGPU, Result, solve_exact

__all__ = ["graphs", "GtdError", "InvalidArgument", "DeadlineExceeded", "Handle",
           "DynamicGPU", "BnBGPU", "Result", "solve_exact"]
