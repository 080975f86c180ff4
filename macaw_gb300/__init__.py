"""macaw_gb300 -- GB300-native particle-tracking hot path of MaCaw.

The compute path is the CUDA library libmacaw_gb300.so (sm_103a kernels
behind the C ABI in include/macaw_gb300.h); this package loads it through
ctypes.  There is no CPU fallback: without the library, import fails.
"""
from ._lib import LIB_PATH, MCError, lib  # noqa: F401
from .problems import Problem, cube_problem, lattice_problem  # noqa: F401
from .tracker import Tracker  # noqa: F401

__all__ = ["Tracker", "Problem", "cube_problem", "lattice_problem", "MCError", "LIB_PATH"]
