"""macaw_gb300 -- GB300-native particle-tracking hot path of MaCaw.

The compute path is the CUDA library libmacaw_gb300.so (sm_103a kernels
behind the C ABI in include/macaw_gb300.h); this package loads it through
ctypes on first use of Tracker, lib or LIB_PATH.  There is no CPU fallback:
without the library, that first use fails.  macaw_gb300.problems (the
synthetic problem generators) can run on another compiled copy of the
generator sources without loading the CUDA library.
"""
from .problems import Problem, cube_problem, lattice_problem  # noqa: F401

__all__ = ["Tracker", "Problem", "cube_problem", "lattice_problem", "MCError", "LIB_PATH", "lib"]


def __getattr__(name):
    if name in ("LIB_PATH", "MCError", "lib"):
        from . import _lib
        return getattr(_lib, name)
    if name == "Tracker":
        from .tracker import Tracker
        return Tracker
    raise AttributeError(name)
