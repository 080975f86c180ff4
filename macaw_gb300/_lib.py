"""ctypes view of the C ABI declared in include/macaw_gb300.h.

Loads the in-tree libmacaw_gb300.so (rebuilding it first if it is missing
or older than its sources).
There is no fallback: if the library cannot be built or loaded, importing
this module raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build
from ._abi import *  # noqa: F401,F403
from ._abi import SIGNATURES


def _load() -> C.CDLL:
    path = _build.build()  # no-op when the library is newer than its sources
    lib = C.CDLL(str(path))
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


lib = _load()
LIB_PATH = Path(_build.LIB)


def ptr(a: np.ndarray | None) -> C.c_void_p | None:
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "arrays passed to the C ABI must be contiguous"
    return C.c_void_p(a.ctypes.data)


class MCError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code
