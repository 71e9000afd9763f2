"""Loads the in-tree CUDA library.  There is no CPU fallback: if the library is
missing or cannot be loaded, every call raises."""
from __future__ import annotations

import ctypes
import os

from .build import LIB

_lib = None


class GAError(RuntimeError):
    pass


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise GAError(f"CUDA library not built: {LIB} (run graphaligner_gb300.build.build())")
        _lib = ctypes.CDLL(LIB)
        _lib.ga_last_error.restype = ctypes.c_char_p
        _lib.ga_version.restype = ctypes.c_char_p
    return _lib


def check(rc: int):
    if rc != 0:
        raise GAError(f"graphaligner_gb300 error {rc}: {lib().ga_last_error().decode()}")
    return rc
