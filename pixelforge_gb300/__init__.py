"""pixelforge-gb300: PixelForge's triangle pipeline on a GB300 (sm_103a).

The product is the shared library libpixelforge_gb300.so, a drop-in for the
reference's C99 ``pf*`` API (include/pixelforge.h).  This package builds it
in-tree (``build.py``), binds it with ctypes (``abi.py``) and provides the
seeded workloads used by the benchmark and the tests (``scenes.py``).
"""
from __future__ import annotations

from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libpixelforge_gb300.so"

_lib = None


def load_library(build_if_missing: bool = True):
    """Load libpixelforge_gb300.so through the C ABI binding.

    Raises if the library is missing and cannot be built: there is no CPU
    fallback.
    """
    global _lib
    if _lib is not None:
        return _lib
    from . import abi
    if not LIB_PATH.exists() or build_if_missing:
        from . import build as _b
        _b.build()
    _lib = abi.PixelForgeLib(str(LIB_PATH))
    return _lib
