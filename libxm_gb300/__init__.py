"""libxm-gb300: the libxm block-tensor API on hand-written sm_103a kernels.

The product is the shared library libxm_gb300/lib/libxmgb.so (C ABI,
include/xm.h + include/xmg.h).  This package builds it and offers a thin
ctypes binding for Python callers; it has no compute path of its own.
"""
import os

from . import api  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libxmgb.so")
_LIB = None


def build(verbose=False):
    from .builder import build as _build
    return _build(verbose=verbose)


def load():
    """Load the engine library.  Raises when it has not been built: there is
    no fallback implementation."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libxm-gb300 engine library missing (%s); "
                               "run libxm_gb300.build()" % LIB_PATH)
        _LIB = api.Lib(LIB_PATH)
    return _LIB
