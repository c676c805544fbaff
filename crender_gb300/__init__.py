"""crender_gb300 — GB300-native render hot path for CRender.

The product is libcrg.so (crender_gb300/csrc, built for sm_103a): BVH build,
closest/any-hit traversal and path-traced rendering behind the C ABI of
include/crg.h.  This Python package only loads that library (ctypes) and
generates seeded synthetic workloads; it never computes a ray or a sample.
Loading fails loudly when the library has not been built: there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _abi

ROOT = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(ROOT, "_build", "libcrg.so")

_lib = None


def load() -> C.CDLL:
    """Loads libcrg.so and binds every entry point declared in include/crg.h."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"libcrg.so not found at {LIB_PATH}: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)"
            )
        _lib = _abi.bind(C.CDLL(LIB_PATH), _abi.CRG_SIGNATURES)
    return _lib


class CrgError(RuntimeError):
    pass


def check(status: int, ctx=None):
    if status != 0:
        msg = _abi.STATUS.get(status, str(status))
        if ctx is not None and _lib is not None:
            msg += ": " + _lib.crg_last_error_string(ctx).decode(errors="replace")
        raise CrgError(msg)
