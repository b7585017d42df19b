"""cftgb - Python access to libcft_gb300, the GB300 backend for cft-fp256's
batched elementwise softfloat path and sequencer.

The binding mirrors the reference's ctypes layer (bindings/python/cftmpfr/
_lib.py): the same C calls, the same argument meanings and errors. Compute
happens only in the CUDA library; this package moves pointers.
"""
from . import _lib  # noqa: F401
from ._lib import (CftError, FMT_NAMES, ESZ, lib, open_device, close_device, run,  # noqa: F401
                   div, sqrt, run_ex, get_caps, supports)

__all__ = ["CftError", "FMT_NAMES", "ESZ", "lib", "open_device", "close_device", "run", "div",
           "sqrt", "run_ex", "get_caps", "supports"]
