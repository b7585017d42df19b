"""The reference's own Python binding (bindings/python/cftmpfr) loaded
against this library through its CFT_LIB override, as INTEGRATION.md tells
a user to do: its _bind() declares every prototype it uses (about 90
symbols, cftmpfr/_lib.py:181-372) and its _audit() checks the ABI version
and every opcode and format number against this library's names
(cftmpfr/_lib.py:378-425). A missing export or a renumbered enum fails
here. Runs in a child process so the binding's module state stays out of
this one; skipped where the reference tree is absent."""
import os
import subprocess
import sys

import pytest

from cftgb import _lib
from refpath import reference_root

CODE = r"""
import ctypes
from cftmpfr import _lib as B
lib = B.lib()                       # binds and audits, or raises
assert lib.cft_abi_version() == (0 << 16) | 18, hex(lib.cft_abi_version())
# a call the binding makes before any device exists: the status words
assert B.lib().cft_strerror(0) == b"ok"
h = ctypes.c_void_p()
st = lib.cft_open(None, 0, ctypes.byref(h))
print("bound", st)
"""


def test_reference_binding_binds_and_audits_this_library():
    ref = reference_root()
    if ref is None or not (ref / "bindings" / "python" / "cftmpfr" / "_lib.py").exists():
        pytest.skip("the reference tree (its Python binding) is not present")
    so = _lib.lib()._name
    env = dict(os.environ, CFT_LIB=str(so), PYTHONPATH=str(ref / "bindings" / "python"))
    p = subprocess.run([sys.executable, "-c", CODE], env=env, capture_output=True, text=True,
                       timeout=120)
    assert p.returncode == 0, p.stderr[-2000:]
    status = int(p.stdout.split()[-1])
    # cft_open reaches this library: CFT_OK on a GPU host, CFT_ERR_NO_DEVICE without one
    assert status in (0, 3), p.stdout
