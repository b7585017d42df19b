"""ctypes access to the oracle (oracle/sfport.c, oracle/seqport.c): the
checker the tests compare the GPU against. Test infrastructure only."""
import ctypes
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
PORT = ROOT / "oracle" / "_build" / "libsfport.so"
REF = ROOT / "oracle" / "_ref" / "libcft_ref.so"


class SeqArgs(ctypes.Structure):
    _fields_ = [("a", ctypes.c_void_p), ("b", ctypes.c_void_p), ("c", ctypes.c_void_p),
                ("n", ctypes.c_size_t), ("bank", ctypes.c_void_p),
                ("scratch_in", ctypes.c_void_p), ("scratch_out", ctypes.c_void_p),
                ("deposits", ctypes.c_void_p), ("counts", ctypes.c_void_p),
                ("lane_mask", ctypes.c_void_p), ("lane_flags", ctypes.c_void_p),
                ("idx_a", ctypes.c_void_p), ("idx_b", ctypes.c_void_p),
                ("idx_c", ctypes.c_void_p), ("idx_scratch_in", ctypes.c_void_p),
                ("depth", ctypes.c_uint32), ("flags_out", ctypes.c_uint32),
                ("status_out", ctypes.c_uint32)]


def ptr(x):
    if x is None:
        return None
    return x.ctypes.data


class Oracle:
    def __init__(self):
        if not PORT.exists():
            subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "port"], check=True)
        self.L = ctypes.CDLL(str(PORT))
        self.L.sfp_run.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p] * 4 + [
            ctypes.c_size_t, ctypes.c_uint32, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32)]
        self.L.sfp_run.restype = ctypes.c_int
        self.L.sfp_seq_run.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(SeqArgs)]
        self.L.sfp_seq_run.restype = ctypes.c_int

    def run(self, kind, fmt, op, rnd, a, b, c, n=None, scalar_mask=0):
        """(d, lane_flags, acc) for numpy (n, W) uint32 operands (or None)."""
        if n is None:
            n = a.shape[0]
        d = np.zeros((n, a.shape[1]), np.uint32)
        lf = np.zeros(n, np.uint8)
        acc = ctypes.c_uint32()
        st = self.L.sfp_run(kind, fmt, op, rnd, ptr(a), ptr(b), ptr(c), ptr(d), n, scalar_mask,
                            ptr(lf), ctypes.byref(acc))
        assert st == 0
        return d, lf, acc.value
