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

    def run_parallel(self, kind, fmt, op, rnd, a, b, c, threads=None, chunk=1 << 15):
        """run() over whole arrays split into chunks across host threads
        (ctypes releases the GIL inside each call): (d, lane_flags, acc).
        Elementwise calls are independent per element, so the chunking
        changes nothing in the results."""
        import os
        from concurrent.futures import ThreadPoolExecutor
        n = a.shape[0]
        d = np.zeros((n, a.shape[1]), np.uint32)
        lf = np.zeros(n, np.uint8)
        accs = []

        def one(s):
            e = min(n, s + chunk)
            acc = ctypes.c_uint32()
            sl = [None if x is None else np.ascontiguousarray(x[s:e]) for x in (a, b, c)]
            dd = np.zeros((e - s, a.shape[1]), np.uint32)
            ll = np.zeros(e - s, np.uint8)
            st = self.L.sfp_run(kind, fmt, op, rnd, ptr(sl[0]), ptr(sl[1]), ptr(sl[2]), ptr(dd),
                                e - s, 0, ptr(ll), ctypes.byref(acc))
            assert st == 0
            d[s:e] = dd
            lf[s:e] = ll
            return acc.value
        with ThreadPoolExecutor(threads or os.cpu_count() or 1) as ex:
            accs = list(ex.map(one, range(0, n, chunk)))
        acc = 0
        for x in accs:
            acc |= x
        return d, lf, acc

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
