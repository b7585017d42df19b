"""Segment lines of an open certificate (the reference's segmented runner,
host/tools/segrun.c, and its certificate format, docs/CERTIFICATES.md):
a program run segment after segment, each run's scratch-out block fed back
as the next run's scratch-in, and for every segment the tagged SHA-256 of
the lane-major state before and after it, the run's flags and its STATUS:

    segment K start <sha256> end <sha256> flags F status S

The state hash is SHA-256 over the tag "cft-certificate 1 state" with its
NUL, then the state's bytes. Runs go through cft_program_run_ex, so a
GPU run writes the lines a reference run of the same program, bank and
state writes."""
import ctypes
import hashlib

import numpy as np

from . import _lib

TAG = b"cft-certificate 1 state\0"


def state_hash(state):
    return hashlib.sha256(TAG + np.ascontiguousarray(state).tobytes()).hexdigest()


def segment_lines(h, image, bank, state0, segments, a=None):
    """The certificate's segment lines for `segments` runs of `image` (a
    .cftp as bytes or a uint8 array) from the lane-major scratch block
    state0 ((lanes * n_scratch_out, W) uint32), with the constant bank
    `bank` (bytes or uint8 array, or None) and r0 stream `a` (default +0).
    Returns (lines, final state)."""
    L = _lib.lib()
    img = np.frombuffer(bytes(image), np.uint8).copy()
    prog = ctypes.c_void_p()
    _lib.check(L.cft_program_load(h, img.ctypes.data, img.size, ctypes.byref(prog)),
               "cft_program_load")
    try:
        state = np.ascontiguousarray(state0, np.uint32).copy()
        W = state.shape[1]
        words = np.frombuffer(img[:32].tobytes(), "<u4")
        slots = int(words[7]) >> 16 if int(words[6]) & 2 else 0
        n = state.shape[0] // max(1, slots)
        a = np.zeros((n, W), np.uint32) if a is None else np.ascontiguousarray(a, np.uint32)
        bk = None if bank is None else np.frombuffer(bytes(bank), np.uint8).copy()
        lines = []
        for k in range(segments):
            out = np.zeros_like(state)
            fl, bus = ctypes.c_uint32(), ctypes.c_uint32()
            A = _lib.RunArgs()
            A.struct_size = ctypes.sizeof(_lib.RunArgs)
            A.a, A.n = a.ctypes.data, n
            if bk is not None:
                A.bank, A.bank_bytes = bk.ctypes.data, bk.size
            A.scratch_in, A.scratch_in_bytes = state.ctypes.data, state.nbytes
            A.scratch_out, A.scratch_out_bytes = out.ctypes.data, out.nbytes
            A.flags_out, A.bus_out = ctypes.pointer(fl), ctypes.pointer(bus)
            _lib.check(L.cft_program_run_ex(prog, ctypes.byref(A)), "cft_program_run_ex")
            lines.append(f"segment {k} start {state_hash(state)} end {state_hash(out)} "
                         f"flags {fl.value} status {bus.value}")
            state = out
        return lines, state
    finally:
        L.cft_program_free(prog)
