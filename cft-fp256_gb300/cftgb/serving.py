"""ctypes view of the serving loop (cftg_server_*, include/cft_gb300.h) and a
thin Python handle over it."""
import ctypes

import numpy as np

from . import _lib

vp = ctypes.c_void_p


class ServerConfig(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("hbm_budget", ctypes.c_uint64),
                ("max_inflight", ctypes.c_uint32), ("max_program_inflight", ctypes.c_uint32),
                ("max_batch_calls", ctypes.c_uint32), ("max_batch_lanes", ctypes.c_uint32),
                ("max_batch_elements", ctypes.c_uint64), ("elem_blocks_per_sm", ctypes.c_uint32)]


class Request(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("type", ctypes.c_int), ("kind", ctypes.c_int),
                ("op", ctypes.c_int), ("fmt", ctypes.c_int), ("rnd", ctypes.c_int),
                ("d_a", vp), ("d_b", vp), ("d_c", vp), ("n", ctypes.c_size_t),
                ("prog", vp), ("d_bank", vp), ("init", vp), ("lanes", ctypes.c_size_t),
                ("runs", ctypes.c_uint32), ("host_out", vp), ("t_arrival_ns", ctypes.c_uint64),
                ("tag", ctypes.c_uint64)]


class Completion(ctypes.Structure):
    _fields_ = [("tag", ctypes.c_uint64), ("result", ctypes.c_int32), ("flags", ctypes.c_uint32),
                ("status", ctypes.c_uint32), ("batch", ctypes.c_uint32),
                ("t_arrival_ns", ctypes.c_uint64), ("t_admit_ns", ctypes.c_uint64),
                ("t_done_ns", ctypes.c_uint64)]


class Stats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_uint64) for k in ("submitted", "completed", "failed", "batches",
                                               "launches", "elements_done", "lane_runs_done",
                                               "bytes_in_use", "bytes_peak", "budget")] + \
               [("inflight", ctypes.c_uint32), ("pending", ctypes.c_uint32),
                ("engine_launch_ns", ctypes.c_uint64), ("engine_retire_ns", ctypes.c_uint64),
                ("slot_full_turns", ctypes.c_uint64)]


REQ_ELEM, REQ_PROGRAM = 0, 1
COMPLETION_DTYPE = np.dtype([("tag", "<u8"), ("result", "<i4"), ("flags", "<u4"), ("status", "<u4"),
                             ("batch", "<u4"), ("t_arrival_ns", "<u8"), ("t_admit_ns", "<u8"),
                             ("t_done_ns", "<u8")])
assert COMPLETION_DTYPE.itemsize == ctypes.sizeof(Completion)


def _bind(L):
    if getattr(L, "_serving_bound", False):
        return
    L.cftg_clock_ns.restype = ctypes.c_uint64
    L.cftg_clock_ns.argtypes = []
    L.cftg_server_create.argtypes = [vp, ctypes.POINTER(ServerConfig), ctypes.POINTER(vp)]
    L.cftg_server_submit.argtypes = [vp, ctypes.POINTER(Request)]
    L.cftg_server_poll.argtypes = [vp, vp, ctypes.c_size_t]
    L.cftg_server_poll.restype = ctypes.c_size_t
    L.cftg_server_drain.argtypes = [vp, ctypes.c_uint32]
    L.cftg_server_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    L.cftg_server_free.argtypes = [vp]
    L._serving_bound = True


def clock_ns():
    L = _lib.lib()
    _bind(L)
    return L.cftg_clock_ns()


class Server:
    """One cftg_server: submit() requests, poll() completions as a numpy
    record array, drain(), stats(); close() (or the context manager) stops
    it after every queued request has finished."""

    def __init__(self, h, budget, max_inflight=4, max_program_inflight=4, max_batch_calls=4096,
                 max_batch_lanes=65536, max_batch_elements=0, elem_blocks_per_sm=0):
        self.L = _lib.lib()
        _bind(self.L)
        cfg = ServerConfig(ctypes.sizeof(ServerConfig), budget, max_inflight, max_program_inflight,
                           max_batch_calls, max_batch_lanes, max_batch_elements, elem_blocks_per_sm)
        self.s = vp()
        _lib.check(self.L.cftg_server_create(h, ctypes.byref(cfg), ctypes.byref(self.s)),
                   "cftg_server_create")
        self._buf = np.zeros(65536, COMPLETION_DTYPE)

    def submit(self, req):
        req.struct_size = ctypes.sizeof(Request)
        return self.L.cftg_server_submit(self.s, ctypes.byref(req))

    def poll(self):
        out = []
        while True:
            k = self.L.cftg_server_poll(self.s, self._buf.ctypes.data, len(self._buf))
            if k:
                out.append(self._buf[:k].copy())
            if k < len(self._buf):
                break
        return np.concatenate(out) if out else np.zeros(0, COMPLETION_DTYPE)

    def drain(self, timeout_ms=600000):
        return self.L.cftg_server_drain(self.s, timeout_ms)

    def stats(self):
        st = Stats()
        self.L.cftg_server_get_stats(self.s, ctypes.byref(st))
        return {k: getattr(st, k) for k, _ in Stats._fields_}

    def close(self):
        if self.s:
            self.L.cftg_server_free(self.s)
            self.s = vp()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
