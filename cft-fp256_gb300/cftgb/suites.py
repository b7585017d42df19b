"""Benchmark suites beside the headline (bench.py --suite NAME): each
measures one of the configurations the project is judged on and returns
a dict that bench.py prints as one JSON line.

uneven  10,000 independent elementwise calls, sizes log-uniform in
        [1, 2^20], formats fp64/fp128/fp256 drawn 0.2/0.4/0.4, operation
        uniform over {add, mul, fma, div, sqrt}, rounding attribute uniform
        over the five: one plain launch per call (cftg_run_device) against
        one persistent work-queue launch replayed from a CUDA graph
        (cftg_batch_*), after the tile autotuner. Outputs of the two are
        compared bit for bit, flags per call included.
"""
import ctypes
import time

import numpy as np

from . import _lib


class Call(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("op", ctypes.c_int), ("fmt", ctypes.c_int),
                ("rnd", ctypes.c_int), ("a", ctypes.c_void_p), ("b", ctypes.c_void_p),
                ("c", ctypes.c_void_p), ("d", ctypes.c_void_p), ("n", ctypes.c_size_t),
                ("scalar_mask", ctypes.c_uint32)]


def _bind(L):
    vp = ctypes.c_void_p
    L.cftg_batch_create.argtypes = [vp, ctypes.POINTER(Call), ctypes.c_size_t, vp, ctypes.POINTER(vp)]
    L.cftg_batch_launch.argtypes = [vp, vp]
    L.cftg_batch_capture.argtypes = [vp, vp]
    L.cftg_batch_free.argtypes = [vp]
    L.cftg_batch_tiles.argtypes = [vp]
    L.cftg_batch_tiles.restype = ctypes.c_uint32
    L.cftg_fill_operands.argtypes = [ctypes.c_int, vp, ctypes.c_size_t, ctypes.c_uint64,
                                     ctypes.c_int, ctypes.c_uint32, vp]
    L.cftg_autotune.argtypes = [vp, vp, vp, vp, vp, ctypes.c_size_t, vp]
    L.cftg_tile_length.argtypes = [ctypes.c_int] * 3
    L.cftg_tile_length.restype = ctypes.c_uint32


def uneven(h, ncalls=10000, seed=4, max_log2=20, reps=3):
    import torch
    L = _lib.lib()
    _bind(L)
    rng = np.random.default_rng(seed)
    fmts = rng.choice([1, 2, 3], size=ncalls, p=[0.2, 0.4, 0.4])
    sizes = np.exp(rng.uniform(0, max_log2 * np.log(2), size=ncalls)).astype(np.int64)
    sizes = np.clip(sizes, 1, 1 << max_log2)
    kinds = [(0, 1), (0, 3), (0, 0), (1, 0), (2, 0)]          # add, mul, fma, div, sqrt
    which = rng.integers(0, 5, size=ncalls)
    rnds = rng.integers(0, 5, size=ncalls)
    esz = {1: 8, 2: 16, 3: 32}
    stream = torch.cuda.current_stream().cuda_stream
    # one arena per format for a, b, c and for the two outputs
    tot = {f: int(sizes[fmts == f].sum()) for f in (1, 2, 3)}
    arena = {}
    for f in (1, 2, 3):
        words = tot[f] * esz[f] // 4
        arena[f] = {k: torch.empty(max(1, words), dtype=torch.int32, device="cuda")
                    for k in ("a", "b", "c", "d1", "d2")}
        for j, k in enumerate(("a", "b", "c")):
            st = L.cftg_fill_operands(f, arena[f][k].data_ptr(), tot[f], seed * 10 + j, 64, 100000,
                                      stream)
            _lib.check(st, "cftg_fill_operands")
    # tile autotune over fp256-sized scratch
    tn = 1 << 20
    tb = [torch.empty(tn * 8, dtype=torch.int32, device="cuda") for _ in range(4)]
    for j in range(3):
        L.cftg_fill_operands(3, tb[j].data_ptr(), tn, 99 + j, 64, 100000, stream)
    t0 = time.perf_counter()
    _lib.check(L.cftg_autotune(h, tb[0].data_ptr(), tb[1].data_ptr(), tb[2].data_ptr(),
                               tb[3].data_ptr(), tn, stream), "cftg_autotune")
    tune_s = time.perf_counter() - t0
    del tb
    off = {1: 0, 2: 0, 3: 0}
    calls = (Call * ncalls)()
    plain = []
    for i in range(ncalls):
        f, n = int(fmts[i]), int(sizes[i])
        kind, op = kinds[int(which[i])]
        base = off[f] * esz[f]
        off[f] += n
        A = arena[f]
        ptr = {k: A[k].data_ptr() + base for k in A}
        calls[i] = Call(kind, op, f, int(rnds[i]), ptr["a"], ptr["b"], ptr["c"], ptr["d2"], n, 0)
        plain.append((kind, op, f, int(rnds[i]), ptr["a"], ptr["b"], ptr["c"], ptr["d1"], n))
    flags_plain = torch.zeros(ncalls, dtype=torch.int32, device="cuda")
    flags_q = torch.zeros(ncalls, dtype=torch.int32, device="cuda")
    fp = flags_plain.data_ptr()

    def run_plain():
        for i, (kind, op, f, rnd, a, b, c, d, n) in enumerate(plain):
            st = L.cftg_run_device(h, kind, op, f, rnd, a, b, c, d, n, 0, None, fp + 4 * i, stream)
            if st:
                _lib.check(st, "cftg_run_device")

    batch = ctypes.c_void_p()
    _lib.check(L.cftg_batch_create(h, calls, ncalls, flags_q.data_ptr(), ctypes.byref(batch)),
               "cftg_batch_create")
    s2 = torch.cuda.Stream()
    _lib.check(L.cftg_batch_capture(batch, s2.cuda_stream), "cftg_batch_capture")
    # warm
    flags_plain.zero_()
    run_plain()
    _lib.check(L.cftg_batch_launch(batch, s2.cuda_stream), "launch")
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    plain_ms = []
    for _ in range(reps):
        flags_plain.zero_()
        torch.cuda.synchronize()
        e0.record()
        run_plain()
        e1.record()
        torch.cuda.synchronize()
        plain_ms.append(e0.elapsed_time(e1))
    q_ms = []
    for _ in range(reps):
        torch.cuda.synchronize()
        e0.record(s2)
        _lib.check(L.cftg_batch_launch(batch, s2.cuda_stream), "launch")
        e1.record(s2)
        s2.synchronize()
        q_ms.append(e0.elapsed_time(e1))
    exact = all(torch.equal(arena[f]["d1"], arena[f]["d2"]) for f in (1, 2, 3)) and \
        torch.equal(flags_plain, flags_q)
    tiles = L.cftg_batch_tiles(batch)
    L.cftg_batch_free(batch)
    total = int(sizes.sum())
    pm, qm = min(plain_ms), min(q_ms)
    return {
        "suite": "uneven", "calls": ncalls, "elements": total,
        "plain_ms": pm, "batched_ms": qm, "speedup": pm / qm,
        "plain_gelem_s": total / pm / 1e6, "batched_gelem_s": total / qm / 1e6,
        "tiles": int(tiles), "autotune_s": tune_s, "bit_exact_vs_plain": bool(exact),
        "tile_lengths": {f"fmt{f}": [int(L.cftg_tile_length(f, k, o)) for k, o in kinds]
                         for f in (1, 2, 3)},
    }
