"""Benchmark suites beside the headline (bench.py --suite NAME): each
measures one of the path's benchmark configurations and returns a dict
that bench.py prints as one JSON line.

uneven  10,000 independent elementwise calls, sizes log-uniform in
        [1, 2^20], formats fp64/fp128/fp256 drawn 0.2/0.4/0.4, operation
        uniform over {add, mul, fma, div, sqrt}, rounding attribute uniform
        over the five: one plain launch per call (cftg_run_device) against
        one persistent work-queue launch replayed from a CUDA graph
        (cftg_batch_*), after the tile autotuner. Outputs of the two are
        compared bit for bit, flags per call included.

trajectories  the batched sequencer: 4,096 Lorenz-63 RK4 lanes at
        binary256 (h = 0.01, initial state (1,1,1) + N(0, 1e-3) per lane)
        with step counts log-uniform in [1e3, 1e5], and 512 Lorenz-96 RK4
        lanes at binary128 (N = 40, F = 8, h = 0.005, initial state
        8 + N(0, 1e-3)) with step counts log-uniform in [1e3, 1e4], all as ONE
        CUDA graph launch (cftg_traj_group_*). Every 1,000 steps each lane's
        state is kept; its tagged SHA-256 and the final states are returned
        for checking against the oracle run segment by segment.

bundles  what one bundle of a trajectory launch costs: binary256 programs
        that are one dependent chain of a single operation (FMA, MUL, ADD,
        SUB, NEG, ABS), 32 lanes at 1, 2 and 8 threads a lane.
"""
import ctypes
import hashlib
import time

import numpy as np

from cftgb import _lib


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
    L.cftg_queue_block_threads.argtypes = []
    L.cftg_queue_block_threads.restype = ctypes.c_int


def uneven(h, ncalls=10000, seed=4, max_log2=20, reps=3, sample=0, timed=None):
    """The uneven batch, plain per-call launches against the batched form.
    `timed` (a context manager, e.g. a clock sampler) wraps the timed
    loops. With sample > 0 the result also carries, under "_samples", the
    first and last `sample` elements of every call (operands, the batched
    form's results) and every call's flag word, for the oracle."""
    import contextlib
    import torch
    timed = timed if timed is not None else contextlib.nullcontext()
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
    timed.__enter__()
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
    timed.__exit__(None, None, None)
    exact = all(torch.equal(arena[f]["d1"], arena[f]["d2"]) for f in (1, 2, 3)) and \
        torch.equal(flags_plain, flags_q)
    tiles = L.cftg_batch_tiles(batch)
    L.cftg_batch_free(batch)
    samples = None
    if sample:
        # each call's head and tail (its ragged last tile included), gathered
        # per format with one index_select a buffer
        esz_w = {f: esz[f] // 4 for f in (1, 2, 3)}
        starts = {1: 0, 2: 0, 3: 0}
        rows = {f: [] for f in (1, 2, 3)}
        taken = {1: 0, 2: 0, 3: 0}
        spans = []
        for i in range(ncalls):
            f, n = int(fmts[i]), int(sizes[i])
            s0 = starts[f]
            starts[f] += n
            idx = np.arange(n) if n <= 2 * sample else np.r_[0:sample, n - sample:n]
            spans.append((f, taken[f], len(idx), n))
            taken[f] += len(idx)
            rows[f].append(s0 + idx)
        got = {}
        for f in (1, 2, 3):
            if not rows[f]:
                continue
            ti = torch.from_numpy(np.concatenate(rows[f]).astype(np.int64)).cuda()
            got[f] = {k: arena[f][k].view(-1, esz_w[f]).index_select(0, ti).cpu().numpy()
                      .view(np.uint32) for k in ("a", "b", "c", "d2")}
        fq = flags_q.cpu().numpy().view(np.uint32)
        samples = []
        for i, (f, r0, k, n) in enumerate(spans):
            kind, op = kinds[int(which[i])]
            g = got[f]
            samples.append(dict(kind=kind, op=op, fmt=f, rnd=int(rnds[i]), n=n, whole=k == n,
                                a=g["a"][r0:r0 + k], b=g["b"][r0:r0 + k], c=g["c"][r0:r0 + k],
                                d=g["d2"][r0:r0 + k], flags=int(fq[i])))
    total = int(sizes.sum())
    pm, qm = min(plain_ms), min(q_ms)
    out = {
        "suite": "uneven", "calls": ncalls, "elements": total,
        "plain_ms": pm, "batched_ms": qm, "speedup": pm / qm,
        "plain_gelem_s": total / pm / 1e6, "batched_gelem_s": total / qm / 1e6,
        "tiles": int(tiles), "autotune_s": tune_s, "bit_exact_vs_plain": bool(exact),
        "tile_lengths": {f"fmt{f}": [int(L.cftg_tile_length(f, k, o)) for k, o in kinds]
                         for f in (1, 2, 3)},
        "block_threads": int(L.cftg_queue_block_threads()),
    }
    if samples is not None:
        out["_samples"] = samples
    return out


TAG = b"cft-certificate 1 state\0"


def _bind_traj(L):
    vp = ctypes.c_void_p
    L.cftg_traj_create.argtypes = [vp, vp, ctypes.c_size_t, vp, vp, vp, vp, vp, vp,
                                   ctypes.c_uint32, ctypes.c_uint32, vp, ctypes.POINTER(vp)]
    L.cftg_traj_result.argtypes = [vp, vp, vp, vp]
    L.cftg_traj_free.argtypes = [vp]
    L.cftg_traj_group_capture.argtypes = [ctypes.POINTER(vp), ctypes.c_size_t, vp,
                                          ctypes.POINTER(vp)]
    L.cftg_traj_group_launch.argtypes = [vp, vp]
    L.cftg_traj_group_free.argtypes = [vp]
    L.cft_program_load.argtypes = [vp, vp, ctypes.c_size_t, ctypes.POINTER(vp)]
    L.cft_program_free.argtypes = [vp]


def ode_lanes(kind, fmt, lanes, slots, base, steps_range, steps_per_run, seed):
    """Seeded initial blocks (lane-major, `slots` elements a lane: base +
    N(0, 1e-3) each, rounded to double then widened exactly) and run counts
    (steps log-uniform in steps_range, rounded to whole runs)."""
    from cftgb import workload as wl
    W = wl.words(fmt)
    rng = np.random.default_rng(seed)
    vals = base + rng.normal(0.0, 1e-3, size=(lanes, slots))
    init = np.zeros((lanes * slots, W), np.uint32)
    for i, v in enumerate(vals.reshape(-1)):
        init[i] = wl.from_int(wl.encode_double(fmt, float(v)), W)
    lo, hi = np.log(steps_range[0]), np.log(steps_range[1])
    steps = np.exp(rng.uniform(lo, hi, size=lanes))
    runs = np.maximum(1, np.rint(steps / steps_per_run)).astype(np.uint32)
    return init, runs


def state_hashes(snaps, runs, snap_every, max_snaps, slots, W):
    """Per lane, the tagged SHA-256 of each kept state (one every
    snap_every runs), and one digest over all of them in lane order."""
    snaps = snaps.reshape(len(runs), max_snaps, slots * W)
    per_lane = []
    outer = hashlib.sha256()
    for i, r in enumerate(runs):
        hs = [hashlib.sha256(TAG + snaps[i, k].tobytes()).digest()
              for k in range(min(max_snaps, int(r) // snap_every))]
        per_lane.append(hs)
        for x in hs:
            outer.update(x)
    return per_lane, outer.hexdigest()


def trajectories(h, progs, reps=2, separate=False, timed=None):
    """progs: a list of dicts with image, bank (uint8 arrays), fmt, slots,
    init (lane-major uint32 blocks), runs (uint32 per lane), snap_every,
    max_snaps, steps_per_run. Runs them all as one graph launch, `reps`
    times from the same initial states (the first launch is the warm one),
    and returns timings plus each program's final states and hashes."""
    import torch
    from cftgb import workload as wl
    L = _lib.lib()
    _bind_traj(L)
    vp = ctypes.c_void_p
    stream = torch.cuda.Stream()
    keep, handles = [], []
    for P in progs:
        W = wl.words(P["fmt"])
        n = len(P["runs"])
        prog = vp()
        img = np.ascontiguousarray(P["image"])
        _lib.check(L.cft_program_load(h, img.ctypes.data, img.size, ctypes.byref(prog)),
                   "cft_program_load")
        t = dict(prog=prog, W=W, n=n)
        t["a"] = torch.zeros(max(1, n) * W, dtype=torch.int32, device="cuda")
        t["bank"] = torch.from_numpy(np.ascontiguousarray(P["bank"]).view(np.int32).copy()).cuda()
        t["init"] = torch.from_numpy(np.ascontiguousarray(P["init"]).view(np.int32).copy()).cuda()
        t["state"] = t["init"].clone()
        t["snaps"] = torch.zeros(n * P["max_snaps"] * P["slots"] * W, dtype=torch.int32,
                                 device="cuda")
        t["lf"] = torch.zeros(max(1, n), dtype=torch.uint8, device="cuda")
        runs = np.ascontiguousarray(P["runs"], np.uint32)
        tr = vp()
        _lib.check(L.cftg_traj_create(prog, runs.ctypes.data, n, t["a"].data_ptr(), None, None,
                                      t["bank"].data_ptr(), t["state"].data_ptr(),
                                      t["snaps"].data_ptr(), P["snap_every"], P["max_snaps"],
                                      t["lf"].data_ptr(), ctypes.byref(tr)), "cftg_traj_create")
        t["traj"] = tr
        keep.append(t)
        handles.append(tr)
    arr = (vp * len(handles))(*[x.value for x in handles])
    group = vp()
    _lib.check(L.cftg_traj_group_capture(arr, len(handles), stream.cuda_stream, ctypes.byref(group)),
               "cftg_traj_group_capture")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times = []
    import contextlib
    for _ in range(reps):
        for t in keep:
            t["state"].copy_(t["init"])
            t["snaps"].zero_()
            t["lf"].zero_()
        torch.cuda.synchronize()
        with (timed if timed is not None else contextlib.nullcontext()):
            e0.record(stream)
            _lib.check(L.cftg_traj_group_launch(group, stream.cuda_stream),
                       "cftg_traj_group_launch")
            e1.record(stream)
            stream.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    out = {"suite": "trajectories", "launch_s": min(times), "launches": reps, "programs": []}
    if separate:
        # each program's launch alone, for the breakdown
        L.cftg_traj_launch.argtypes = [vp, vp]
        for P, t in zip(progs, keep):
            t["state"].copy_(t["init"])
            torch.cuda.synchronize()
            e0.record(stream)
            _lib.check(L.cftg_traj_launch(t["traj"], stream.cuda_stream), "cftg_traj_launch")
            e1.record(stream)
            stream.synchronize()
            t["alone_s"] = e0.elapsed_time(e1) / 1e3
        for t in keep:                  # the reported states are the group launch's
            t["state"].copy_(t["init"])
        _lib.check(L.cftg_traj_group_launch(group, stream.cuda_stream), "cftg_traj_group_launch")
        stream.synchronize()
    total_steps = 0
    for P, t in zip(progs, keep):
        fl, st = ctypes.c_uint32(), ctypes.c_uint32()
        _lib.check(L.cftg_traj_result(t["traj"], ctypes.byref(fl), ctypes.byref(st),
                                      stream.cuda_stream), "cftg_traj_result")
        W = t["W"]
        final = t["state"].cpu().numpy().view(np.uint32).reshape(-1, W)
        snaps = t["snaps"].cpu().numpy().view(np.uint32)
        per_lane, digest = state_hashes(snaps, P["runs"], P["snap_every"], P["max_snaps"],
                                        P["slots"], W)
        steps = int(np.sum(P["runs"], dtype=np.int64)) * P["steps_per_run"]
        total_steps += steps
        out["programs"].append({
            "name": P.get("name", "?"), "lanes": t["n"], "lane_steps": steps,
            "alone_s": t.get("alone_s"),
            "max_steps": int(np.max(P["runs"])) * P["steps_per_run"],
            "flags": fl.value, "status": st.value, "state_hash_digest": digest,
            "final_digest": hashlib.sha256(TAG + final.tobytes()).hexdigest(),
            "_final": final, "_hashes": per_lane,
            "_lane_flags": t["lf"].cpu().numpy().copy()})
    L.cftg_traj_group_free(group)
    for t in keep:
        L.cftg_traj_free(t["traj"])
        L.cft_program_free(t["prog"])
    out["lane_steps"] = total_steps
    out["lane_steps_per_s"] = total_steps / out["launch_s"]
    return out


SWEEP_OPS = (("add", 0, 1), ("sub", 0, 2), ("mul", 0, 3), ("fma", 0, 0), ("div", 1, 0),
             ("sqrt", 2, 0))


BUNDLE_CHAINS = (("fma", "fma r0, r0, r1, r2"), ("mul", "mul r0, r0, r1"),
                 ("add", "add r0, r0, r2"), ("sub", "sub r0, r0, r2"), ("neg", "neg r0, r0"),
                 ("abs", "abs r0, r0"))


def bundles(h, lanes=32, reps=1000, per_rep=10, threads=(1, 2, 8), timed=None):
    """What one bundle of a trajectory launch costs: for each operation, a
    binary256 program that is one dependent chain of it (`per_rep` a REPEAT
    body, `reps` times; r0 the running value, r1 ~ 0.999, r2 ~ 0.001, so
    the chain stays normal), run as one trajectory launch of `lanes` lanes
    at G threads a lane (CFTG_LANE_THREADS), best of three. A chain's
    operations each take a bundle of their own, so the time over the
    operations is one bundle's: the operation's latency plus the bundle's
    own work (a NEG chain's is nearly all the latter)."""
    import os
    import torch
    from cftgb import asm
    from cftgb import workload as wl
    L = _lib.lib()
    _bind_traj(L)
    vp = ctypes.c_void_p
    init = np.zeros((lanes * 3, 8), np.uint32)
    for i in range(lanes):
        for k, v in enumerate((1.5, 0.9990234375, 0.0009765625)):
            init[i * 3 + k] = wl.from_int(wl.encode_double(3, v), 8)
    out = {"suite": "bundles", "lanes": lanes, "ops": reps * per_rep, "cells": []}
    old = os.environ.get("CFTG_LANE_THREADS")
    stream = torch.cuda.Stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    import contextlib
    try:
        for G in threads:
            os.environ["CFTG_LANE_THREADS"] = str(G)
            for name, body in BUNDLE_CHAINS:
                src = (".format fp256\n.deposits 0\n.scratch in 3\n.scratch out 3\n"
                       "ldl r0, 0\nldl r1, 1\nldl r2, 2\n"
                       f"repeat {reps}\n" + "\n".join([body] * per_rep) +
                       "\nendrep\nstl r0, 0\nstl r1, 1\nstl r2, 2\nhalt\n")
                img = np.frombuffer(asm.assemble(src), np.uint8).copy()
                prog = vp()
                _lib.check(L.cft_program_load(h, img.ctypes.data, img.size, ctypes.byref(prog)),
                           "cft_program_load")
                state = torch.from_numpy(init.view(np.int32).copy()).cuda()
                ta = torch.zeros((lanes, 8), dtype=torch.int32, device="cuda")
                runs = np.ones(lanes, np.uint32)
                tr = vp()
                _lib.check(L.cftg_traj_create(prog, runs.ctypes.data, lanes, ta.data_ptr(), None,
                                              None, None, state.data_ptr(), None, 0, 0, None,
                                              ctypes.byref(tr)), "cftg_traj_create")
                best = 1e9
                for _ in range(3):
                    state.copy_(torch.from_numpy(init.view(np.int32)).cuda())
                    torch.cuda.synchronize()
                    with (timed if timed is not None else contextlib.nullcontext()):
                        e0.record(stream)
                        _lib.check(L.cftg_traj_launch(tr, stream.cuda_stream), "cftg_traj_launch")
                        e1.record(stream)
                        stream.synchronize()
                    best = min(best, e0.elapsed_time(e1) / 1e3)
                L.cftg_traj_free(tr)
                L.cft_program_free(prog)
                out["cells"].append({"G": G, "op": name, "s": best,
                                     "ns_per_bundle": best / (reps * per_rep) * 1e9})
    finally:
        if old is None:
            os.environ.pop("CFTG_LANE_THREADS", None)
        else:
            os.environ["CFTG_LANE_THREADS"] = old
    return out


def sweep(h, n=1 << 24, reps=3, seed=11, check=None, spread=1 << 20, timed=None):
    """The elementwise sweep: every format x {add, sub, mul, fma, div, sqrt}
    x rounding attribute over n device-generated operands a cell (the
    benchmark's value mix, with exact-cancellation triples and halfway cases
    planted). Each cell is timed over `reps` launches with CUDA events
    (inside `timed`, a context manager such as a clock sampler); the cell is
    run once more with per-element flag bytes and, when `check` is given,
    handed to it: check(cell, operands, results, flag bytes) with host
    arrays of every element for add/sub/mul/fma and of `spread` elements
    spread evenly over the array (first and last included) for div and
    sqrt. check returns a dict merged into the cell."""
    import contextlib
    import torch
    from cftgb import workload as wl
    L = _lib.lib()
    _bind(L)
    stream = torch.cuda.current_stream()
    s = stream.cuda_stream
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    word = torch.zeros(1, dtype=torch.int32, device="cuda")
    cells = []
    pick = np.unique(np.linspace(0, n - 1, min(n, spread)).astype(np.int64))
    tpick = torch.from_numpy(pick).cuda()
    for fmt in range(4):
        W = wl.words(fmt)
        ops = [torch.empty(n * W, dtype=torch.int32, device="cuda") for _ in range(4)]
        for j in range(3):
            _lib.check(L.cftg_fill_operands(fmt, ops[j].data_ptr(), n, seed * 16 + fmt * 4 + j, 64,
                                            100000, s), "cftg_fill_operands")
        wl.plant(fmt, ops[:3], n, seed * 16 + fmt)
        lf = torch.zeros(n, dtype=torch.uint8, device="cuda")
        pa, pb, pc, pd = (x.data_ptr() for x in ops)
        host_all = host_pick = None
        if check is not None:
            host_all = [x.cpu().numpy().view(np.uint32).reshape(n, W) for x in ops[:3]]
            host_pick = [x[pick] for x in host_all]
        for name, kind, op in SWEEP_OPS:
            for rnd in range(5):
                def go(nn, lfp):
                    st = L.cftg_run_device(h, kind, op, fmt, rnd, pa, pb, pc, pd, nn, 0, lfp,
                                           word.data_ptr(), s)
                    _lib.check(st, "cftg_run_device")
                go(n, None)
                torch.cuda.synchronize()
                with (timed if timed is not None else contextlib.nullcontext()):
                    e0.record(stream)
                    for _ in range(reps):
                        go(n, None)
                    e1.record(stream)
                    torch.cuda.synchronize()
                ms = e0.elapsed_time(e1) / reps
                cell = {"fmt": ("fp32", "fp64", "fp128", "fp256")[fmt], "op": name, "rnd": rnd,
                        "ms": ms, "gelem_s": n / ms / 1e6}
                if check is not None:
                    # the checked results come from a full-size launch (the
                    # kernel the cell timed), with per-element flag bytes
                    word.zero_()
                    go(n, lf.data_ptr())
                    torch.cuda.synchronize()
                    d = ops[3].view(n, W)
                    if kind == 0:
                        hd, hl, hops = d.cpu().numpy().view(np.uint32), lf.cpu().numpy(), host_all
                    else:
                        hd = d.index_select(0, tpick).cpu().numpy().view(np.uint32)
                        hl, hops = lf.index_select(0, tpick).cpu().numpy(), host_pick
                    cell.update(check(dict(fmt=fmt, kind=kind, op=op, rnd=rnd,
                                           word=int(word.item()) & 0x1F, whole=kind == 0),
                                      hops, hd, hl))
                cells.append(cell)
        del ops, host_all, host_pick
        torch.cuda.empty_cache()
    return {"suite": "sweep", "elements_per_cell": n, "spread_checked": int(len(pick)),
            "cells": cells}


def hh_init(lanes, seed):
    """Henon-Heiles initial blocks (x, y, px, py) at energy 1/8, lane-major
    binary256: x = 0, y and py drawn, px from the energy in double, each
    value widened exactly."""
    from cftgb import workload as wl
    rng = np.random.default_rng(seed)
    out = np.zeros((lanes * 4, 8), np.uint32)
    for i in range(lanes):
        while True:
            y = rng.uniform(-0.3, 0.4)
            py = rng.uniform(-0.3, 0.3)
            rest = 2 * (0.125 - (y * y / 2 - y ** 3 / 3)) - py * py
            if rest > 0:
                break
        for j, v in enumerate((0.0, y, float(np.sqrt(rest)), py)):
            out[i * 4 + j] = wl.from_int(wl.encode_double(3, v), 8)
    return out


def serving(h, hh_image, hh_bank, rate=20000.0, seconds=60.0, seed=5, budget=40 << 30,
            program_frac=0.02, hh_lanes=32, max_log2=22, sample_every=2000, max_inflight=6,
            max_program_inflight=2, max_batch_elements=1 << 24, elem_blocks_per_sm=0,
            sample_max_n=1 << 20, timed=None):
    """Open-loop serving: requests arrive as a Poisson stream of `rate` a
    second for `seconds`; each is an element call (binary128 or binary256
    1:1, size log-uniform in [64, 2^max_log2], operation uniform over add,
    sub, mul, fma, div, sqrt, rounding attribute uniform) over operands
    resident in HBM, or (a fraction program_frac) a Henon-Heiles leapfrog
    ensemble of hh_lanes lanes at binary256 (h = 1e-3, energy 1/8) for
    1e3..1e4 steps (log-uniform). The server admits them by a budget of
    `budget` bytes. Latency is completion time minus scheduled arrival.
    Every sample_every-th request (element requests of at most
    sample_max_n elements) keeps its output, in pinned memory allocated
    before the stream starts, for the comparison with the same request run
    alone: pinning memory while requests arrive would stall the submitting
    thread and charge the stall to the requests behind it."""
    import contextlib
    import torch
    from cftgb import serving as sv
    timed = timed if timed is not None else contextlib.nullcontext()
    from cftgb import workload as wl
    L = _lib.lib()
    _bind(L)
    sv._bind(L)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(seed)
    maxn = 1 << max_log2
    POOL = 1 << 23
    pools = {}
    for fmt in (2, 3):
        W = wl.words(fmt)
        pools[fmt] = [torch.empty((POOL + maxn) * W, dtype=torch.int32, device="cuda")
                      for _ in range(3)]
        for j in range(3):
            _lib.check(L.cftg_fill_operands(fmt, pools[fmt][j].data_ptr(), POOL + maxn,
                                            seed * 10 + fmt * 3 + j, 64, 100000, stream), "fill")
    prog = ctypes.c_void_p()
    img = np.ascontiguousarray(hh_image)
    _lib.check(L.cft_program_load(h, img.ctypes.data, img.size, ctypes.byref(prog)), "load")
    bank = torch.from_numpy(np.ascontiguousarray(hh_bank).view(np.int32).copy()).cuda()
    inits = [hh_init(hh_lanes, 7000 + k) for k in range(16)]
    torch.cuda.synchronize()

    count = int(rate * seconds * 1.05) + 16
    gaps = rng.exponential(1.0 / rate, size=count)
    arrive = np.cumsum(gaps)
    count = int(np.searchsorted(arrive, seconds))
    arrive = arrive[:count]
    is_prog = rng.random(count) < program_frac
    fmts = rng.choice([2, 3], size=count)
    sizes = np.exp(rng.uniform(np.log(64), np.log(maxn), size=count)).astype(np.int64)
    opsel = rng.integers(0, 6, size=count)
    rnds = rng.integers(0, 5, size=count)
    offs = rng.integers(0, POOL, size=count)
    steps = np.exp(rng.uniform(np.log(1e3), np.log(1e4), size=count))
    runs = np.maximum(10, np.rint(steps / 100)).astype(np.int64)   # the image runs 100 steps
    which_init = rng.integers(0, 16, size=count)
    OPS = SWEEP_OPS
    base = {f: [x.data_ptr() for x in pools[f]] for f in (2, 3)}
    # the sampled requests and their output buffers, carved from one pinned
    # block allocated now
    sampled, nxt = set(), 0
    for i in range(count):
        if i >= nxt and (is_prog[i] or sizes[i] <= sample_max_n):
            sampled.add(i)
            nxt = (i // sample_every + 1) * sample_every
    out_bytes = {i: (inits[0].nbytes if is_prog[i] else int(sizes[i]) * 4 * wl.words(int(fmts[i])))
                 for i in sampled}
    pinned = torch.empty(max(1, sum(out_bytes.values())), dtype=torch.uint8, pin_memory=True)
    out_views, off = {}, 0
    for i in sorted(sampled):
        out_views[i] = pinned[off:off + out_bytes[i]]
        off += out_bytes[i]
    samples = {}
    req = sv.Request()
    comp = []
    with sv.Server(h, budget, max_inflight=max_inflight, max_program_inflight=max_program_inflight,
                   max_batch_calls=4096, max_batch_lanes=1 << 16,
                   max_batch_elements=max_batch_elements,
                   elem_blocks_per_sm=elem_blocks_per_sm) as srv, timed:
        t0 = sv.clock_ns() + 20_000_000
        arr_ns = (t0 + arrive * 1e9).astype(np.int64)
        i = loops = 0
        while i < count:
            now = sv.clock_ns()
            while i < count and arr_ns[i] <= now:
                sample = i in sampled
                req.tag = i
                req.t_arrival_ns = int(arr_ns[i])
                req.host_out = None
                if is_prog[i]:
                    req.type = sv.REQ_PROGRAM
                    req.prog = prog
                    req.d_bank = bank.data_ptr()
                    init = inits[int(which_init[i])]
                    req.init = init.ctypes.data
                    req.lanes = hh_lanes
                    req.runs = int(runs[i])
                    req.n = 0
                    if sample:
                        out = out_views[i]
                        req.host_out = out.data_ptr()
                        samples[i] = ("prog", int(which_init[i]), int(runs[i]), out)
                else:
                    f = int(fmts[i])
                    esz = 4 * wl.words(f)
                    n = int(sizes[i])
                    _, kind, op = OPS[int(opsel[i])]
                    o = int(offs[i]) * esz
                    req.type = sv.REQ_ELEM
                    req.kind, req.op, req.fmt, req.rnd = kind, op, f, int(rnds[i])
                    req.d_a, req.d_b, req.d_c = base[f][0] + o, base[f][1] + o, base[f][2] + o
                    req.n = n
                    req.prog = None
                    if sample:
                        out = out_views[i]
                        req.host_out = out.data_ptr()
                        samples[i] = ("elem", kind, op, f, int(rnds[i]), req.d_a, req.d_b, req.d_c,
                                      n, out)
                st = srv.submit(req)
                if st:
                    raise RuntimeError(f"submit refused request {i}: status {st}")
                i += 1
            loops += 1
            if loops % 64 == 0:
                comp.append(srv.poll())
            time.sleep(0.0002)
        t_sub_end = sv.clock_ns()
        _lib.check(srv.drain(), "cftg_server_drain")
        t_end = sv.clock_ns()
        comp.append(srv.poll())
        stats = srv.stats()
    done = np.concatenate(comp)
    lat = (done["t_done_ns"].astype(np.int64) - done["t_arrival_ns"].astype(np.int64)) / 1e6
    wait = (done["t_admit_ns"].astype(np.int64) - done["t_arrival_ns"].astype(np.int64)) / 1e6
    tags = done["tag"].astype(np.int64)
    prog_mask = is_prog[tags]

    def pct(x):
        return {"p50_ms": float(np.percentile(x, 50)), "p99_ms": float(np.percentile(x, 99)),
                "p999_ms": float(np.percentile(x, 99.9)), "max_ms": float(np.max(x))} if len(x) else {}
    wall = (t_end - t0) / 1e9
    elem_done = int(sizes[tags[~prog_mask]].sum())
    lane_steps = int((runs[tags[prog_mask]] * 100 * hh_lanes).sum())
    # each sampled request again, alone
    word = torch.zeros(1, dtype=torch.int32, device="cuda")
    flags = {int(t): int(f) for t, f in zip(done["tag"], done["flags"])}
    bad = []
    for tag, m in samples.items():
        if m[0] == "elem":
            _, kind, op, f, rnd, pa, pb, pc, n, out = m
            d = torch.empty(n * 4 * wl.words(f), dtype=torch.uint8, device="cuda")
            word.zero_()
            _lib.check(L.cftg_run_device(h, kind, op, f, rnd, pa, pb, pc, d.data_ptr(), n, 0, None,
                                         word.data_ptr(), stream), "cftg_run_device")
            torch.cuda.synchronize()
            if not torch.equal(d.cpu(), out) or flags[tag] != (int(word.item()) & 0x1F):
                bad.append({"tag": tag, "n": n, "fmt": f, "kind": kind, "op": op,
                            "bits_equal": bool(torch.equal(d.cpu(), out)),
                            "flags_mix": flags[tag], "flags_alone": int(word.item()) & 0x1F})
        else:
            _, k, r, out = m
            final, fl = _traj_alone(L, prog, bank, inits[k], hh_lanes, r)
            mix = out.numpy().view(np.uint32).reshape(hh_lanes, -1)
            alone = final.reshape(hh_lanes, -1)
            lanes_off = [j for j in range(hh_lanes) if not np.array_equal(mix[j], alone[j])]
            if lanes_off or flags[tag] != fl:
                bad.append({"tag": tag, "runs": r, "lanes_differ": lanes_off[:8],
                            "n_lanes_differ": len(lanes_off), "flags_mix": flags[tag],
                            "flags_alone": fl, "zero_lanes_mix": int((~mix.any(axis=1)).sum())})
    L.cft_program_free(prog)
    return {
        "suite": "serving", "offered_req_s": rate, "seconds": seconds, "requests": int(count),
        "program_requests": int(is_prog.sum()), "completed": int(len(done)),
        "failed": int((done["result"] != 0).sum()),
        "wall_s": wall, "submit_lag_s": (t_sub_end - t0) / 1e9 - float(arrive[-1]),
        "served_gelem_s": elem_done / wall / 1e9, "elements": elem_done,
        "program_lane_steps_per_s": lane_steps / wall,
        "latency_all": pct(lat), "latency_elem": pct(lat[~prog_mask]),
        "latency_program": pct(lat[prog_mask]),
        "admission_wait_elem": pct(wait[~prog_mask]),
        "admission_wait_program": pct(wait[prog_mask]),
        "batch_requests_mean": float(len(done) / max(1, stats["batches"])),
        "engine": {"launch_s": stats["engine_launch_ns"] / 1e9,
                   "retire_s": stats["engine_retire_ns"] / 1e9,
                   "slot_full_turns": int(stats["slot_full_turns"]),
                   "max_inflight": max_inflight, "max_program_inflight": max_program_inflight,
                   "max_batch_elements": max_batch_elements},
        "batches": int(stats["batches"]), "bytes_peak": int(stats["bytes_peak"]),
        "budget": int(budget), "samples_checked": len(samples), "sample_mismatches": bad,
        "bit_exact_alone_vs_mix": not bad,
        "mix": {"formats": "fp128:fp256 1:1", "sizes": f"log-uniform [64, 2^{max_log2}]",
                "ops": "add/sub/mul/fma/div/sqrt uniform", "program_frac": program_frac,
                "program": f"henonheiles-lf-fp256 h=1e-3 E=1/8, {hh_lanes} lanes, 1e3..1e4 steps"},
    }


def _traj_alone(L, prog, bank, init, lanes, runs):
    import torch
    _bind_traj(L)
    L.cftg_traj_launch.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    ts = torch.from_numpy(init.view(np.int32).copy()).cuda()
    ta = torch.zeros(lanes * 8, dtype=torch.int32, device="cuda")
    lf = torch.zeros(lanes, dtype=torch.uint8, device="cuda")
    segs = np.full(lanes, runs, np.uint32)
    t = ctypes.c_void_p()
    _lib.check(L.cftg_traj_create(prog, segs.ctypes.data, lanes, ta.data_ptr(), None, None,
                                  bank.data_ptr(), ts.data_ptr(), None, 0, 0, lf.data_ptr(),
                                  ctypes.byref(t)), "cftg_traj_create")
    s = torch.cuda.current_stream().cuda_stream
    _lib.check(L.cftg_traj_launch(t, s), "cftg_traj_launch")
    fl, st = ctypes.c_uint32(), ctypes.c_uint32()
    _lib.check(L.cftg_traj_result(t, ctypes.byref(fl), ctypes.byref(st), s), "cftg_traj_result")
    L.cftg_traj_free(t)
    return ts.cpu().numpy().view(np.uint32), int(np.bitwise_or.reduce(lf.cpu().numpy() & 0x1F))


RED_OPS = (("sum", 24), ("dot", 25), ("sumsq", 28), ("sumabs", 29), ("maxall", 31))


def reduce(h, n=1 << 24, reps=3, check_n=65536, seed=17, seg_sizes=(1024, 65536)):
    """The reductions over n device-resident elements a format (normals with
    exponents in [-20, 20], no specials, so the sums stay finite), and the
    segmented SUM over segments of each of seg_sizes at binary128 and
    binary256, timed with CUDA events; the first check_n elements (whole
    segments of them) are reduced again and returned with their operands
    for the oracle."""
    import torch
    from cftgb import workload as wl
    L = _lib.lib()
    _bind(L)
    vp = ctypes.c_void_p
    i = ctypes.c_int
    L.cftg_reduce_device.argtypes = [vp, i, i, i, vp, vp, vp, ctypes.c_size_t, ctypes.c_size_t,
                                     vp, vp, vp]
    L.cftg_reduce_partial_bytes.argtypes = [i, ctypes.c_size_t]
    L.cftg_reduce_partial_bytes.restype = ctypes.c_size_t
    stream = torch.cuda.current_stream()
    s = stream.cuda_stream
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    cells, checks = [], []
    word = torch.zeros(2, dtype=torch.int32, device="cuda")
    for fmt in (1, 2, 3):
        W = wl.words(fmt)
        a = torch.empty(n * W, dtype=torch.int32, device="cuda")
        b = torch.empty(n * W, dtype=torch.int32, device="cuda")
        _lib.check(L.cftg_fill_operands(fmt, a.data_ptr(), n, seed + fmt, 20, 0, s), "fill")
        _lib.check(L.cftg_fill_operands(fmt, b.data_ptr(), n, seed + 8 + fmt, 20, 0, s), "fill")
        part = torch.empty(L.cftg_reduce_partial_bytes(fmt, n) // 4 + 8, dtype=torch.int32,
                           device="cuda")
        out = torch.zeros(W, dtype=torch.int32, device="cuda")
        for name, op in RED_OPS:
            def go(nn):
                _lib.check(L.cftg_reduce_device(h, op, fmt, 0, a.data_ptr(), b.data_ptr(),
                                                out.data_ptr(), nn, nn, part.data_ptr(),
                                                word.data_ptr(), s), "cftg_reduce_device")
            go(n)
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(reps):
                go(n)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            cells.append({"fmt": ("fp32", "fp64", "fp128", "fp256")[fmt], "op": name, "ms": ms,
                          "gelem_s": n / ms / 1e6})
            go(check_n)
            torch.cuda.synchronize()
            checks.append(dict(fmt=fmt, op=op, seg=check_n, d=out.cpu().numpy().view(np.uint32).copy(),
                               flags=int(word[0].item()) & 0x1F,
                               a=a[:check_n * W].cpu().numpy().view(np.uint32).reshape(-1, W),
                               b=b[:check_n * W].cpu().numpy().view(np.uint32).reshape(-1, W)))
        # the segmented form: SUM over consecutive segments of `seg` elements
        if fmt >= 2:
            for seg in seg_sizes:
                outs = torch.zeros((n // seg) * W, dtype=torch.int32, device="cuda")

                def gs(nn):
                    _lib.check(L.cftg_reduce_device(h, 24, fmt, 0, a.data_ptr(), b.data_ptr(),
                                                    outs.data_ptr(), nn, seg, part.data_ptr(),
                                                    word.data_ptr(), s), "cftg_reduce_device")
                gs(n)
                torch.cuda.synchronize()
                e0.record(stream)
                for _ in range(reps):
                    gs(n)
                e1.record(stream)
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1) / reps
                cells.append({"fmt": ("fp32", "fp64", "fp128", "fp256")[fmt], "op": "sum",
                              "seg": seg, "ms": ms, "gelem_s": n / ms / 1e6})
                cn = max(seg, check_n - check_n % seg)
                gs(cn)
                torch.cuda.synchronize()
                checks.append(dict(fmt=fmt, op=24, seg=seg,
                                   d=outs[:(cn // seg) * W].cpu().numpy().view(np.uint32).copy(),
                                   flags=int(word[0].item()) & 0x1F,
                                   a=a[:cn * W].cpu().numpy().view(np.uint32).reshape(-1, W),
                                   b=b[:cn * W].cpu().numpy().view(np.uint32).reshape(-1, W)))
    return {"suite": "reduce", "elements": n, "cells": cells, "_checks": checks}


def link(h, nbytes=1 << 30, reps=3):
    """The host link's rates: copy-engine copies of pinned memory each way
    and both ways at once (torch), and this library's kernel reading and
    writing pinned host memory in place - a binary64 NEG through cft_run
    (reads 8 bytes and writes 8 an element, almost no arithmetic); then
    host-to-device copies split over 2 and 4 streams, and a copy beside the
    kernel's in-place reads (each on half the bytes), to see whether the
    link carries more than one engine or one kernel draws from it."""
    import torch
    L = _lib.lib()
    out = {}
    hp = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    hq = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    hp.fill_(1)
    dv = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    dw = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3 / reps

    out["h2d_gbs"] = nbytes / timed(lambda: dv.copy_(hp, non_blocking=True)) / 1e9
    out["d2h_gbs"] = nbytes / timed(lambda: hq.copy_(dv, non_blocking=True)) / 1e9

    def both():
        with torch.cuda.stream(s1):
            dv.copy_(hp, non_blocking=True)
        with torch.cuda.stream(s2):
            hq.copy_(dw, non_blocking=True)
        torch.cuda.current_stream().wait_stream(s1)
        torch.cuda.current_stream().wait_stream(s2)
    out["both_ways_gbs_each"] = nbytes / timed(both) / 1e9
    n = nbytes // 8
    fl = ctypes.c_uint32()

    def neg():
        _lib.check(L.cft_run(h, 5, 1, 0, hp.data_ptr(), None, None, hq.data_ptr(), n,
                             ctypes.byref(fl), None), "cft_run")
    t = timed(neg)
    out["kernel_in_place_read_gbs"] = nbytes / t / 1e9
    out["kernel_in_place_write_gbs"] = nbytes / t / 1e9

    # host-to-device over k streams at once (one slice each: several copy
    # engines, if the driver spreads them)
    extra = [torch.cuda.Stream() for _ in range(4)]
    for k in (2, 4):
        part = nbytes // k

        def many():
            for j in range(k):
                with torch.cuda.stream(extra[j]):
                    dv[j * part:(j + 1) * part].copy_(hp[j * part:(j + 1) * part], non_blocking=True)
            for j in range(k):
                torch.cuda.current_stream().wait_stream(extra[j])
        out[f"h2d_{k}_streams_gbs"] = nbytes / timed(many) / 1e9

    # a copy engine and the kernel's in-place reads at once, each on its own
    # half of the bytes: their sum is what the link carries for both
    half = nbytes // 2
    hn = half // 8

    def mixed():
        with torch.cuda.stream(extra[0]):
            dv[:half].copy_(hp[half:], non_blocking=True)
        _lib.check(L.cft_run(h, 5, 1, 0, hp.data_ptr(), None, None, hq.data_ptr(), hn,
                             ctypes.byref(fl), None), "cft_run")
        torch.cuda.current_stream().wait_stream(extra[0])
    out["copy_plus_kernel_read_gbs"] = 2 * half / timed(mixed) / 1e9
    return {"suite": "link", "bytes": nbytes, **out}
