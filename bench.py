#!/usr/bin/env python3
"""Benchmark: binary256 FMA throughput (Gelem/s, bit-exact) on GB300.

Workload (one "step" = one pass of the hot path over one batch):
    binary256 fused multiply-add d = a*b + c, roundTiesToEven, n = 2^24
    elements - the fp256 x FMA x RNE cell of the elementwise sweep - over
    seeded synthetic operands with the sweep's value mix (90% normals with
    exponents in [-64, 64], 10% specials, exact-cancellation triples).
    Inputs are 1.5 GiB, larger than L2, so no flush is needed between steps.

value   whole-job Gelem/s with operands resident in HBM (device pointers
        through cftg_run_device), timed with CUDA events on the launch
        stream, max over ranks.
e2e     the same through the reference-facing C ABI (cft_run) with pinned
        HOST buffers: uploads, kernel and download inside the timed region.
roofline  the FMA kernel's algorithmic bytes (4 x 32 B an element) per
        launch over its measured launch time, against the measured HBM copy
        bandwidth.
cpu_baseline  the oracle's C restatement of the reference softfloat, on all
        host cores, over a bounded sample of the same operands.

--impl reference runs the reference path's CPU arithmetic (the oracle port;
the reference library itself cannot be built on the GPU host) on the host
cores and prints the same line with "impl": "reference".

Multi-GPU: one process per GPU (torchrun); each rank runs its own 2^24
elements (the path shards by element with no exchange but an OR of the
flag word), "scaling": "weak", value = all ranks' elements / slowest rank.
"""
import argparse
import contextlib
import ctypes
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "cft-fp256_gb300"))

METRIC = "fp256/fp128 FMA Gelem/s bit-exact (plain vs batched); mixed-load p50/p99 latency"
# GPU reads of pinned host memory, GB/s, on a GB300 with a Grace host (the
# copy engines' host-to-device rate and a streaming kernel's, which agree;
# bench.py --suite link measures it)
LINK_READ_GBS = 211.0
# DRAM bytes (read + write) an element of the FMA kernel: dram__bytes_read.sum
# + dram__bytes_write.sum of one ncu-captured launch over 4,194,304 elements
# of the same operand mix (402.7 + 112.3 MB)
TRAFFIC_B_PER_ELEM = {3: 515.05e6 / 4194304}
N_DEFAULT = 1 << 24


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        j = json.loads(p.read_text())
        return float(j["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples (every 20 ms, each with its own timestamp) kept for
    the timed regions. `with clk:` marks one region; the sampler starts at
    the first region and stops at close() (or at the end of the region when
    keep is False). A sample counts for a region when its timestamp lies in
    it or within `slack` seconds of it, so a region shorter than the
    sampling interval still has its nearest samples."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index, keep=False, slack=0.06):
        self.index = index
        self.keep = keep
        self.slack = slack
        self.proc = None
        self.lines = []
        self.regions = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=timestamp," + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)                 # the first sample arrives before the region
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __enter__(self):
        if self.proc is None:
            self.start()
        self.regions.append([time.time(), None])
        return self

    def __exit__(self, *a):
        self.regions[-1][1] = time.time()
        if not self.keep:
            self.close()

    def close(self):
        if self.proc:
            time.sleep(0.1)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.proc = None

    @staticmethod
    def _stamp(s):
        import datetime
        for fmt in ("%Y/%m/%d %H:%M:%S.%f", "%Y/%m/%d %H:%M:%S"):
            try:
                return datetime.datetime.strptime(s, fmt).timestamp()
            except ValueError:
                pass
        return None

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        regions = [(a, b if b is not None else time.time()) for a, b in self.regions]
        for ln in list(self.lines):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            ts = self._stamp(f[0])
            if ts is None or not any(a - self.slack <= ts <= b + self.slack for a, b in regions):
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "sm_min_mhz": min(sm),
                "reasons": sorted(reasons), "samples": len(sm),
                "timed_s": round(sum(b - a for a, b in regions), 3)}


def cpu_baseline(fmt, a, b, c, seconds=12.0, per_call=2048):
    """The oracle (C restatement of the reference softfloat) on all host
    cores: threads each run chunks of `per_call` elements until the time
    budget is spent. ctypes releases the GIL inside the call."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_lib
    o = oracle_lib.Oracle()
    threads = os.cpu_count() or 1
    n = a.shape[0]
    done = [0] * threads
    stop = time.perf_counter() + seconds

    def worker(t):
        L = o.L
        d = np.zeros((per_call, a.shape[1]), np.uint32)
        acc = ctypes.c_uint32()
        k = t
        while time.perf_counter() < stop:
            s = (k * per_call) % (n - per_call)
            L.sfp_run(0, fmt, 0, 0, a[s:].ctypes.data, b[s:].ctypes.data, c[s:].ctypes.data,
                      d.ctypes.data, per_call, 0, None, ctypes.byref(acc))
            done[t] += per_call
            k += threads
    t0 = time.perf_counter()
    th = [threading.Thread(target=worker, args=(i,)) for i in range(threads)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    dt = time.perf_counter() - t0
    return sum(done) / dt, threads, sum(done), dt


ODE_PROGRAMS = (
    # name, image/bank key, format, state slots, initial value, steps range,
    # steps a run (the image's REPEAT count), lanes, runs between kept states
    ("lorenz63-rk4-fp256 h=0.01", "l63", 3, 3, 1.0, (1e3, 1e5), 100, 4096, 10),
    ("lorenz96-rk4-fp128 N=40 F=8 h=0.005", "l96", 2, 40, 8.0, (1e3, 1e4), 20, 512, 50),
)


def ode_programs(scale=1.0, steps_scale=1.0):
    """The trajectory workload's programs: images and banks from the
    committed fixture (the reference's own ODE images; banks for the named
    step sizes), seeded initial states and uneven run counts. `scale`
    scales the lane counts and `steps_scale` the step range (both 1 for
    the configuration; smaller for profiler captures)."""
    import bench_suites as suites
    z = np.load(ROOT / "tests" / "golden" / "odes.npz")
    progs = []
    for i, (name, key, fmt, slots, base, rng, spr, lanes, every) in enumerate(ODE_PROGRAMS):
        lanes = max(1, int(lanes * scale))
        rng = (max(spr, rng[0] * steps_scale), max(spr, rng[1] * steps_scale))
        init, runs = suites.ode_lanes(key, fmt, lanes, slots, base, rng, spr, 1000 + i)
        progs.append(dict(name=name, image=z[key + "_image"], bank=z[key + "_bank"], fmt=fmt,
                          slots=slots, init=init, runs=runs, snap_every=every,
                          max_snaps=int(np.max(runs)) // every + 1, steps_per_run=spr))
    return progs


def traj_oracle_check(progs, res, per_prog=8):
    """The oracle runs a sample of each program's lanes segment by segment
    on all host cores: the shortest lanes, lanes at the quartiles and the
    longest. Every kept state's hash and the final state must equal the
    GPU's. Returns (mismatches, lanes checked, oracle lane-steps/s, threads,
    seconds)."""
    sys.path.insert(0, str(ROOT / "tests"))
    import hashlib
    import oracle_lib
    import bench_suites as suites
    from cftgb import workload as wl
    o = oracle_lib.Oracle()
    jobs = []
    for P, R in zip(progs, res["programs"]):
        order = np.argsort(P["runs"], kind="stable")
        n = len(order)
        pick = list(order[:per_prog // 2]) + [order[int(q * (n - 1))] for q in (0.25, 0.5, 0.75)]
        pick.append(order[-1])
        for lane in dict.fromkeys(int(x) for x in pick):
            jobs.append((P, R, lane))
    bad = []
    steps_done = [0]
    lock = threading.Lock()

    def one(job):
        P, R, lane = job
        W = wl.words(P["fmt"])
        slots = P["slots"]
        img = np.ascontiguousarray(P["image"])
        bank = np.ascontiguousarray(P["bank"])
        s = np.ascontiguousarray(P["init"][lane * slots:(lane + 1) * slots])
        a = np.zeros((1, W), np.uint32)
        hs = R["_hashes"][lane]
        for k in range(int(P["runs"][lane])):
            out = np.zeros_like(s)
            A = oracle_lib.SeqArgs()
            A.a, A.n, A.bank = a.ctypes.data, 1, bank.ctypes.data
            A.scratch_in, A.scratch_out, A.depth = s.ctypes.data, out.ctypes.data, 256
            if o.L.sfp_seq_run(img.ctypes.data, img.size, ctypes.byref(A)) != 0:
                return (P["name"], lane, "oracle refused")
            s = out
            if (k + 1) % P["snap_every"] == 0:
                j = (k + 1) // P["snap_every"] - 1
                if j >= len(hs) or hashlib.sha256(suites.TAG + s.tobytes()).digest() != hs[j]:
                    return (P["name"], lane, f"state hash after run {k + 1}")
        with lock:
            steps_done[0] += int(P["runs"][lane]) * P["steps_per_run"]
        if not np.array_equal(R["_final"][lane * slots:(lane + 1) * slots], s):
            return (P["name"], lane, "final state")
        return None

    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    from concurrent.futures import ThreadPoolExecutor
    # longest jobs first so the pool's last worker is not the long one
    jobs.sort(key=lambda j: -int(j[0]["runs"][j[2]]) * j[0]["steps_per_run"] * j[0]["slots"])
    with ThreadPoolExecutor(threads) as ex:
        for r in ex.map(one, jobs):
            if r:
                bad.append(r)
    dt = time.perf_counter() - t0
    return bad, len(jobs), steps_done[0] / dt, min(threads, len(jobs)), dt


def traj_reference_check(progs, res):
    """Every lane of every program against the reference library's own
    results for the same workload (tests/golden/traj_digests.npz, made by
    tests/golden/make_traj_digests.py): the final state's tagged SHA-256,
    the digest over every kept state's hash, and the lane's flags."""
    import hashlib
    z = np.load(ROOT / "tests" / "golden" / "traj_digests.npz")
    from bench_suites import TAG
    out = {"lanes_checked": 0, "final_mismatches": 0, "kept_mismatches": 0,
           "flag_mismatches": 0, "first_bad": []}
    for i, (P, R) in enumerate(zip(progs, res["programs"])):
        if f"p{i}_final" not in z.files or not np.array_equal(z[f"p{i}_runs"], P["runs"]):
            out["first_bad"].append(f"{P['name']}: no reference digests for this workload")
            continue
        slots, W = P["slots"], R["_final"].shape[1]
        fin = R["_final"].reshape(-1, slots, W)
        for lane in range(len(P["runs"])):
            f = hashlib.sha256(TAG + fin[lane].tobytes()).digest()
            k = hashlib.sha256(b"".join(R["_hashes"][lane])).digest()
            bad = []
            if f != z[f"p{i}_final"][lane].tobytes():
                out["final_mismatches"] += 1
                bad.append("final")
            if k != z[f"p{i}_kept"][lane].tobytes():
                out["kept_mismatches"] += 1
                bad.append("kept")
            if int(R["_lane_flags"][lane]) & 0x1F != int(z[f"p{i}_flags"][lane]):
                out["flag_mismatches"] += 1
                bad.append("flags")
            if bad and len(out["first_bad"]) < 8:
                out["first_bad"].append(f"{P['name']} lane {lane}: {'/'.join(bad)}")
            out["lanes_checked"] += 1
    return out


def run_trajectories(h, suites, args):
    progs = ode_programs(args.scale, args.steps_scale)
    clk = Clocks(0, keep=True)
    try:
        res = suites.trajectories(h, progs, reps=2, separate=args.separate, timed=clk)
    finally:
        clk.close()
    res["clocks"] = clk.summary()
    if args.scale == 1.0 and args.steps_scale == 1.0:
        res["reference_check"] = traj_reference_check(progs, res)
    bad, checked, cpu_rate, thr, cpu_s = traj_oracle_check(progs, res)
    for p in res["programs"]:
        p.pop("_final")
        p.pop("_hashes")
        p.pop("_lane_flags")
    res["oracle_lanes_checked"] = checked
    res["oracle_mismatches"] = [list(map(str, b)) for b in bad]
    res["cpu_baseline"] = {"value": cpu_rate, "unit": "lane-steps/s", "cores": thr, "kind": "port",
                           "sample": f"{checked} lanes (shortest, quartiles, longest of each "
                                     f"program) run whole by the oracle, {cpu_s:.1f} s"}
    return res


def run_sweep(h, suites, args):
    """The sweep suite with every cell checked against the oracle on all
    host cores as it finishes: every element of every add, sub, mul and
    fma cell (values and per-element flag bytes, and the launch's flag
    word), and 2^20 elements spread over the array for each div and sqrt
    cell (values and flag bytes). Clocks are sampled over the timed
    launches of all cells."""
    o = _oracle()
    t_or = [0.0]

    def check(cell, ops, d, lf):
        t0 = time.perf_counter()
        rd, rlf, racc = o.run_parallel(cell["kind"], cell["fmt"], cell["op"], cell["rnd"],
                                       ops[0], ops[1], ops[2])
        t_or[0] += time.perf_counter() - t0
        r = {"checked": int(d.shape[0]),
             "value_mismatches": int(np.count_nonzero((d != rd).any(1))),
             "flag_mismatches": int(np.count_nonzero(lf != rlf))}
        if cell["whole"]:
            r["flag_word_equal"] = cell["word"] == racc
        return r
    clk = Clocks(0, keep=True)
    try:
        res = suites.sweep(h, n=min(args.n, 1 << 24), check=check, timed=clk)
    finally:
        clk.close()
    cells = res["cells"]
    res["oracle_cells_checked"] = len(cells)
    res["oracle_elements_checked"] = int(sum(c["checked"] for c in cells))
    res["cells_checked_whole"] = int(sum(c["checked"] == res["elements_per_cell"] for c in cells))
    res["value_mismatches"] = int(sum(c["value_mismatches"] for c in cells))
    res["flag_mismatches"] = int(sum(c["flag_mismatches"] for c in cells))
    res["flag_word_mismatches"] = int(sum(not c.get("flag_word_equal", True) for c in cells))
    res["oracle_s"] = round(t_or[0], 1)
    res["oracle_threads"] = os.cpu_count()
    res["clocks"] = clk.summary()
    return res


def run_reduce(h, suites, args):
    """The reduction suite, then the oracle over each cell's checked prefix."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_lib
    res = suites.reduce(h, n=min(args.n, 1 << 24))
    checks = res.pop("_checks")
    o = oracle_lib.Oracle()
    vp, i, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t
    o.L.sfp_reduce.argtypes = [i, i, i, vp, vp, vp, sz, ctypes.POINTER(ctypes.c_uint32)]
    o.L.sfp_reduce_seg.argtypes = [i, i, i, vp, vp, vp, sz, sz, ctypes.POINTER(ctypes.c_uint32)]
    bad = 0
    for ck in checks:
        d = np.zeros_like(ck["d"])
        fl = ctypes.c_uint32()
        n = ck["a"].shape[0]
        if ck["seg"] == n:
            st = o.L.sfp_reduce(ck["fmt"], ck["op"], 0, ck["a"].ctypes.data, ck["b"].ctypes.data,
                                d.ctypes.data, n, ctypes.byref(fl))
        else:
            st = o.L.sfp_reduce_seg(ck["fmt"], ck["op"], 0, ck["a"].ctypes.data, ck["b"].ctypes.data,
                                    d.ctypes.data, n, ck["seg"], ctypes.byref(fl))
        assert st == 0
        bad += int(not np.array_equal(d, ck["d"]) or fl.value != ck["flags"])
    res["oracle_cells_checked"] = len(checks)
    res["oracle_mismatches"] = bad
    return res


def device_operands(L, fmt, n, seed, stream):
    """a, b, c: n seeded elements each, generated on the device
    (cftg_fill_operands: 90 % normals with exponents in [-64, 64], 10 %
    specials), with exact-cancellation triples and halfway cases planted
    over 4.5 % of the positions (cftgb.workload.plant)."""
    import torch
    import cftgb
    from cftgb import workload as wl
    W = wl.words(fmt)
    ops = [torch.empty(n * W, dtype=torch.int32, device="cuda") for _ in range(3)]
    for j, x in enumerate(ops):
        cftgb._lib.check(L.cftg_fill_operands(fmt, x.data_ptr(), n, seed * 16 + fmt * 4 + j, 64,
                                              100000, stream.cuda_stream), "cftg_fill_operands")
    wl.plant(fmt, ops, n, seed * 16 + fmt)
    torch.cuda.synchronize()
    return ops


def _oracle():
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_lib
    return oracle_lib.Oracle()


def check_against_oracle(fmt, ops, got, got_lf, word, kind=0, op=0, rnd=0):
    """Every element of one launch against the oracle on all host cores:
    values, each element's flag byte, and the launch's flag word."""
    t0 = time.perf_counter()
    rd, rlf, racc = _oracle().run_parallel(kind, fmt, op, rnd, ops[0], ops[1], ops[2])
    return {"elements_checked": int(got.shape[0]),
            "value_mismatches": int(np.count_nonzero((got != rd).any(1))),
            "flag_mismatches": int(np.count_nonzero(got_lf != rlf)),
            "flag_word": word, "oracle_flag_word": racc, "flag_word_equal": word == racc,
            "oracle_s": round(time.perf_counter() - t0, 2), "oracle_threads": os.cpu_count(),
            "_rd": rd}


def check_batch_samples(samples):
    """The batched form's results against the oracle: the first and last
    elements of every call (all of a call of at most twice that many, so
    its ragged last tile too), values; the flag word of each call wholly
    sampled equals the oracle's, and every flag the oracle raises on a
    sampled part of a larger call is in that call's word."""
    from concurrent.futures import ThreadPoolExecutor
    o = _oracle()
    t0 = time.perf_counter()

    def one(s):
        d, _, acc = o.run(s["kind"], s["fmt"], s["op"], s["rnd"], s["a"], s["b"], s["c"])
        vbad = int(np.count_nonzero((d != s["d"]).any(1)))
        fbad = int(acc != s["flags"] & 0x1F) if s["whole"] else int(acc & ~s["flags"] & 0x1F != 0)
        return vbad, fbad, len(d)
    with ThreadPoolExecutor(os.cpu_count() or 1) as ex:
        out = list(ex.map(one, samples))
    return {"calls_checked": len(samples), "elements_checked": int(sum(x[2] for x in out)),
            "calls_wholly_checked": int(sum(s["whole"] for s in samples)),
            "value_mismatches": int(sum(x[0] for x in out)),
            "flag_mismatches": int(sum(x[1] for x in out)),
            "oracle_s": round(time.perf_counter() - t0, 2)}


def slowest(seconds, ws, device="cuda"):
    """The whole job's time: the slowest rank's (an all-reduce MAX over the
    ranks; the path shards by element and exchanges nothing else)."""
    if ws <= 1:
        return seconds
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(seconds)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def run_reference(args):
    ws, rank, _ = dist_init()
    if rank != 0:
        return
    fmt = 3
    a, b, c = (np.ascontiguousarray(x) for x in
               __import__("cftgb.workload", fromlist=["x"]).gen_operands(fmt, 1 << 16, 1))
    # each step is a bounded sample: the whole run stays near 90 s of host work
    step_s = max(0.05, min(2.0, 90.0 / max(1, args.steps + args.warmup)))
    per_step = []
    for _ in range(args.warmup):
        cpu_baseline(fmt, a, b, c, seconds=step_s)
    total, thr = 0, 1
    t_all = 0.0
    for _ in range(args.steps):
        rate, thr, cnt, dt = cpu_baseline(fmt, a, b, c, seconds=step_s)
        per_step.append(dt)
        total += cnt
        t_all += dt
    value = total / t_all / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Gelem/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * t_all / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32-limb binary256", "data": "synthetic",
        "config": {"workload": "binary256 FMA RNE, n=2^24 per GPU, seeded operand mix (90% "
                               "normals exp in [-64,64], 10% specials, cancellation triples)",
                   "elements_per_step": f"{step_s:.2f} s of host work (a bounded sample)",
                   "parallelism": "host threads"},
        "cpu_baseline": {"value": value, "unit": "Gelem/s", "cores": thr, "kind": "port",
                         "sample": f"{step_s:.2f} s per step of 2048-element calls over the first "
                                   "65,536 operands of the same seeded workload"},
        "e2e": {"value": value, "unit": "Gelem/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--profile", action="store_true",
                    help="only the device-resident leg (for ncu captures on a small n)")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="lane-count scale of the trajectories suite (1.0 = 4,096 + 512 lanes)")
    ap.add_argument("--steps-scale", type=float, default=1.0,
                    help="step-range scale of the trajectories suite (1.0 = the configuration)")
    ap.add_argument("--separate", action="store_true",
                    help="trajectories suite: also time each program's launch alone")
    ap.add_argument("--rate", type=float, default=20000.0,
                    help="offered requests a second of the serving suite")
    ap.add_argument("--program-frac", type=float, default=0.02,
                    help="serving suite: fraction of requests that are program ensembles")
    ap.add_argument("--inflight", type=int, default=6,
                    help="serving suite: element batches on the device at once")
    ap.add_argument("--program-inflight", type=int, default=2,
                    help="serving suite: program batches on the device at once")
    ap.add_argument("--elem-blocks-per-sm", type=int, default=0,
                    help="serving suite: work-queue blocks an SM per element batch (0: the server's default, two)")
    ap.add_argument("--seconds", type=float, default=60.0,
                    help="length of the serving suite's request stream")
    ap.add_argument("--serve-seconds", type=float, default=12.0,
                    help="length of the headline run's serving leg (0: leave it out)")
    ap.add_argument("--batch-calls", type=int, default=10000,
                    help="calls of the headline run's batched leg")
    ap.add_argument("--no-batched", action="store_true",
                    help="leave the batched leg out of the headline run")
    ap.add_argument("--fmt", type=int, default=3, help="format of the headline leg (3 = binary256)")
    ap.add_argument("--op", default="fma", choices=["fma", "add", "mul", "div", "sqrt"],
                    help="operation of the --profile leg")
    ap.add_argument("--suite", default=None, choices=["uneven", "trajectories", "sweep", "serving", "reduce", "link",
                                                      "bundles"],
                    help="run one of the secondary configurations instead of the headline")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.suite:
        import torch
        import cftgb
        import bench_suites as suites
        torch.cuda.set_device(0)
        h = cftgb.open_device("cuda:0")
        if args.suite == "trajectories":
            print(json.dumps(run_trajectories(h, suites, args)))
        elif args.suite == "sweep":
            print(json.dumps(run_sweep(h, suites, args)))
        elif args.suite == "reduce":
            print(json.dumps(run_reduce(h, suites, args)))
        elif args.suite == "serving":
            z = np.load(ROOT / "tests" / "golden" / "odes.npz")
            clk = Clocks(0, keep=True)
            try:
                res = suites.serving(h, z["hh_image"], z["hh_bank"], rate=args.rate,
                                     seconds=args.seconds, program_frac=args.program_frac,
                                     max_inflight=args.inflight,
                                     max_program_inflight=args.program_inflight,
                                     elem_blocks_per_sm=args.elem_blocks_per_sm, timed=clk)
            finally:
                clk.close()
            res["clocks"] = clk.summary()
            print(json.dumps(res))
        elif args.suite == "bundles":
            clk = Clocks(0, keep=True)
            try:
                res = suites.bundles(h, timed=clk)
            finally:
                clk.close()
            res["clocks"] = clk.summary()
            mhz = res["clocks"].get("sm_mhz") or 0
            for c in res["cells"]:
                c["cycles_per_bundle"] = c["ns_per_bundle"] * mhz / 1e3 if mhz else None
            print(json.dumps(res))
        elif args.suite == "uneven":
            clk = Clocks(0, keep=True)
            try:
                res = suites.uneven(h, ncalls=args.batch_calls, sample=128, timed=clk)
            finally:
                clk.close()
            res["clocks"] = clk.summary()
            res["oracle"] = check_batch_samples(res.pop("_samples"))
            print(json.dumps(res))
        else:
            print(json.dumps(getattr(suites, args.suite)(h)))
        cftgb.close_device(h)
        return

    import torch
    import cftgb
    from cftgb import algorithmic as alg
    from cftgb import workload as wl
    import bench_suites as suites

    ws, rank, local = dist_init()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev_index = local if ws > 1 else 0
    torch.cuda.set_device(dev_index)
    h = cftgb.open_device(f"cuda:{dev_index}")
    L = cftgb.lib()
    suites._bind(L)
    n = args.n
    fmt = args.fmt
    W = wl.words(fmt)
    stream = torch.cuda.current_stream()
    ta, tb, tc = device_operands(L, fmt, n, 1 + rank, stream)
    td = torch.zeros_like(ta)
    tf = torch.zeros(1, dtype=torch.int32, device="cuda")

    kind_op = {"fma": (0, 0), "add": (0, 1), "mul": (0, 3), "div": (1, 0), "sqrt": (2, 0)}
    pkind, pop = kind_op[args.op] if args.profile else (0, 0)

    def launch(fmt_, A, B, C, D, nn, lf=None, word=tf):
        st = L.cftg_run_device(h, pkind, pop, fmt_, 0, A.data_ptr(), B.data_ptr(), C.data_ptr(),
                               D.data_ptr(), nn, 0, lf, word.data_ptr(), stream.cuda_stream)
        if st:
            cftgb._lib.check(st, "cftg_run_device")

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    # ---- device-resident leg (value, roofline) ----
    for _ in range(max(3, args.warmup)):
        launch(fmt, ta, tb, tc, td, n)
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    tf.zero_()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(dev_index) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            launch(fmt, ta, tb, tc, td, n)
        e1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    if args.profile:
        print(json.dumps({"profile_leg": "device-resident", "fmt": fmt, "op": args.op, "n": n,
                          "ms_per_launch": ms / args.steps,
                          "gelem_s": n * args.steps / (ms / 1e3) / 1e9}))
        cftgb.close_device(h)
        return
    ms = slowest(ms, ws)
    sec = ms / 1e3
    value = ws * n * args.steps / sec / 1e9
    per_launch = sec / args.steps
    hbm_peak, peak_kind = peaks()
    alg_bytes = 4 * 4 * wl.words(fmt) * n
    achieved = alg_bytes / per_launch / 1e9
    timed_word = int(tf.item()) & 0x1F

    # fp128 FMA on the same terms (the metric's second format)
    t2 = device_operands(L, 2, n, 7 + rank, stream)
    td2 = torch.zeros_like(t2[0])
    tf2 = torch.zeros(1, dtype=torch.int32, device="cuda")
    for _ in range(3):
        launch(2, t2[0], t2[1], t2[2], td2, n, word=tf2)
    torch.cuda.synchronize()
    tf2.zero_()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(dev_index) as clk128:
        f0.record(stream)
        for _ in range(args.steps):
            launch(2, t2[0], t2[1], t2[2], td2, n, word=tf2)
        f1.record(stream)
        torch.cuda.synchronize()
    fp128_value = ws * n * args.steps / (slowest(f0.elapsed_time(f1), ws) / 1e3) / 1e9

    # ---- every element of both legs against the oracle (outside the timed
    # regions): values, each element's flags (one more launch with flag
    # bytes) and the timed launches' flag word ----
    parity = {}
    host = {}
    for key, f_, ops, dd, word in (("fp256_fma", fmt, (ta, tb, tc), td, timed_word),
                                   ("fp128_fma", 2, t2, td2, int(tf2.item()) & 0x1F)):
        lf = torch.zeros(n, dtype=torch.uint8, device="cuda")
        d_chk = torch.empty_like(dd)
        w_chk = torch.zeros(1, dtype=torch.int32, device="cuda")
        launch(f_, ops[0], ops[1], ops[2], d_chk, n, lf.data_ptr(), w_chk)
        torch.cuda.synchronize()
        same_as_timed = bool(torch.equal(d_chk, dd))
        ha = [x.cpu().numpy().view(np.uint32).reshape(n, -1) for x in ops]
        got, glf = dd.cpu().numpy().view(np.uint32).reshape(n, -1), lf.cpu().numpy()
        del d_chk, lf
        if args.no_cpu:
            parity[key] = {"elements_checked": 0}
            host[key] = ha
            continue
        parity[key] = check_against_oracle(f_, ha, got, glf, word)
        parity[key]["timed_output_equals_checked_launch"] = same_as_timed
        host[key] = ha
        host[key + "_oracle"] = parity[key].pop("_rd")
    del t2, td2

    # ---- end-to-end leg through cft_run with pinned host buffers ----
    ha, hb, hc = (torch.from_numpy(x.view(np.int32)).pin_memory() for x in host["fp256_fma"])
    hd = torch.zeros_like(ha).pin_memory()
    fl = ctypes.c_uint32()
    for _ in range(max(2, args.warmup // 2)):
        L.cft_run(h, 0, fmt, 0, ha.data_ptr(), hb.data_ptr(), hc.data_ptr(), hd.data_ptr(), n,
                  ctypes.byref(fl), None)
    e2e_steps = max(3, args.steps // 4)
    barrier()
    with Clocks(dev_index) as clk_e2e:
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            st = L.cft_run(h, 0, fmt, 0, ha.data_ptr(), hb.data_ptr(), hc.data_ptr(), hd.data_ptr(),
                           n, ctypes.byref(fl), None)
            cftgb._lib.check(st, "cft_run")
        e2e_sec = slowest(time.perf_counter() - t0, ws)
    e2e_value = ws * n * e2e_steps / e2e_sec / 1e9
    e2e_parity = {"elements_checked": 0}
    if "fp256_fma_oracle" in host:
        got = hd.numpy().view(np.uint32).reshape(n, -1)
        rd = host["fp256_fma_oracle"]
        e2e_parity = {"elements_checked": n,
                      "value_mismatches": int(np.count_nonzero((got != rd).any(1))),
                      "flag_word_equal": fl.value == parity["fp256_fma"]["oracle_flag_word"]}

    cpu = None
    if rank == 0 and not args.no_cpu:
        a, b, c = (x[:1 << 16] for x in host["fp256_fma"])
        rate, thr, cnt, dt = cpu_baseline(fmt, a, b, c)
        cpu = {"value": rate / 1e9, "unit": "Gelem/s", "cores": thr, "kind": "port",
               "sample": f"{cnt} elements ({dt:.1f} s) of the same operands in 2048-element calls"}
    del ha, hb, hc, hd, host, ta, tb, tc, td
    torch.cuda.empty_cache()

    # ---- the batched form against plain launches (the uneven batch) ----
    batched = None
    if not args.no_batched:
        clk_b = Clocks(dev_index, keep=True)
        try:
            res = suites.uneven(h, ncalls=args.batch_calls, sample=0 if args.no_cpu else 128,
                                timed=clk_b)
        finally:
            clk_b.close()
        batched = {k: res[k] for k in ("calls", "elements", "plain_ms", "batched_ms",
                                       "plain_gelem_s", "batched_gelem_s", "bit_exact_vs_plain",
                                       "tiles", "autotune_s", "block_threads")}
        batched["batched_vs_plain"] = res["speedup"]
        batched["clocks"] = clk_b.summary()
        if "_samples" in res:
            batched["oracle"] = check_batch_samples(res["_samples"])
        torch.cuda.empty_cache()

    # ---- serving: a Poisson request stream, latency percentiles ----
    serving = None
    if args.serve_seconds > 0:
        z = np.load(ROOT / "tests" / "golden" / "odes.npz")
        clk_s = Clocks(dev_index, keep=True)
        try:
            res = suites.serving(h, z["hh_image"], z["hh_bank"], rate=args.rate,
                                 seconds=args.serve_seconds, program_frac=args.program_frac,
                                 max_inflight=args.inflight,
                                 max_program_inflight=args.program_inflight,
                                 elem_blocks_per_sm=args.elem_blocks_per_sm, timed=clk_s)
        finally:
            clk_s.close()
        serving = {k: res[k] for k in ("offered_req_s", "seconds", "requests", "program_requests",
                                       "completed", "failed", "served_gelem_s",
                                       "program_lane_steps_per_s", "samples_checked",
                                       "bit_exact_alone_vs_mix", "bytes_peak", "budget")}
        for k in ("latency_all", "latency_elem", "latency_program"):
            serving[k] = {q: round(v, 4) for q, v in res[k].items()}
        serving["p50_ms"] = res["latency_all"].get("p50_ms")
        serving["p99_ms"] = res["latency_all"].get("p99_ms")
        serving["clocks"] = clk_s.summary()
        torch.cuda.empty_cache()

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Gelem/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u32-limb binary256", "data": "synthetic",
            "config": {"workload": "binary256 FMA RNE, n=2^24 per GPU, seeded operand mix (90% "
                                   "normals exp in [-64,64], 10% specials, 2.25% exact-cancellation "
                                   "triples, 2.25% halfway cases)",
                       "elements_per_gpu": n, "l2": "inputs 1.5 GiB > L2, no flush",
                       "parallelism": f"replicas x{ws} (element shards)"},
            "e2e": {"value": e2e_value, "unit": "Gelem/s", "h2d_bytes_per_step": 3 * 4 * W * n,
                    "d2h_bytes_per_step": 4 * W * n + 8, "path": "cft_run, pinned host buffers",
                    "steps": e2e_steps, "parity": e2e_parity, "clocks": clk_e2e.summary(),
                    "link_bound_gelem_s": LINK_READ_GBS / (3 * 4 * W),
                    "link_note": f"the kernel reads the operands in host memory in place; GPU "
                                 f"reads of pinned host memory top out at {LINK_READ_GBS:.0f} GB/s "
                                 f"on this host (bench.py --suite link), so e2e is bound at "
                                 f"{LINK_READ_GBS / (3 * 4 * W):.2f} Gelem/s"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak,
                         "traffic": (TRAFFIC_B_PER_ELEM[fmt] * n) if fmt in TRAFFIC_B_PER_ELEM else None,
                         "traffic_source": "dram read+write bytes per element of one ncu capture "
                                           "(n = 4,194,304) scaled to n",
                         "peak_source": peak_kind,
                         "note": f"integer-pipe bound kernel: algorithmic {4 * 4 * wl.words(fmt)} "
                                 "B/element"},
            "int_pipe": {"alg_ops_per_elem": alg.int_ops(fmt, "fma"),
                         "achieved_tops": value / ws * alg.int_ops(fmt, "fma") / 1e3,
                         "issue_peak_tops": alg.int_issue_peak_tops(),
                         "frac": value / ws * alg.int_ops(fmt, "fma") / 1e3 / alg.int_issue_peak_tops(),
                         "note": "algorithmic integer operations (2L^2 product halves + 8L) over "
                                 "the nominal issue rate 152 SMs x 128 lanes x 2070 MHz; no "
                                 "measured integer peak exists"},
            "cpu_baseline": cpu,
            "gpu_launches": args.steps,
            "clocks": clk.summary(),
            "fp128_fma_gelem_s": fp128_value,
            "fp128_clocks": clk128.summary(),
            "parity": parity,
            "batched": batched,
            "serving": serving,
        }
        print(json.dumps(line))
    cftgb.close_device(h)
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
