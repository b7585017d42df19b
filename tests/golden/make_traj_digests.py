"""Generate tests/golden/traj_digests.npz: the trajectory workload's expected
results for EVERY lane, computed by the reference library itself
(oracle/_ref/libcft_ref.so, built from the reference's own sources by
`make -C oracle ref`, software backend) - run here, where the reference
tree is present:

    make -C oracle ref
    python tests/golden/make_traj_digests.py [THREADS]

The workload is bench.py's trajectory configuration (ode_programs(), the
same seeded initial states and run counts): 4,096 Lorenz-63 RK4 lanes at
binary256 (h = 0.01, 1e3..1e5 steps) and 512 Lorenz-96 RK4 lanes at
binary128 (N = 40, F = 8, h = 0.005, 1e3..1e4 steps), images and banks
from tests/golden/odes.npz. Each lane runs segment by segment as the
reference's host/tools/segrun.c runs a trajectory: one
cft_program_run_ex a segment (the image's REPEAT count of steps), its
scratch-out fed back as the next segment's scratch-in. Lanes run
together, a call over every lane still running, split over threads with a
handle each (a handle is not thread-safe).

Per program and lane it stores:
  * final: SHA-256 of the certificate tag and the lane's final state;
  * kept: SHA-256 over the concatenated tagged SHA-256 of every state kept
    on the way (one every 1,000 steps: every 10 Lorenz-63 segments, every
    50 Lorenz-96 segments);
  * flags: the IEEE flags the lane's runs raised, ORed.
The GPU's trajectory launch must reproduce all three for every lane
(bench.py --suite trajectories).
"""
import ctypes
import hashlib
import os
import sys
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "cft-fp256_gb300"))
sys.path.insert(0, str(ROOT / "tests" / "golden"))

import bench  # noqa: E402  (the workload's definition)
import bench_suites  # noqa: E402
from make_programs import RunArgs, header, lib  # noqa: E402

OUT = ROOT / "tests" / "golden" / "traj_digests.npz"


def run_lanes(P, lanes, log):
    """One thread's share of a program's lanes, on its own handle."""
    L = lib()
    dev = ctypes.c_void_p()
    assert L.cft_open(None, 0, ctypes.byref(dev)) == 0
    img = np.ascontiguousarray(P["image"])
    prog = ctypes.c_void_p()
    assert L.cft_program_load(dev, img.ctypes.data, img.size, ctypes.byref(prog)) == 0, \
        L.cft_last_error()
    h = header(bytes(img[:32]))
    W = (1, 2, 4, 8)[h["prec"]]
    slots = P["slots"]
    assert h["sin"] == slots and h["sout"] == slots
    bank = np.ascontiguousarray(P["bank"])
    runs = P["runs"][lanes].astype(np.int64)
    state = np.ascontiguousarray(P["init"].reshape(-1, slots, W)[lanes])
    kept = [hashlib.sha256() for _ in lanes]
    flags = np.zeros(len(lanes), np.uint32)
    for k in range(int(runs.max())):
        act = np.nonzero(runs > k)[0]
        n = len(act)
        sin = np.ascontiguousarray(state[act])
        sout = np.zeros_like(sin)
        a = np.zeros((n, W), np.uint32)
        lf = np.zeros(n, np.uint8)
        fl, bus = ctypes.c_uint32(), ctypes.c_uint32()
        A = RunArgs()
        A.struct_size = ctypes.sizeof(RunArgs)
        A.a, A.n = a.ctypes.data, n
        A.bank, A.bank_bytes = bank.ctypes.data, bank.nbytes
        A.scratch_in, A.scratch_in_bytes = sin.ctypes.data, sin.nbytes
        A.scratch_out, A.scratch_out_bytes = sout.ctypes.data, sout.nbytes
        A.flags_out, A.bus_out = ctypes.pointer(fl), ctypes.pointer(bus)
        A.lane_flags, A.lane_flags_bytes = lf.ctypes.data, n
        st = L.cft_program_run_ex(prog, ctypes.byref(A))
        assert st == 0, L.cft_last_error()
        state[act] = sout
        flags[act] |= lf & 0x1F
        if (k + 1) % P["snap_every"] == 0:
            for j in act:
                kept[j].update(hashlib.sha256(bench_suites.TAG + state[j].tobytes()).digest())
        if k % 200 == 0:
            log(f"{P['name']}: segment {k} of {int(runs.max())}, {n} lanes running")
    L.cft_program_free(prog)
    final = [hashlib.sha256(bench_suites.TAG + state[j].tobytes()).digest()
             for j in range(len(lanes))]
    return lanes, final, [x.digest() for x in kept], flags


def main(threads):
    progs = bench.ode_programs()
    out = {}
    t0 = time.time()

    def log(msg):
        print(f"[{time.time() - t0:7.1f} s] {msg}", flush=True)
    for i, P in enumerate(progs):
        n = len(P["runs"])
        # interleave lanes over threads so each gets long and short ones
        shares = [np.arange(t, n, threads) for t in range(threads)]
        final = np.zeros((n, 32), np.uint8)
        kept = np.zeros((n, 32), np.uint8)
        flags = np.zeros(n, np.uint32)
        with ThreadPoolExecutor(threads) as ex:
            for lanes, f, k, fl in ex.map(lambda s: run_lanes(P, s, log), shares):
                final[lanes] = np.frombuffer(b"".join(f), np.uint8).reshape(-1, 32)
                kept[lanes] = np.frombuffer(b"".join(k), np.uint8).reshape(-1, 32)
                flags[lanes] = fl
        out[f"p{i}_final"] = final
        out[f"p{i}_kept"] = kept
        out[f"p{i}_flags"] = flags
        out[f"p{i}_runs"] = P["runs"]
        out[f"p{i}_name"] = np.array(P["name"])
        log(f"{P['name']}: {n} lanes done")
    np.savez_compressed(OUT, **out)
    log(f"wrote {OUT}")


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 1))
