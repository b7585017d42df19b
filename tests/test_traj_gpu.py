"""The batched sequencer (cftg_traj_*): uneven trajectories of the fp256
Lorenz-63 RK4 segment program as one launch (and as a replayed graph),
against the oracle running the same segments one run at a time, and
against the reference's certificate for three segments."""
import ctypes
import hashlib

import numpy as np
import pytest

import cftgb
import oracle_lib
import seq_util as su
from cftgb import workload as wl

pytestmark = pytest.mark.gpu
TAG = b"cft-certificate 1 state\0"


def _bind(L):
    vp = ctypes.c_void_p
    L.cftg_traj_create.argtypes = [vp, vp, ctypes.c_size_t, vp, vp, vp, vp, vp, vp,
                                   ctypes.c_uint32, ctypes.c_uint32, vp, ctypes.POINTER(vp)]
    L.cftg_traj_launch.argtypes = [vp, vp]
    L.cftg_traj_capture.argtypes = [vp, vp]
    L.cftg_traj_result.argtypes = [vp, vp, vp, vp]
    L.cftg_traj_free.argtypes = [vp]


def _traj(h, img, bank, state, segs, snap_every, max_snaps, graph=False):
    import torch
    L = cftgb.lib()
    _bind(L)
    n = len(segs)
    prog = ctypes.c_void_p()
    cftgb._lib.check(L.cft_program_load(h, img.ctypes.data, img.size, ctypes.byref(prog)), "load")
    W = state.shape[1]
    ta = torch.zeros((n, W), dtype=torch.int32, device="cuda")
    tbank = torch.from_numpy(bank.view(np.int32).copy()).cuda()
    tstate = torch.from_numpy(state.view(np.int32).copy()).cuda()
    slots = state.shape[0] // n
    tsnap = torch.zeros((n * max_snaps * slots, W), dtype=torch.int32, device="cuda")
    tlf = torch.zeros(n, dtype=torch.uint8, device="cuda")
    sg = np.asarray(segs, np.uint32)
    t = ctypes.c_void_p()
    cftgb._lib.check(L.cftg_traj_create(prog, sg.ctypes.data, n, ta.data_ptr(), None, None,
                                        tbank.data_ptr(), tstate.data_ptr(), tsnap.data_ptr(),
                                        snap_every, max_snaps, tlf.data_ptr(), ctypes.byref(t)),
                     "cftg_traj_create")
    s = torch.cuda.Stream()
    if graph:
        cftgb._lib.check(L.cftg_traj_capture(t, s.cuda_stream), "capture")
    cftgb._lib.check(L.cftg_traj_launch(t, s.cuda_stream), "launch")
    fl, st = ctypes.c_uint32(), ctypes.c_uint32()
    cftgb._lib.check(L.cftg_traj_result(t, ctypes.byref(fl), ctypes.byref(st), s.cuda_stream), "result")
    L.cftg_traj_free(t)
    L.cft_program_free(prog)
    return (tstate.cpu().numpy().view(np.uint32), tsnap.cpu().numpy().view(np.uint32),
            tlf.cpu().numpy(), fl.value, st.value)


def test_certificate_segments_as_one_trajectory_launch(gpu):
    z = np.load(su.GOLD / "lorenz63_cert.npz")
    state = z["state0"].copy().view(np.uint32).reshape(-1, 8)
    n = state.shape[0] // 3
    segs = [len(z["ends"])] * n
    final, snaps, lf, fl, st = _traj(gpu, z["image"].copy(), z["bank"].copy(), state, segs, 1, 3)
    snaps = snaps.reshape(n, 3, 3, 8)
    for k, end in enumerate(z["ends"]):
        blk = snaps[:, k].reshape(-1, 8)          # lane-major block after segment k
        assert hashlib.sha256(TAG + blk.tobytes()).hexdigest() == str(end), k
    assert hashlib.sha256(TAG + final.tobytes()).hexdigest() == str(z["ends"][-1])
    assert fl == int(np.bitwise_or.reduce(z["flags"])) and st == 0


@pytest.fixture(params=["auto", "1", "2", "4", "32", "8c", "32c"])
def lane_threads(request, monkeypatch):
    """Threads a lane for the trajectory launches: the planner's choice, or
    forced (1 = the plain interpreter, else the bundle schedule; "c": with
    the cooperative binary128/256 arithmetic, W threads an operation)."""
    if request.param != "auto":
        monkeypatch.setenv("CFTG_LANE_THREADS", request.param.rstrip("c"))
        monkeypatch.setenv("CFTG_LANE_COOP", "1" if request.param.endswith("c") else "0")
    return request.param


@pytest.mark.parametrize("graph", [False, True])
def test_uneven_trajectories_match_oracle(gpu, oracle, graph, lane_threads):
    z = np.load(su.GOLD / "lorenz63_cert.npz")
    img, bank = z["image"].copy(), z["bank"].copy()
    rng = np.random.default_rng(5)
    n = 37
    init = np.zeros((n * 3, 8), np.uint32)
    for i in range(n):
        for j in range(3):
            init[i * 3 + j] = wl.from_int(wl.encode_double(3, 1.0 + rng.normal(0, 1e-3)), 8)
    segs = rng.integers(1, 7, n).tolist()
    final, snaps, lf, fl, st = _traj(gpu, img, bank, init, segs, 2, 3, graph=graph)
    snaps = snaps.reshape(n, 3, 3, 8)
    # the oracle: each lane's segments one run at a time
    acc = 0
    for i in range(n):
        s = init[i * 3:(i + 1) * 3].copy()
        for k in range(segs[i]):
            out = np.zeros_like(s)
            A = oracle_lib.SeqArgs()
            a = np.zeros((1, 8), np.uint32)
            A.a, A.n, A.bank = a.ctypes.data, 1, bank.ctypes.data
            A.scratch_in, A.scratch_out, A.depth = s.ctypes.data, out.ctypes.data, 256
            assert oracle.L.sfp_seq_run(img.ctypes.data, img.size, ctypes.byref(A)) == 0
            acc |= A.flags_out
            s = out
            if (k + 1) % 2 == 0:
                assert np.array_equal(snaps[i, (k + 1) // 2 - 1], s), (i, k)
        assert np.array_equal(final[i * 3:(i + 1) * 3], s), i
    assert fl == acc


def test_group_launch_two_programs_two_formats(gpu, oracle, lane_threads):
    """Lorenz-63 at binary256 and Lorenz-96 at binary128, uneven run counts,
    as one graph launch (cftg_traj_group_*): every kept state's hash and
    every final state equal the oracle's segment-by-segment runs."""
    import bench_suites as suites
    z = np.load(su.GOLD / "odes.npz")
    progs = []
    for i, (key, fmt, slots, base, spr, lanes, every) in enumerate(
            (("l63", 3, 3, 1.0, 100, 45, 2), ("l96", 2, 40, 8.0, 20, 5, 3))):
        init, runs = suites.ode_lanes(key, fmt, lanes, slots, base, (spr, 8 * spr), spr, 7 + i)
        progs.append(dict(name=key, image=z[key + "_image"], bank=z[key + "_bank"], fmt=fmt,
                          slots=slots, init=init, runs=runs, snap_every=every,
                          max_snaps=int(runs.max()) // every + 1, steps_per_run=spr))
    res = suites.trajectories(gpu, progs, reps=2)
    for P, R in zip(progs, res["programs"]):
        W = wl.words(P["fmt"])
        slots = P["slots"]
        img, bank = P["image"].copy(), P["bank"].copy()
        acc = 0
        for lane in range(len(P["runs"])):
            s = P["init"][lane * slots:(lane + 1) * slots].copy()
            for k in range(int(P["runs"][lane])):
                out = np.zeros_like(s)
                A = oracle_lib.SeqArgs()
                a = np.zeros((1, W), np.uint32)
                A.a, A.n, A.bank = a.ctypes.data, 1, bank.ctypes.data
                A.scratch_in, A.scratch_out, A.depth = s.ctypes.data, out.ctypes.data, 256
                assert oracle.L.sfp_seq_run(img.ctypes.data, img.size, ctypes.byref(A)) == 0
                acc |= A.flags_out
                s = out
                if (k + 1) % P["snap_every"] == 0:
                    j = (k + 1) // P["snap_every"] - 1
                    assert hashlib.sha256(TAG + s.tobytes()).digest() == R["_hashes"][lane][j]
            assert np.array_equal(R["_final"][lane * slots:(lane + 1) * slots], s), (P["name"], lane)
        assert R["flags"] == acc and R["status"] == 0
