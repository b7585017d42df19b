"""The serving loop (cftg_server_*): mixed element and program requests
admitted under a device-memory budget and batched as they arrive; every
result (bits and flags) must equal the same request run alone."""
import ctypes

import numpy as np
import pytest

import cftgb
import seq_util as su
from cftgb import serving, workload as wl

pytestmark = pytest.mark.gpu

OPS = (("add", 0, 1), ("sub", 0, 2), ("mul", 0, 3), ("fma", 0, 0), ("div", 1, 0), ("sqrt", 2, 0))


def hh_init(lanes, seed):
    """Henon-Heiles initial blocks (x, y, px, py) at energy 1/8: x = 0, y and
    py drawn, px from the energy (in double), widened exactly to binary256."""
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


def _bind_traj(L):
    vp = ctypes.c_void_p
    L.cftg_traj_create.argtypes = [vp, vp, ctypes.c_size_t, vp, vp, vp, vp, vp, vp,
                                   ctypes.c_uint32, ctypes.c_uint32, vp, ctypes.POINTER(vp)]
    L.cftg_traj_launch.argtypes = [vp, vp]
    L.cftg_traj_result.argtypes = [vp, vp, vp, vp]
    L.cftg_traj_free.argtypes = [vp]


def traj_alone(prog, bank, init, lanes, runs):
    import torch
    L = cftgb.lib()
    _bind_traj(L)
    ta = torch.zeros(lanes * 8, dtype=torch.int32, device="cuda")
    ts = torch.from_numpy(init.view(np.int32).copy()).cuda()
    lf = torch.zeros(lanes, dtype=torch.uint8, device="cuda")
    segs = np.full(lanes, runs, np.uint32)
    t = ctypes.c_void_p()
    cftgb._lib.check(L.cftg_traj_create(prog, segs.ctypes.data, lanes, ta.data_ptr(), None, None,
                                        bank.data_ptr(), ts.data_ptr(), None, 0, 0, lf.data_ptr(),
                                        ctypes.byref(t)), "cftg_traj_create")
    s = torch.cuda.current_stream().cuda_stream
    cftgb._lib.check(L.cftg_traj_launch(t, s), "launch")
    fl, st = ctypes.c_uint32(), ctypes.c_uint32()
    cftgb._lib.check(L.cftg_traj_result(t, ctypes.byref(fl), ctypes.byref(st), s), "result")
    L.cftg_traj_free(t)
    return ts.cpu().numpy().view(np.uint32), int(np.bitwise_or.reduce(lf.cpu().numpy() & 0x1F)), st.value


def test_program_requests_match_the_oracle(gpu, oracle):
    """Program requests through the server against the oracle run segment
    by segment (so that a difference between the mix and a run alone can be
    placed)."""
    import torch
    import oracle_lib
    L = cftgb.lib()
    z = np.load(su.GOLD / "odes.npz")
    img = z["hh_image"].copy()
    hbank = z["hh_bank"].copy()
    prog = ctypes.c_void_p()
    cftgb._lib.check(L.cft_program_load(gpu, img.ctypes.data, img.size, ctypes.byref(prog)), "load")
    bank = torch.from_numpy(hbank.view(np.int32).copy()).cuda()
    rng = np.random.default_rng(3)
    reqs, outs, meta = [], [], []
    for i in range(4):
        lanes, runs = int(rng.integers(3, 12)), int(rng.integers(1, 4))
        init = hh_init(lanes, 500 + i)
        out = torch.zeros(init.nbytes, dtype=torch.uint8, pin_memory=True)
        reqs.append(serving.Request(type=serving.REQ_PROGRAM, prog=prog, d_bank=bank.data_ptr(),
                                    init=init.ctypes.data, lanes=lanes, runs=runs,
                                    host_out=out.data_ptr(), tag=i))
        outs.append(out)
        meta.append((init, lanes, runs))
    with serving.Server(gpu, 1 << 24, max_inflight=1, max_program_inflight=1) as srv:
        for r in reqs:
            assert srv.submit(r) == 0
        assert srv.drain() == 0
        done = srv.poll()
    assert len(done) == 4 and (done["result"] == 0).all()
    flags = {int(t): int(f) for t, f in zip(done["tag"], done["flags"])}
    a = np.zeros((1, 8), np.uint32)
    for i, (init, lanes, runs) in enumerate(meta):
        mix = outs[i].numpy().view(np.uint32).reshape(lanes, 4, 8)
        acc = 0
        for j in range(lanes):
            s = init[j * 4:(j + 1) * 4].copy()
            for _ in range(runs):
                o = np.zeros_like(s)
                A = oracle_lib.SeqArgs()
                A.a, A.n, A.bank = a.ctypes.data, 1, hbank.ctypes.data
                A.scratch_in, A.scratch_out, A.depth = s.ctypes.data, o.ctypes.data, 256
                assert oracle.L.sfp_seq_run(img.ctypes.data, img.size, ctypes.byref(A)) == 0
                acc |= A.flags_out
                s = o
            assert np.array_equal(mix[j], s), f"request {i} lane {j} of {lanes}, {runs} runs"
        assert flags[i] == acc
    L.cft_program_free(prog)


def test_mixed_requests_same_alone_and_in_the_mix(gpu):
    import torch
    L = cftgb.lib()
    import bench_suites as suites
    suites._bind(L)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(21)
    P = 1 << 16
    pools = {}
    for fmt in (2, 3):
        W = wl.words(fmt)
        pools[fmt] = [torch.empty(P * W, dtype=torch.int32, device="cuda") for _ in range(3)]
        for j in range(3):
            cftgb._lib.check(L.cftg_fill_operands(fmt, pools[fmt][j].data_ptr(), P, 50 + fmt * 3 + j,
                                                  64, 100000, stream), "fill")
    z = np.load(su.GOLD / "odes.npz")
    img = z["hh_image"].copy()
    prog = ctypes.c_void_p()
    cftgb._lib.check(L.cft_program_load(gpu, img.ctypes.data, img.size, ctypes.byref(prog)), "load")
    bank = torch.from_numpy(z["hh_bank"].view(np.int32).copy()).cuda()
    torch.cuda.synchronize()

    budget = 3 << 19                          # 1.5 MiB: admission has to wait for memory
    reqs, outs, meta = [], [], []
    for i in range(60):
        fmt = int(rng.choice([2, 3]))
        n = int(np.exp(rng.uniform(0, np.log(20000))))
        name, kind, op = OPS[int(rng.integers(0, 6))]
        rnd = int(rng.integers(0, 5))
        off = int(rng.integers(0, P - n))
        esz = 4 * wl.words(fmt)
        pa, pb, pc = (x.data_ptr() + off * esz for x in pools[fmt])
        out = torch.zeros(n * esz, dtype=torch.uint8, pin_memory=True)
        r = serving.Request(type=serving.REQ_ELEM, kind=kind, op=op, fmt=fmt, rnd=rnd, d_a=pa,
                            d_b=pb, d_c=pc, n=n, host_out=out.data_ptr(), tag=i)
        reqs.append(r)
        outs.append(out)
        meta.append(("elem", kind, op, fmt, rnd, pa, pb, pc, n))
    for i in range(6):
        lanes, runs = int(rng.integers(5, 41)), int(rng.integers(1, 7))
        init = hh_init(lanes, 300 + i)
        out = torch.zeros(init.nbytes, dtype=torch.uint8, pin_memory=True)
        r = serving.Request(type=serving.REQ_PROGRAM, prog=prog, d_bank=bank.data_ptr(),
                            init=init.ctypes.data, lanes=lanes, runs=runs, host_out=out.data_ptr(),
                            tag=100 + i)
        reqs.append(r)
        outs.append(out)
        meta.append(("prog", init, lanes, runs))
    order = rng.permutation(len(reqs))
    with serving.Server(gpu, budget, max_inflight=3, max_program_inflight=2,
                        max_batch_calls=8) as srv:
        for k in order:
            assert srv.submit(reqs[k]) == 0, k
        # a request larger than the whole budget is refused at submit
        big = serving.Request(type=serving.REQ_ELEM, kind=0, op=0, fmt=3, rnd=0, d_a=pools[3][0].data_ptr(),
                              d_b=pools[3][1].data_ptr(), d_c=pools[3][2].data_ptr(), n=P, tag=999)
        assert srv.submit(big) == 6           # CFT_ERR_OUT_OF_MEMORY
        assert srv.drain() == 0
        done = srv.poll()
        st = srv.stats()
    assert len(done) == len(reqs) and (done["result"] == 0).all()
    assert st["bytes_peak"] <= budget and st["batches"] > 1 and st["completed"] == len(reqs)
    flags = {int(t): int(f) for t, f in zip(done["tag"], done["flags"])}
    status = {int(t): int(s) for t, s in zip(done["tag"], done["status"])}
    word = torch.zeros(1, dtype=torch.int32, device="cuda")
    for i, m in enumerate(meta):
        tag = int(reqs[i].tag)
        if m[0] == "elem":
            _, kind, op, fmt, rnd, pa, pb, pc, n = m
            d = torch.zeros(n * 4 * wl.words(fmt), dtype=torch.uint8, device="cuda")
            word.zero_()
            st_ = L.cftg_run_device(gpu, kind, op, fmt, rnd, pa, pb, pc, d.data_ptr(), n, 0, None,
                                    word.data_ptr(), stream)
            assert st_ == 0
            torch.cuda.synchronize()
            assert torch.equal(d.cpu(), outs[i]), f"request {tag}: bits differ from the call alone"
            assert flags[tag] == int(word.item()) & 0x1F, f"request {tag}: flags"
        else:
            _, init, lanes, runs = m
            final, fl, stt = traj_alone(prog, bank, init, lanes, runs)
            mix = outs[i].numpy().view(np.uint32).reshape(lanes, -1)
            alone = final.reshape(lanes, -1)
            diff = [j for j in range(lanes) if not np.array_equal(mix[j], alone[j])]
            assert not diff, f"program request {tag} ({lanes} lanes, {runs} runs): lanes {diff} differ"
            assert flags[tag] == fl and status[tag] == stt == 0, (tag, flags[tag], fl, status[tag], stt)
    L.cft_program_free(prog)


def test_short_program_request_completes_before_its_batch(gpu):
    """A short ensemble batched with a long one completes when its own lanes
    have finished (its completion time is before the long one's), and both
    results equal the same requests run alone; so does a request whose
    output is pageable host memory (written by the kernel where the GPU
    walks the host's page tables, else copied when its batch completes)."""
    import torch
    L = cftgb.lib()
    z = np.load(su.GOLD / "odes.npz")
    img = z["hh_image"].copy()
    prog = ctypes.c_void_p()
    cftgb._lib.check(L.cft_program_load(gpu, img.ctypes.data, img.size, ctypes.byref(prog)), "load")
    bank = torch.from_numpy(z["hh_bank"].copy().view(np.int32)).cuda()
    # lanes, runs, pinned output; the first request occupies the one program
    # slot while the other three queue, so those three form one batch
    plan = [(32, 60, True), (32, 2, True), (32, 120, True), (8, 3, False)]
    reqs, outs, inits = [], [], []
    for i, (lanes, runs, pinned) in enumerate(plan):
        init = hh_init(lanes, 900 + i)
        out = (torch.zeros(init.nbytes, dtype=torch.uint8, pin_memory=True) if pinned
               else np.zeros(init.nbytes, np.uint8))
        ptr = out.data_ptr() if pinned else out.ctypes.data
        reqs.append(serving.Request(type=serving.REQ_PROGRAM, prog=prog, d_bank=bank.data_ptr(),
                                    init=init.ctypes.data, lanes=lanes, runs=runs,
                                    host_out=ptr, tag=i))
        outs.append(out)
        inits.append(init)
    import time
    with serving.Server(gpu, 1 << 26, max_inflight=1, max_program_inflight=1) as srv:
        assert srv.submit(reqs[0]) == 0
        t_end = time.time() + 10
        while srv.stats()["batches"] < 1 and time.time() < t_end:   # the first is on the device
            time.sleep(0.0005)
        for r in reqs[1:]:
            assert srv.submit(r) == 0
        assert srv.drain() == 0
        done = srv.poll()
    assert len(done) == 4 and (done["result"] == 0).all()
    by = {int(d["tag"]): d for d in done}
    assert by[1]["batch"] == by[2]["batch"] == by[3]["batch"] != by[0]["batch"]
    assert by[1]["t_done_ns"] < by[2]["t_done_ns"]
    for i, (lanes, runs, pinned) in enumerate(plan):
        got = (outs[i].numpy() if pinned else outs[i]).view(np.uint32)
        want, fl, st = traj_alone(prog, bank, inits[i], lanes, runs)
        assert np.array_equal(got.reshape(-1), want.reshape(-1)), f"request {i}"
        assert int(by[i]["flags"]) == fl and int(by[i]["status"]) == st
    L.cft_program_free(prog)
