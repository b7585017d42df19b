"""The batched form: many uneven calls of mixed formats, operations and
rounding attributes as one persistent work-queue launch (and as a replayed
CUDA graph) give exactly the bits and per-call flags of one plain launch a
call."""
import ctypes

import numpy as np
import pytest

import cftgb
from cftgb import workload as wl

pytestmark = pytest.mark.gpu


class Call(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("op", ctypes.c_int), ("fmt", ctypes.c_int),
                ("rnd", ctypes.c_int), ("a", ctypes.c_void_p), ("b", ctypes.c_void_p),
                ("c", ctypes.c_void_p), ("d", ctypes.c_void_p), ("n", ctypes.c_size_t),
                ("scalar_mask", ctypes.c_uint32)]


@pytest.mark.parametrize("threads", [256, 128])
def test_queue_matches_plain_launches(gpu, threads):
    """at both block shapes the autotuner chooses between"""
    import torch
    L = cftgb.lib()
    before = L.cftg_queue_block_threads()
    cftgb._lib.check(L.cftg_set_queue_block_threads(threads), "cftg_set_queue_block_threads")
    try:
        _queue_matches_plain(gpu, L)
    finally:
        cftgb._lib.check(L.cftg_set_queue_block_threads(before), "cftg_set_queue_block_threads")


def _queue_matches_plain(gpu, L):
    import torch
    vp = ctypes.c_void_p
    L.cftg_batch_create.argtypes = [vp, ctypes.POINTER(Call), ctypes.c_size_t, vp, ctypes.POINTER(vp)]
    L.cftg_batch_launch.argtypes = [vp, vp]
    L.cftg_batch_capture.argtypes = [vp, vp]
    L.cftg_batch_free.argtypes = [vp]
    rng = np.random.default_rng(4)
    ncalls = 300
    calls = (Call * ncalls)()
    keep = []
    outs_plain, outs_q = [], []
    plain_flags = []
    stream = torch.cuda.current_stream().cuda_stream
    for i in range(ncalls):
        fmt = int(rng.choice([1, 2, 3], p=[0.2, 0.4, 0.4]))
        n = int(np.exp(rng.uniform(0, np.log(20000))))
        kind, op = [(0, 1), (0, 3), (0, 0), (1, 0), (2, 0)][int(rng.integers(0, 5))]
        rnd = int(rng.integers(0, 5))
        a, b, c = wl.gen_operands(fmt, n, 1000 + i, triples_frac=0.0)
        ta, tb, tc = (torch.from_numpy(x.view(np.int32)).cuda() for x in (a, b, c))
        td1, td2 = torch.zeros_like(ta), torch.zeros_like(ta)
        fw = torch.zeros(1, dtype=torch.int32, device="cuda")
        st = L.cftg_run_device(gpu, kind, op, fmt, rnd, ta.data_ptr(), tb.data_ptr(), tc.data_ptr(),
                               td1.data_ptr(), n, 0, None, fw.data_ptr(), stream)
        cftgb._lib.check(st, "cftg_run_device")
        calls[i] = Call(kind, op, fmt, rnd, ta.data_ptr(), tb.data_ptr(), tc.data_ptr(),
                        td2.data_ptr(), n, 0)
        keep += [ta, tb, tc]
        outs_plain.append(td1)
        outs_q.append(td2)
        plain_flags.append(fw)
    flags = torch.zeros(ncalls, dtype=torch.int32, device="cuda")
    b = ctypes.c_void_p()
    cftgb._lib.check(L.cftg_batch_create(gpu, calls, ncalls, flags.data_ptr(), ctypes.byref(b)), "create")
    cftgb._lib.check(L.cftg_batch_launch(b, stream), "launch")
    torch.cuda.synchronize()
    for i in range(ncalls):
        assert torch.equal(outs_plain[i], outs_q[i]), i
    assert torch.equal(torch.cat(plain_flags), flags)
    # the same batch captured in a graph and replayed
    s2 = torch.cuda.Stream()
    for o in outs_q:
        o.zero_()
    flags.zero_()
    cftgb._lib.check(L.cftg_batch_capture(b, s2.cuda_stream), "capture")
    for _ in range(2):
        cftgb._lib.check(L.cftg_batch_launch(b, s2.cuda_stream), "replay")
    s2.synchronize()
    for i in range(ncalls):
        assert torch.equal(outs_plain[i], outs_q[i]), i
    assert torch.equal(torch.cat(plain_flags), flags)
    L.cftg_batch_free(b)


KINDS5 = [(0, 1, "add"), (0, 3, "mul"), (0, 0, "fma"), (1, 0, "div"), (2, 0, "sqrt")]


@pytest.mark.parametrize("threads", [256, 128])
def test_queue_matches_oracle(gpu, oracle, threads):
    """The batched form against the oracle itself, not only against the
    plain kernels (which share its element code): binary64/128/256 x add,
    mul, fma, div, sqrt x all five attributes, sizes across tile edges
    (1 to 4,097 elements) and three calls of 2^20 (the uneven batch's
    largest), every element's value and every call's flag word, as one
    launch and again replayed from a CUDA graph, at both block shapes."""
    import torch
    L = cftgb.lib()
    vp = ctypes.c_void_p
    L.cftg_batch_create.argtypes = [vp, ctypes.POINTER(Call), ctypes.c_size_t, vp, ctypes.POINTER(vp)]
    L.cftg_batch_launch.argtypes = [vp, vp]
    L.cftg_batch_capture.argtypes = [vp, vp]
    L.cftg_batch_free.argtypes = [vp]
    before = L.cftg_queue_block_threads()
    cftgb._lib.check(L.cftg_set_queue_block_threads(threads), "cftg_set_queue_block_threads")
    try:
        rng = np.random.default_rng(77)
        edges = [1, 2, 31, 255, 256, 257, 1023, 1025, 4097]
        spec = []
        for fmt in (1, 2, 3):
            for kind, op, _ in KINDS5:
                for rnd in range(5):
                    spec.append((fmt, kind, op, rnd, edges[int(rng.integers(0, len(edges)))]))
        spec += [(1, 1, 0, 2, 1 << 20), (2, 2, 0, 4, 1 << 20), (3, 0, 0, 0, 1 << 20)]
        calls = (Call * len(spec))()
        keep, host, outs = [], [], []
        for i, (fmt, kind, op, rnd, n) in enumerate(spec):
            a, b, c = wl.gen_operands(fmt, n, 5000 + i, ties=n >= 4)
            ta, tb, tc = (torch.from_numpy(x.view(np.int32)).cuda() for x in (a, b, c))
            td = torch.zeros_like(ta)
            calls[i] = Call(kind, op, fmt, rnd, ta.data_ptr(), tb.data_ptr(), tc.data_ptr(),
                            td.data_ptr(), n, 0)
            keep += [ta, tb, tc]
            host.append((a, b, c))
            outs.append(td)
        want = [oracle.run_parallel(kind, fmt, op, rnd, *host[i])
                for i, (fmt, kind, op, rnd, n) in enumerate(spec)]
        flags = torch.zeros(len(spec), dtype=torch.int32, device="cuda")
        bt = ctypes.c_void_p()
        cftgb._lib.check(L.cftg_batch_create(gpu, calls, len(spec), flags.data_ptr(), ctypes.byref(bt)),
                         "create")
        stream = torch.cuda.current_stream().cuda_stream

        def check(where):
            got_flags = flags.cpu().numpy().view(np.uint32)
            for i, (fmt, kind, op, rnd, n) in enumerate(spec):
                d = outs[i].cpu().numpy().view(np.uint32).reshape(n, -1)
                rd, _, racc = want[i]
                bad = np.nonzero((d != rd).any(1))[0]
                assert bad.size == 0, (where, fmt, kind, op, rnd, n, bad[:4])
                assert int(got_flags[i]) & 0x1F == racc, (where, fmt, kind, op, rnd, n)

        cftgb._lib.check(L.cftg_batch_launch(bt, stream), "launch")
        torch.cuda.synchronize()
        check("launch")
        s2 = torch.cuda.Stream()
        for o in outs:
            o.zero_()
        flags.zero_()
        cftgb._lib.check(L.cftg_batch_capture(bt, s2.cuda_stream), "capture")
        cftgb._lib.check(L.cftg_batch_launch(bt, s2.cuda_stream), "replay")
        s2.synchronize()
        check("graph replay")
        L.cftg_batch_free(bt)
    finally:
        cftgb._lib.check(L.cftg_set_queue_block_threads(before), "cftg_set_queue_block_threads")
