"""The allocation-free program run (cftg_program_run_noalloc) against the
ordinary one (cft_program_run_ex), through the C ABI, on two calls in a row.

It serves callers that cannot let the library call cudaMalloc - a host
whose device memory is all owned by its own pool or budget, or a loop that
cannot take cudaMalloc's implicit synchronisation - so the run's scratch
lives in a fixed array inside the library. The comparison is bit for bit
(no tolerance): values, counts, deposits, flags and STATUS, against the
ordinary run and against the reference library's own outputs for the same
program and lanes (the committed fixture). Two calls in a
row show that what the shared array kept from the first call does not leak
into the second. This file sorts last so that a failure here stops a run
only after every other test has run; it also passes alone.
"""
import ctypes

import numpy as np
import pytest

import cftgb
import seq_util as su
from cftgb._lib import RunArgs

pytestmark = pytest.mark.gpu


def _bind(L):
    vp = ctypes.c_void_p
    L.cftg_program_run_noalloc.argtypes = [vp] * 9 + [ctypes.c_size_t, vp, vp, vp]
    L.cftg_program_run_noalloc.restype = ctypes.c_int
    L.cftg_noalloc_scratch_bytes.restype = ctypes.c_size_t


def _reference_run(h, case):
    got = su.run_gpu(h, case)
    assert isinstance(got, dict)
    return got


def _pick(pred):
    for p in su.cases():
        c = su.load(p)
        if not su.uses_augadd(c["image"]) and pred(su.header(c["image"])):
            return c
    pytest.skip("no fixture of that shape")


@pytest.mark.parametrize("shape", ["bank+scratch", "deposits"])
def test_noalloc_matches_program_run_ex_twice(gpu, shape):
    import torch
    L = cftgb.lib()
    _bind(L)
    if shape == "bank+scratch":
        case = _pick(lambda h: h["flags"] & 1 and h["sin"] and h["sout"])
    else:
        case = _pick(lambda h: h["maxdep"] > 0 and not h["flags"] & 2)
    want = _reference_run(gpu, case)
    img = case["image"]
    hd = su.header(img)
    n = int(case["n"])
    W = (1, 2, 4, 8)[hd["prec"]]

    def dev(x):
        return torch.from_numpy(np.ascontiguousarray(x).view(np.int32)).cuda()

    ta, tb, tc = dev(case["a"]), dev(case["b"]), dev(case["c"])
    tbank = dev(case["bank"]) if case["bank"].size else None
    tsin = dev(case["scratch_in"]) if case["scratch_in"].size else None
    tsout = torch.zeros((max(1, n * hd["sout"]), W), dtype=torch.int32, device="cuda")
    tdep = torch.zeros((max(1, n * hd["maxdep"]), W), dtype=torch.int32, device="cuda")
    tcnt = torch.zeros(n, dtype=torch.int32, device="cuda")
    prog = ctypes.c_void_p()
    cftgb._lib.check(L.cft_program_load(gpu, img.ctypes.data, img.size, ctypes.byref(prog)), "load")
    stream = torch.cuda.current_stream().cuda_stream
    try:
        for call in range(2):
            tsout.fill_(-1)                  # stale bytes must not survive a call
            tcnt.fill_(-1)
            fl, st = ctypes.c_uint32(), ctypes.c_uint32()
            rc = L.cftg_program_run_noalloc(
                prog, ta.data_ptr(), tb.data_ptr(), tc.data_ptr(),
                tbank.data_ptr() if tbank is not None else None,
                tsin.data_ptr() if tsin is not None else None,
                tsout.data_ptr() if hd["sout"] else None,
                tdep.data_ptr() if hd["maxdep"] else None, tcnt.data_ptr(), n,
                ctypes.byref(fl), ctypes.byref(st), stream)
            cftgb._lib.check(rc, "cftg_program_run_noalloc")
            torch.cuda.synchronize()
            got_sout = tsout.cpu().numpy().view(np.uint32)[: n * hd["sout"]]
            got_dep = tdep.cpu().numpy().view(np.uint32)[: n * hd["maxdep"]]
            got_cnt = tcnt.cpu().numpy().view(np.uint32)
            assert np.array_equal(got_sout, want["scratch_out"]), f"call {call}: scratch-out"
            assert np.array_equal(got_dep, want["deposits"]), f"call {call}: deposits"
            assert np.array_equal(got_cnt, want["counts"]), f"call {call}"
            assert fl.value == want["flags"] and st.value == want["status"], f"call {call}"
            # and the reference library's own outputs for the same lanes
            # (the fixture, produced by its cft_program_run_ex)
            assert np.array_equal(got_sout.reshape(-1), case["exp_scratch_out"].reshape(-1)), call
            assert np.array_equal(got_dep.reshape(-1), case["exp_deposits"].reshape(-1)), call
            assert np.array_equal(got_cnt, case["exp_counts"].astype(np.uint32)), call
            assert fl.value == int(case["exp_flags"]) and st.value == int(case["exp_status"]), call
    finally:
        L.cft_program_free(prog)


def test_noalloc_refuses_a_run_past_its_array(gpu):
    L = cftgb.lib()
    _bind(L)
    case = _pick(lambda h: h["flags"] & 2 and h["sin"])
    img = case["image"]
    hd = su.header(img)
    esz = (4, 8, 16, 32)[hd["prec"]]
    prog = ctypes.c_void_p()
    cftgb._lib.check(L.cft_program_load(gpu, img.ctypes.data, img.size, ctypes.byref(prog)), "load")
    import torch
    too_many = L.cftg_noalloc_scratch_bytes() // (max(hd["sin"], hd["sout"]) * esz) + 1
    # a real (small) buffer: the size rule refuses the call before any of
    # it is read or written
    small = torch.zeros(64, dtype=torch.int32, device="cuda")
    p = small.data_ptr()
    rc = L.cftg_program_run_noalloc(prog, p, None, None, p, p, p, p, None, too_many, None, None,
                                    None)
    L.cft_program_free(prog)
    assert rc == 1
    assert b"allocates nothing" in L.cft_last_error()
