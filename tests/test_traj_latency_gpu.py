"""The trajectory kernel's arithmetic (FMA, ADD, SUB, MUL in the latency
form its bundles use: the split product, selects on the integer ALU, the
one-test unpack of usual operands; and the cooperative form, W threads an
operation) against the oracle's sequencer, element by element. Each lane runs a one-operation program once, so every lane is
one element: every format x operation x rounding attribute, over the
benchmark's operand mix, rows that are all hard cases (exact cancellations,
ties) and, at binary32/64, operands aimed at the rounding edges (results
near the subnormal boundary and the largest magnitude); every lane's
result and flag byte, through cftg_traj_create/launch with the operands as
the a/b/c streams."""
import ctypes

import numpy as np
import pytest

import cftgb
import oracle_lib
from cftgb import asm
from cftgb import workload as wl

pytestmark = pytest.mark.gpu

FMT_NAMES = ("fp32", "fp64", "fp128", "fp256")
RND_NAMES = ("rne", "rtz", "rdn", "rup", "rmm")
# the sources a lane reads: r0, r1, r2 are the a, b, c streams; ADD/SUB take
# a and c, so the hard rows' ADD ties (c half an ulp of a) are exercised
OPS = (("fma", "r0, r1, r2"), ("add", "r0, r2"), ("sub", "r0, r2"), ("mul", "r0, r1"))


def program(fmt, op, srcs, rnd):
    return asm.assemble(f""".format   {FMT_NAMES[fmt]}
.deposits 0
.scratch  in 1
.scratch  out 1
{op}.{RND_NAMES[rnd]} r3, {srcs}
stl r3, 0
halt
""")


def gpu_run(h, img, a, b, c):
    import torch
    L = cftgb.lib()
    vp = ctypes.c_void_p
    L.cftg_traj_create.argtypes = [vp, vp, ctypes.c_size_t, vp, vp, vp, vp, vp, vp,
                                   ctypes.c_uint32, ctypes.c_uint32, vp, ctypes.POINTER(vp)]
    L.cftg_traj_launch.argtypes = [vp, vp]
    L.cftg_traj_result.argtypes = [vp, vp, vp, vp]
    L.cftg_traj_free.argtypes = [vp]
    n, W = a.shape
    img = np.frombuffer(img, np.uint8).copy()
    prog = vp()
    cftgb._lib.check(L.cft_program_load(h, img.ctypes.data, img.size, ctypes.byref(prog)), "load")
    ta, tb, tc = (torch.from_numpy(x.view(np.int32)).cuda() for x in (a, b, c))
    state = torch.zeros((n, W), dtype=torch.int32, device="cuda")
    lf = torch.zeros(n, dtype=torch.uint8, device="cuda")
    segs = np.ones(n, np.uint32)
    t = vp()
    try:
        cftgb._lib.check(L.cftg_traj_create(prog, segs.ctypes.data, n, ta.data_ptr(), tb.data_ptr(),
                                            tc.data_ptr(), None, state.data_ptr(), None, 0, 0,
                                            lf.data_ptr(), ctypes.byref(t)), "cftg_traj_create")
        s = torch.cuda.Stream()
        cftgb._lib.check(L.cftg_traj_launch(t, s.cuda_stream), "launch")
        fl, st = ctypes.c_uint32(), ctypes.c_uint32()
        cftgb._lib.check(L.cftg_traj_result(t, ctypes.byref(fl), ctypes.byref(st), s.cuda_stream),
                         "result")
    finally:
        if t:
            L.cftg_traj_free(t)
        L.cft_program_free(prog)
    return state.cpu().numpy().view(np.uint32), lf.cpu().numpy(), fl.value, st.value


def oracle_run(oracle, img, a, b, c):
    n, W = a.shape
    img = np.frombuffer(img, np.uint8).copy()
    sin = np.zeros((n, W), np.uint32)
    sout = np.zeros((n, W), np.uint32)
    lf = np.zeros(n, np.uint8)
    A = oracle_lib.SeqArgs()
    A.a, A.b, A.c, A.n = a.ctypes.data, b.ctypes.data, c.ctypes.data, n
    A.scratch_in, A.scratch_out, A.lane_flags, A.depth = sin.ctypes.data, sout.ctypes.data, \
        lf.ctypes.data, 256
    assert oracle.L.sfp_seq_run(img.ctypes.data, img.size, ctypes.byref(A)) == 0
    return sout, lf, A.flags_out


def operand_sets(fmt, n):
    sets = [wl.gen_operands(fmt, n, 900 + fmt, ties=True, triples_frac=0.05),
            wl.hard_rows(fmt, min(n, 4096), 910 + fmt)]
    if fmt <= 1:
        from test_elem_hw_gpu import edge_operands
        sets.append(edge_operands(fmt, n, 920 + fmt))
    return [tuple(np.ascontiguousarray(x, np.uint32) for x in s) for s in sets]


@pytest.fixture(params=["2", "8", "8c", "32c"])
def lane_threads(request, monkeypatch):
    """Threads a lane, "c": the cooperative arithmetic (W threads an
    operation at binary128/256; the one-thread form at binary32/64)."""
    monkeypatch.setenv("CFTG_LANE_THREADS", request.param.rstrip("c"))
    monkeypatch.setenv("CFTG_LANE_COOP", "1" if request.param.endswith("c") else "0")
    return request.param


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
def test_latency_form_matches_oracle(gpu, oracle, fmt, lane_threads):
    n = 1 << 14
    for si, (a, b, c) in enumerate(operand_sets(fmt, n)):
        for op, srcs in OPS:
            for rnd in range(5):
                img = program(fmt, op, srcs, rnd)
                got, glf, gfl, gst = gpu_run(gpu, img, a, b, c)
                want, wlf, wfl = oracle_run(oracle, img, a, b, c)
                bad = np.nonzero((got != want).any(1))[0]
                assert bad.size == 0, (fmt, si, op, rnd, bad[:4], a[bad[:1]], b[bad[:1]], c[bad[:1]])
                fbad = np.nonzero(glf != wlf)[0]
                assert fbad.size == 0, (fmt, si, op, rnd, "flags", fbad[:4], glf[fbad[:4]], wlf[fbad[:4]])
                assert gfl == wfl and gst == 0, (fmt, si, op, rnd)
