"""Helpers for the sequencer tests: fixture loading and runs through the
oracle (CPU) and through the library's C ABI (GPU)."""
import ctypes
from pathlib import Path

import numpy as np

GOLD = Path(__file__).resolve().parent / "golden"


def header(img):
    w = np.frombuffer(bytes(img[:32]), "<u4")
    return dict(n_insns=int(w[2]), n_consts=int(w[3]), maxdep=int(w[4]), prec=int(w[5]),
                flags=int(w[6]), sin=int(w[7]) & 0xFFFF if w[6] & 2 else 0,
                sout=int(w[7]) >> 16 if w[6] & 2 else 0)


def uses_augadd(img):
    h = header(img)
    esz = (4, 8, 16, 32)[h["prec"]] if h["prec"] <= 3 else 4
    base = 32 + (0 if h["flags"] & 1 else h["n_consts"] * esz)
    body = bytes(img[base:base + 8 * h["n_insns"]])
    for i in range(0, len(body) - 7, 8):
        w = int.from_bytes(body[i:i + 8], "little")
        if (w >> 31) & 1 and (w & 0xFF) in (10, 11):
            return True
    return False


def cases():
    return sorted((GOLD / "programs").glob("*.npz"))


def load(path):
    z = np.load(path)
    return {k: z[k] for k in z.files}


def ptr(x):
    return None if x is None else x.ctypes.data


def run_oracle(oracle, case, variant=1):
    """(outputs dict) via the oracle's seqport, or None if it cannot run it."""
    import oracle_lib
    img = case["image"]
    h = header(img)
    W = (1, 2, 4, 8)[h["prec"]]
    n = int(case["n"])
    dep = np.zeros((max(1, n * h["maxdep"]), W), np.uint32)
    cnt = np.zeros(n, np.uint32)
    lf = np.zeros(n, np.uint8)
    sout = np.zeros((max(1, n * h["sout"]), W), np.uint32)
    A = oracle_lib.SeqArgs()
    a = case["a"]
    if variant == 2:
        a = case["a"][: int(case["idx_a_src"])].copy()
        A.idx_a = ptr(case["idx_a"])
        A.lane_mask = ptr(case["mask"])
    A.a, A.b, A.c, A.n = ptr(a), ptr(case["b"]), ptr(case["c"]), n
    A.bank = ptr(case["bank"]) if case["bank"].size else None
    A.scratch_in = ptr(case["scratch_in"]) if case["scratch_in"].size else None
    A.scratch_out = ptr(sout)
    A.deposits = ptr(dep)
    A.counts = ptr(cnt)
    A.lane_flags = ptr(lf)
    A.depth = 256
    st = oracle.L.sfp_seq_run(img.ctypes.data, img.size, ctypes.byref(A))
    if st:
        return None
    return dict(deposits=dep[: n * h["maxdep"]], counts=cnt, lane_flags=lf, flags=A.flags_out,
                status=A.status_out, scratch_out=sout[: n * h["sout"]])


def compare(got, case, prefix="exp_"):
    bad = []
    for k in ("deposits", "counts", "lane_flags", "scratch_out"):
        e = case[prefix + k]
        g = got[k]
        if not np.array_equal(np.asarray(g).reshape(e.shape), e):
            bad.append(k)
    for k in ("flags", "status"):
        if int(got[k]) != int(case[prefix + k]):
            bad.append(f"{k} {int(got[k]):#x} != {int(case[prefix + k]):#x}")
    return bad


def run_gpu(h, case, variant=1):
    """Outputs through cft_program_load + cft_program_run_ex, or the load
    status (an int) when the load refuses."""
    import cftgb
    from cftgb._lib import RunArgs
    L = cftgb.lib()
    img = case["image"]
    hd = header(img)
    W = (1, 2, 4, 8)[hd["prec"]]
    esz = 4 * W
    n = int(case["n"])
    prog = ctypes.c_void_p()
    st = L.cft_program_load(h, img.ctypes.data, img.size, ctypes.byref(prog))
    if st:
        return st
    dep = np.zeros((max(1, n * hd["maxdep"]), W), np.uint32)
    cnt = np.zeros(n, np.uint32)
    lf = np.zeros(n, np.uint8)
    sout = np.zeros((max(1, n * hd["sout"]), W), np.uint32)
    fl, bus = ctypes.c_uint32(), ctypes.c_uint32()
    A = RunArgs()
    A.struct_size = ctypes.sizeof(RunArgs)
    a = case["a"]
    if variant == 2:
        a = case["a"][: int(case["idx_a_src"])].copy()
        A.idx_a, A.idx_a_src = ptr(case["idx_a"]), int(case["idx_a_src"])
        A.lane_mask, A.lane_mask_bytes = ptr(case["mask"]), case["mask"].size
    A.a, A.b, A.c, A.n = ptr(a), ptr(case["b"]), ptr(case["c"]), n
    if hd["flags"] & 1:
        A.bank, A.bank_bytes = ptr(case["bank"]), case["bank"].nbytes
    if hd["flags"] & 2:
        if hd["sin"]:
            A.scratch_in, A.scratch_in_bytes = ptr(case["scratch_in"]), case["scratch_in"].nbytes
        if hd["sout"]:
            A.scratch_out, A.scratch_out_bytes = ptr(sout), n * hd["sout"] * esz
    A.deposits = ptr(dep) if hd["maxdep"] else None
    A.counts = ptr(cnt)
    A.flags_out = ctypes.pointer(fl)
    A.bus_out = ctypes.pointer(bus)
    A.lane_flags, A.lane_flags_bytes = ptr(lf), n
    st = L.cft_program_run_ex(prog, ctypes.byref(A))
    L.cft_program_free(prog)
    cftgb._lib.check(st, "cft_program_run_ex")
    return dict(deposits=dep[: n * hd["maxdep"]], counts=cnt, lane_flags=lf, flags=fl.value,
                status=bus.value, scratch_out=sout[: n * hd["sout"]])
