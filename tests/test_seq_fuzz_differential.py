"""The oracle's sequencer executor against the reference library's on
mutated programs (CPU tests).

Every program the reference ships (tests/golden/programs) is mutated by
seeded bit flips in the opcode, register and rounding fields of its
arithmetic instructions (never a control instruction, a constant flag or an
immediate, so every loop keeps its trip count). Each mutant that the
reference's cft_program_load accepts runs on the same 70 lanes through the
oracle (oracle/seqport.c, which the GPU executor is held to) and through
the reference library's cft_program_run_ex on its software device
(host/src/seq_exec.h:412-923, host/src/program.c:1823-2040); deposits,
counts, lane flags, scratch-out, the flag word and STATUS must agree.
Skipped where the reference library (oracle/_ref) is not built."""
import ctypes
from pathlib import Path

import numpy as np
import pytest

import seq_util as su
from cftgb._lib import RunArgs

REF = Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "libcft_ref.so"
pytestmark = pytest.mark.skipif(not REF.exists(),
                                reason="the reference library (oracle/_ref) is not built here")


@pytest.fixture(scope="module")
def ref():
    R = ctypes.CDLL(str(REF))
    vp = ctypes.c_void_p
    R.cft_open.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(vp)]
    R.cft_close.argtypes = [vp]
    R.cft_program_load.argtypes = [vp, vp, ctypes.c_size_t, ctypes.POINTER(vp)]
    R.cft_program_free.argtypes = [vp]
    R.cft_program_run_ex.argtypes = [vp, ctypes.POINTER(RunArgs)]
    h = vp()
    assert R.cft_open(None, 0, ctypes.byref(h)) == 0
    yield R, h
    R.cft_close(h)


def run_ref(R, h, case):
    """Outputs of the reference library, or None when its loader refuses."""
    img = case["image"]
    hd = su.header(img)
    W = (1, 2, 4, 8)[hd["prec"]]
    esz = 4 * W
    n = int(case["n"])
    prog = ctypes.c_void_p()
    if R.cft_program_load(h, img.ctypes.data, img.size, ctypes.byref(prog)) != 0:
        return None
    dep = np.zeros((max(1, n * hd["maxdep"]), W), np.uint32)
    cnt = np.zeros(n, np.uint32)
    lf = np.zeros(n, np.uint8)
    sout = np.zeros((max(1, n * hd["sout"]), W), np.uint32)
    fl, bus = ctypes.c_uint32(), ctypes.c_uint32()
    A = RunArgs()
    A.struct_size = ctypes.sizeof(RunArgs)
    A.a, A.b, A.c, A.n = su.ptr(case["a"]), su.ptr(case["b"]), su.ptr(case["c"]), n
    if hd["flags"] & 1:
        A.bank, A.bank_bytes = su.ptr(case["bank"]), case["bank"].nbytes
    if hd["flags"] & 2:
        if hd["sin"]:
            A.scratch_in, A.scratch_in_bytes = su.ptr(case["scratch_in"]), case["scratch_in"].nbytes
        if hd["sout"]:
            A.scratch_out, A.scratch_out_bytes = su.ptr(sout), n * hd["sout"] * esz
    A.deposits = su.ptr(dep) if hd["maxdep"] else None
    A.counts = su.ptr(cnt)
    A.flags_out = ctypes.pointer(fl)
    A.bus_out = ctypes.pointer(bus)
    A.lane_flags, A.lane_flags_bytes = su.ptr(lf), n
    st = R.cft_program_run_ex(prog, ctypes.byref(A))
    R.cft_program_free(prog)
    assert st == 0
    return dict(deposits=dep[: n * hd["maxdep"]], counts=cnt, lane_flags=lf, flags=fl.value,
                status=bus.value, scratch_out=sout[: n * hd["sout"]])


def _arith_words(img):
    hd = su.header(img)
    esz = (4, 8, 16, 32)[hd["prec"]]
    base = 32 + (0 if hd["flags"] & 1 else hd["n_consts"] * esz)
    out = []
    for i in range(hd["n_insns"]):
        w = int.from_bytes(bytes(img[base + 8 * i:base + 8 * i + 8]), "little")
        if not (w >> 27) & 0x1F:              # no constant flags, kx or ctrl
            out.append(base + 8 * i)
    return out


def test_executor_matches_reference_on_mutants(oracle, ref):
    R, h = ref
    rng = np.random.default_rng(99)
    ran = 0
    bad = []
    for path in su.cases():
        case = su.load(path)
        sites = _arith_words(case["image"])
        if not sites:
            continue
        for _ in range(12):
            m = dict(case)
            img = case["image"].copy()
            for _ in range(int(rng.integers(1, 4))):
                off = sites[int(rng.integers(0, len(sites)))]
                bit = int(rng.choice([*range(0, 24), 24, 25, 26]))   # op, rd/ra/rb/rc, rnd
                img[off + bit // 8] ^= np.uint8(1 << (bit % 8))
            m["image"] = img
            want = run_ref(R, h, m)
            if want is None:
                continue
            got = su.run_oracle(oracle, m)
            assert got is not None, path.stem
            diff = [k for k in ("deposits", "counts", "lane_flags", "scratch_out")
                    if not np.array_equal(np.asarray(got[k]).reshape(np.shape(want[k])), want[k])]
            diff += [k for k in ("flags", "status") if int(got[k]) != int(want[k])]
            if diff:
                bad.append((path.stem, diff))
            ran += 1
    assert not bad, bad[:5]
    assert ran > 150, ran
