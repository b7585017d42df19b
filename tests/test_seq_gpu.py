"""The sequencer on the GPU against the reference's own outputs: every
program the reference ships (tests/golden/programs), with and without a
lane mask and index tables; the reference's photograph known answer (an
NVIDIA GPU's recorded deposit hashes for a million-lane camera program);
and the fp256 ODE certificates' segment chains."""
import ctypes
import hashlib

import numpy as np
import pytest

import cftgb
import seq_util as su
from cftgb._lib import RunArgs

pytestmark = pytest.mark.gpu
CASES = su.cases()


@pytest.mark.parametrize("path", CASES, ids=[p.stem for p in CASES])
def test_program_matches_reference(gpu, path):
    case = su.load(path)
    got = su.run_gpu(gpu, case)
    assert isinstance(got, dict), f"load refused: {got} {cftgb.lib().cft_last_error()}"
    assert su.compare(got, case) == []
    if "mask" in case:
        got2 = su.run_gpu(gpu, case, variant=2)
        assert su.compare(got2, case, "exp2_") == []


def _run_bank_iota(h, img, bank, n):
    L = cftgb.lib()
    hd = su.header(img)
    W = (1, 2, 4, 8)[hd["prec"]]
    prog = ctypes.c_void_p()
    cftgb._lib.check(L.cft_program_load(h, img.ctypes.data, img.size, ctypes.byref(prog)),
                     "cft_program_load")
    a = np.zeros((n, W), np.uint32)
    a[:, 0] = np.arange(n, dtype=np.uint32)
    z = np.zeros_like(a)
    dep = np.zeros((n * hd["maxdep"], W), np.uint32)
    fl, bus = ctypes.c_uint32(), ctypes.c_uint32()
    L.cft_program_run_bank.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t] + \
        [ctypes.c_void_p] * 5 + [ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]
    st = L.cft_program_run_bank(prog, bank.ctypes.data, bank.size, a.ctypes.data, z.ctypes.data,
                                z.ctypes.data, dep.ctypes.data, None, n, ctypes.byref(fl),
                                ctypes.byref(bus))
    L.cft_program_free(prog)
    cftgb._lib.check(st, "cft_program_run_bank")
    return dep, fl.value, bus.value


def test_photograph_known_answer(gpu):
    """camera.cftp over 1,048,576 samples a pass, four passes: the deposit
    buffer's SHA-256 must be the one an NVIDIA GPU recorded rendering the
    same frame from pinned GLSL (reference host/tests/photograph/hopf)."""
    d = su.GOLD / "photograph"
    img = np.frombuffer((d / "camera.cftp").read_bytes(), np.uint8).copy()
    want = (d / "deposits.SHA256").read_text().split()
    for p in range(4):
        bank = np.frombuffer((d / f"camera.p{p:04d}.bank").read_bytes(), np.uint8).copy()
        dep, fl, bus = _run_bank_iota(gpu, img, bank, 1 << 20)
        assert bus == 0
        assert hashlib.sha256(dep.tobytes()).hexdigest() == want[p], f"pass {p}"


CERTS = ["lorenz63", "lorenz96", "henonheiles"]


@pytest.mark.parametrize("cert", CERTS)
def test_certificate_chain(gpu, cert):
    """The fp256 ODE certificates (Lorenz-63 RK4, Lorenz-96 RK4, Henon-Heiles
    leapfrog): each segment run from the certificate's boundary state, every
    boundary's tagged hash, flags and STATUS as the certificate records them."""
    z = np.load(su.GOLD / f"{cert}_cert.npz")
    img = z["image"].copy()
    bank = z["bank"].copy()
    slots = su.header(img)["sout"]
    state = z["state0"].copy().view(np.uint32).reshape(-1, 8)
    n = state.shape[0] // slots
    L = cftgb.lib()
    prog = ctypes.c_void_p()
    cftgb._lib.check(L.cft_program_load(gpu, img.ctypes.data, img.size, ctypes.byref(prog)), "load")
    tag = b"cft-certificate 1 state\0"
    a = np.zeros((n, 8), np.uint32)
    for k, end in enumerate(z["ends"]):
        out = np.zeros_like(state)
        fl, bus = ctypes.c_uint32(), ctypes.c_uint32()
        A = RunArgs()
        A.struct_size = ctypes.sizeof(RunArgs)
        A.a, A.n = a.ctypes.data, n
        A.bank, A.bank_bytes = bank.ctypes.data, bank.size
        A.scratch_in, A.scratch_in_bytes = state.ctypes.data, state.nbytes
        A.scratch_out, A.scratch_out_bytes = out.ctypes.data, out.nbytes
        A.flags_out, A.bus_out = ctypes.pointer(fl), ctypes.pointer(bus)
        cftgb._lib.check(L.cft_program_run_ex(prog, ctypes.byref(A)), "run")
        assert hashlib.sha256(tag + out.tobytes()).hexdigest() == str(end), f"segment {k}"
        assert fl.value == int(z["flags"][k]) and bus.value == int(z["status"][k])
        state = out
    L.cft_program_free(prog)


def test_program_info_and_digest(gpu):
    case = next(c for c in map(su.load, su.cases())
                if not su.uses_augadd(c["image"]) and c["bank"].size)
    L = cftgb.lib()
    img = case["image"]
    prog = ctypes.c_void_p()
    cftgb._lib.check(L.cft_program_load(gpu, img.ctypes.data, img.size, ctypes.byref(prog)), "load")
    info = cftgb._lib.ProgramInfo()
    info.struct_size = ctypes.sizeof(info)
    assert L.cft_program_get_info(prog, ctypes.byref(info)) == 0
    hd = su.header(img)
    assert (info.n_insns, info.n_consts, info.max_deposits, info.format) == \
        (hd["n_insns"], hd["n_consts"], hd["maxdep"], hd["prec"])
    out = (ctypes.c_uint8 * 32)()
    L.cft_program_digest.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    bank = case["bank"]
    st = L.cft_program_digest(prog, bank.ctypes.data if bank.size else None, bank.nbytes, out)
    assert st == 0
    assert bytes(out) == hashlib.sha256(img.tobytes() + bank.tobytes()).digest()
    L.cft_program_free(prog)


@pytest.mark.parametrize("cert", CERTS)
def test_certificate_segment_lines(gpu, cert):
    """The GPU run writes the certificate's own segment lines (start and end
    state hashes, flags, STATUS) for the reference's fp256 certificates."""
    from cftgb import certify
    z = np.load(su.GOLD / f"{cert}_cert.npz")
    state0 = z["state0"].copy().view(np.uint32).reshape(-1, 8)
    starts = [certify.state_hash(state0)] + [str(e) for e in z["ends"][:-1]]
    want = [f"segment {k} start {starts[k]} end {z['ends'][k]} flags {int(z['flags'][k])} "
            f"status {int(z['status'][k])}" for k in range(len(z["ends"]))]
    lines, _ = certify.segment_lines(gpu, z["image"].tobytes(), z["bank"].tobytes(), state0,
                                     len(z["ends"]))
    assert lines == want
