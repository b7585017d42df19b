"""The sequencer's checker pinned, and the loader's decisions checked,
without a GPU: the oracle's executor (oracle/seqport.c) against the
outputs the reference library produced (tests/golden/programs), and the
library's loader (cftg_program_check) against the statuses the
reference's cft_program_load returned on the same images."""
import ctypes

import numpy as np
import pytest

import cftgb
import seq_util as su

CASES = su.cases()


@pytest.mark.parametrize("path", CASES, ids=[p.stem for p in CASES])
def test_oracle_executor_matches_reference_outputs(oracle, path):
    case = su.load(path)
    got = su.run_oracle(oracle, case)
    assert got is not None
    assert su.compare(got, case) == []
    if "mask" in case:
        got2 = su.run_oracle(oracle, case, variant=2)
        assert su.compare(got2, case, "exp2_") == []


@pytest.mark.parametrize("cert", ["lorenz63", "lorenz96", "henonheiles"])
def test_oracle_reproduces_certificates(oracle, cert):
    """The fp256 ODE certificates' segment chains through the oracle: every
    boundary's tagged state hash, flags and STATUS as recorded."""
    import hashlib
    import oracle_lib
    z = np.load(su.GOLD / f"{cert}_cert.npz")
    img, bank = z["image"].copy(), z["bank"].copy()
    slots = su.header(img)["sout"]
    state = z["state0"].copy().view(np.uint32).reshape(-1, 8)
    n = state.shape[0] // slots
    a = np.zeros((n, 8), np.uint32)
    for k, end in enumerate(z["ends"]):
        out = np.zeros_like(state)
        A = oracle_lib.SeqArgs()
        A.a, A.n, A.bank = a.ctypes.data, n, bank.ctypes.data
        A.scratch_in, A.scratch_out, A.depth = state.ctypes.data, out.ctypes.data, 256
        assert oracle.L.sfp_seq_run(img.ctypes.data, img.size, ctypes.byref(A)) == 0
        assert hashlib.sha256(b"cft-certificate 1 state\0" + out.tobytes()).hexdigest() == str(end)
        assert A.flags_out == int(z["flags"][k]) and A.status_out == int(z["status"][k])
        state = out


def test_loader_decisions_match_the_reference():
    z = np.load(su.GOLD / "loader_cases.npz")
    L = cftgb.lib()
    L.cftg_program_check.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint32]
    L.cftg_program_check.restype = ctypes.c_int
    off = 0
    bad = []
    for i, (n, want) in enumerate(zip(z["lens"], z["status"])):
        img = z["blob"][off:off + n].copy()
        off += n
        buf = img if n else np.zeros(1, np.uint8)
        got = L.cftg_program_check(buf.ctypes.data, int(n), 256)
        if got != want:
            bad.append((i, int(want), got, L.cft_last_error()))
    assert not bad, f"{len(bad)} of {len(z['lens'])} differ, first {bad[:4]}"
    assert (z["status"] == 0).sum() > 100 and len(set(z["status"].tolist())) >= 3


def test_sha256_known_answers():
    import hashlib
    L = cftgb.lib()
    out = (ctypes.c_uint8 * 32)()
    for msg in (b"", b"abc", b"a" * 55, b"a" * 56, b"a" * 64, bytes(range(256)) * 5):
        buf = ctypes.create_string_buffer(msg, len(msg) or 1)
        assert L.cft_sha256(buf if msg else None, len(msg), out) == 0
        assert bytes(out) == hashlib.sha256(msg).digest()
