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
    if su.uses_augadd(case["image"]):
        pytest.skip("augmented addition is outside this oracle and this backend")
    got = su.run_oracle(oracle, case)
    assert got is not None
    assert su.compare(got, case) == []
    if "mask" in case:
        got2 = su.run_oracle(oracle, case, variant=2)
        assert su.compare(got2, case, "exp2_") == []


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
        if want == 0 and su.uses_augadd(img):
            want = 2            # this device does not publish CFT_SEQ_FEAT_AUGADD
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
