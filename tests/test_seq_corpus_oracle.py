"""The reference's sequencer differential corpus (host/tests/seq_check.py's
first corpus: random programs from the golden model's generator, plain and
with IMUL and kx-indexed constants, 30 % corrupted; results from the golden
model) against this library's loader decision (cftg_program_check, no
device) and the oracle's executor (CPU): every refusal the model makes is
made here, and every accepted program's deposits, counts, flags and status
equal the model's."""
import ctypes

import numpy as np
import pytest

import cftgb
import oracle_lib
import seqcorpus


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
def test_seq_corpus_loader_and_oracle(oracle, fmt):
    L = cftgb.lib()
    L.cftg_program_check.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_uint32]
    ran = refused = 0
    for t in seqcorpus.trials(fmt):
        img = t["image"]
        st = L.cftg_program_check(img.tobytes(), img.size, 256)
        if t["refused"]:
            assert st != 0, (fmt, t["trial"], "the model refuses it")
            refused += 1
            continue
        assert st == 0, (fmt, t["trial"], L.cft_last_error())
        n, W = t["n"], t["a"].shape[1]
        hd = np.frombuffer(img[:32].tobytes(), "<u4")
        maxdep = int(hd[4])
        dep = np.zeros((max(1, n * maxdep), W), np.uint32)
        cnt = np.zeros(n, np.uint32)
        A = oracle_lib.SeqArgs()
        A.a, A.b, A.c, A.n = t["a"].ctypes.data, t["b"].ctypes.data, t["c"].ctypes.data, n
        A.deposits, A.counts, A.depth = dep.ctypes.data, cnt.ctypes.data, 256
        assert oracle.L.sfp_seq_run(img.ctypes.data, img.size, ctypes.byref(A)) == 0
        assert np.array_equal(dep[:n * maxdep], t["deposits"]), (fmt, t["trial"], "deposits")
        assert np.array_equal(cnt, t["counts"]), (fmt, t["trial"], "counts")
        assert A.flags_out == t["flags"] and A.status_out == t["status"], (fmt, t["trial"])
        ran += 1
    assert ran > 100 and refused > 20, (ran, refused)
