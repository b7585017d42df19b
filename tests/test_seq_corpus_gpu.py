"""The reference's sequencer differential corpus (host/tests/seq_check.py's
first corpus, golden-model results; tests/golden/make_seq_corpus.py)
through the GPU: cft_program_load refuses what the model refuses, and
cft_program_run on host buffers (lane counts either side of 64 and 128)
gives the model's deposits, counts, flags and status for every other
program."""
import ctypes

import numpy as np
import pytest

import cftgb
import seqcorpus

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
def test_seq_corpus_on_gpu(gpu, fmt):
    L = cftgb.lib()
    vp = ctypes.c_void_p
    L.cft_program_run.argtypes = [vp, vp, vp, vp, vp, vp, ctypes.c_size_t,
                                  ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32)]
    ran = 0
    for t in seqcorpus.trials(fmt):
        img = t["image"]
        prog = ctypes.c_void_p()
        st = L.cft_program_load(gpu, img.ctypes.data, img.size, ctypes.byref(prog))
        if t["refused"]:
            assert st != 0, (fmt, t["trial"], "the model refuses it")
            continue
        assert st == 0, (fmt, t["trial"], L.cft_last_error())
        try:
            n, W = t["n"], t["a"].shape[1]
            maxdep = int(np.frombuffer(img[:32].tobytes(), "<u4")[4])
            dep = np.zeros((max(1, n * maxdep), W), np.uint32)
            cnt = np.zeros(n, np.uint32)
            fl, bus = ctypes.c_uint32(), ctypes.c_uint32()
            cftgb._lib.check(L.cft_program_run(prog, t["a"].ctypes.data, t["b"].ctypes.data,
                                               t["c"].ctypes.data, dep.ctypes.data,
                                               cnt.ctypes.data, n, ctypes.byref(fl),
                                               ctypes.byref(bus)), "cft_program_run")
        finally:
            L.cft_program_free(prog)
        assert np.array_equal(dep[:n * maxdep], t["deposits"]), (fmt, t["trial"], "deposits")
        assert np.array_equal(cnt, t["counts"]), (fmt, t["trial"], "counts")
        assert fl.value == t["flags"] and bus.value == t["status"], (fmt, t["trial"])
        ran += 1
    assert ran > 100
