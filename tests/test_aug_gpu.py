"""The augmented operations on the GPU (cft_augmented_add / _sub / _mul)
against the oracle's restatement of IEEE 754-2019 9.5, element by element:
both results and the flags."""
import ctypes

import numpy as np
import pytest

import cftgb
from cftgb import workload as wl
from test_aug_oracle import aug_operands

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
def test_augmented_match_oracle(gpu, oracle, fmt):
    L = cftgb.lib()
    vp, i, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t
    for fn in ("cft_augmented_add", "cft_augmented_sub", "cft_augmented_mul"):
        getattr(L, fn).argtypes = [vp, i, vp, vp, vp, vp, sz, ctypes.POINTER(ctypes.c_uint32)]
    oracle.L.sfp_aug.argtypes = [i, i, vp, vp, vp, vp, ctypes.POINTER(ctypes.c_uint32)]
    n = 4000
    a, b = aug_operands(fmt, n, 900 + fmt)
    W = wl.words(fmt)
    for k, name in enumerate(("cft_augmented_add", "cft_augmented_sub", "cft_augmented_mul")):
        r = np.zeros((n, W), np.uint32)
        e = np.zeros((n, W), np.uint32)
        fl = ctypes.c_uint32()
        assert getattr(L, name)(gpu, fmt, a.ctypes.data, b.ctypes.data, r.ctypes.data,
                                e.ctypes.data, n, ctypes.byref(fl)) == 0
        r1 = np.zeros(W, np.uint32)
        e1 = np.zeros(W, np.uint32)
        f1 = ctypes.c_uint32()
        acc = 0
        bad = []
        for j in range(n):
            assert oracle.L.sfp_aug(fmt, k, a[j].ctypes.data, b[j].ctypes.data, r1.ctypes.data,
                                    e1.ctypes.data, ctypes.byref(f1)) == 0
            if not (np.array_equal(r1, r[j]) and np.array_equal(e1, e[j])):
                bad.append(j)
            acc |= f1.value
        assert not bad, (name, len(bad), bad[:5])
        assert fl.value == acc, name
        # per-element flags through single-element calls on a sample
        for j in range(0, n, 37):
            fr = ctypes.c_uint32()
            assert getattr(L, name)(gpu, fmt, a[j:].ctypes.data, b[j:].ctypes.data, r.ctypes.data,
                                    e.ctypes.data, 1, ctypes.byref(fr)) == 0
            oracle.L.sfp_aug(fmt, k, a[j].ctypes.data, b[j].ctypes.data, r1.ctypes.data,
                             e1.ctypes.data, ctypes.byref(f1))
            assert fr.value == f1.value, (name, j)


def test_augmented_argument_rules(gpu):
    L = cftgb.lib()
    x = np.zeros((4, 2), np.uint32)
    fl = ctypes.c_uint32()
    vp, i, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t
    L.cft_augmented_add.argtypes = [vp, i, vp, vp, vp, vp, sz, ctypes.POINTER(ctypes.c_uint32)]
    assert L.cft_augmented_add(gpu, 1, x.ctypes.data, x.ctypes.data, x.ctypes.data, x.ctypes.data,
                               4, ctypes.byref(fl)) == 1          # r and e the same buffer
    assert L.cft_augmented_add(gpu, 1, None, x.ctypes.data, x.ctypes.data, x[2:].ctypes.data,
                               2, ctypes.byref(fl)) == 1          # a NULL
    assert L.cft_augmented_add(gpu, 9, x.ctypes.data, x.ctypes.data, x.ctypes.data,
                               x[2:].ctypes.data, 2, ctypes.byref(fl)) == 1   # no such format
    assert L.cft_augmented_add(gpu, 1, None, None, None, None, 0, ctypes.byref(fl)) == 0
