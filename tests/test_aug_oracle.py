"""The oracle's augmented operations (IEEE 754-2019 9.5: augmentedAddition,
augmentedSubtraction, augmentedMultiplication) pinned element by element,
values of both results and flags, against the reference library's
cft_augmented_add / _sub / _mul built from the reference's sources."""
import ctypes
from pathlib import Path

import numpy as np
import pytest

from cftgb import workload as wl


def _ref():
    p = Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "libcft_ref.so"
    if not p.exists():
        pytest.skip("the reference library is built only where the reference tree is present")
    L = ctypes.CDLL(str(p))
    vp, i, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t
    L.cft_open.argtypes = [ctypes.c_char_p, i, ctypes.POINTER(vp)]
    for fn in ("cft_augmented_add", "cft_augmented_sub", "cft_augmented_mul"):
        getattr(L, fn).argtypes = [vp, i, vp, vp, vp, vp, sz, ctypes.POINTER(ctypes.c_uint32)]
    dev = ctypes.c_void_p()
    assert L.cft_open(None, 0, ctypes.byref(dev)) == 0
    return L, dev


def aug_operands(fmt, n, seed):
    """A mix for 9.5: the benchmark's operands (specials included), pairs
    whose exponents are close (rounding and residuals), far apart (the FAR
    case), near the overflow threshold and near the subnormal range."""
    a, b, _ = wl.gen_operands(fmt, n, seed, special_frac=0.10, exp_range=64, ties=True)
    e_w, m_w = wl.GEOM[fmt]
    bias = (1 << (e_w - 1)) - 1
    rng = np.random.default_rng(seed)
    W = wl.words(fmt)
    for i in range(0, n, 4):
        kind = rng.integers(0, 5)
        ea = int(rng.integers(1, 2 * bias))
        if kind == 0:       # near each other
            eb = ea + int(rng.integers(-3, 4))
        elif kind == 1:     # far apart, around the FAR bound p + 2
            eb = ea - (m_w + 1) + int(rng.integers(-2, 3))
        elif kind == 2:     # near overflow
            ea = 2 * bias - int(rng.integers(0, 2))
            eb = ea - int(rng.integers(0, m_w + 3))
        elif kind == 3:     # near the subnormal range
            ea = int(rng.integers(1, 4))
            eb = int(rng.integers(0, 3))
        else:               # products that underflow
            ea = int(rng.integers(1, bias // 2))
            eb = int(rng.integers(1, bias // 2))
        for arr, ex in ((a, ea), (b, eb)):
            ex = min(max(ex, 0), 2 * bias)
            frac = int(rng.integers(0, 1 << 62)) << max(0, m_w - 62) if m_w > 62 else int(rng.integers(0, 1 << m_w))
            frac &= (1 << m_w) - 1
            sign = int(rng.integers(0, 2))
            arr[i] = wl.from_int((sign << (e_w + m_w)) | (ex << m_w) | frac, W)
    return a, b


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
def test_augmented_match_reference(oracle, fmt):
    L, dev = _ref()
    u8 = ctypes.c_void_p
    oracle.L.sfp_aug.argtypes = [ctypes.c_int, ctypes.c_int, u8, u8, u8, u8,
                                 ctypes.POINTER(ctypes.c_uint32)]
    n = 3000
    a, b = aug_operands(fmt, n, 600 + fmt)
    W = wl.words(fmt)
    for fn, name in enumerate(("cft_augmented_add", "cft_augmented_sub", "cft_augmented_mul")):
        rr = np.zeros((n, W), np.uint32)
        re = np.zeros((n, W), np.uint32)
        fl = ctypes.c_uint32()
        # whole array through the reference, then per element through the oracle
        assert getattr(L, name)(dev, fmt, a.ctypes.data, b.ctypes.data, rr.ctypes.data,
                                re.ctypes.data, n, ctypes.byref(fl)) == 0
        acc = 0
        r1 = np.zeros(W, np.uint32)
        e1 = np.zeros(W, np.uint32)
        f1 = ctypes.c_uint32()
        for i in range(n):
            assert oracle.L.sfp_aug(fmt, fn, a[i].ctypes.data, b[i].ctypes.data, r1.ctypes.data,
                                    e1.ctypes.data, ctypes.byref(f1)) == 0
            assert np.array_equal(r1, rr[i]) and np.array_equal(e1, re[i]), (name, i)
            acc |= f1.value
        assert acc == fl.value, name
        # every element's flags through n=1 calls
        for i in range(n):
            fr = ctypes.c_uint32()
            getattr(L, name)(dev, fmt, a[i:].ctypes.data, b[i:].ctypes.data, rr.ctypes.data,
                             re.ctypes.data, 1, ctypes.byref(fr))
            oracle.L.sfp_aug(fmt, fn, a[i].ctypes.data, b[i].ctypes.data, r1.ctypes.data,
                             e1.ctypes.data, ctypes.byref(f1))
            assert fr.value == f1.value, (name, i)
