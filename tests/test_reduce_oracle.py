"""The oracle's reductions (sfp_reduce, sfp_reduce_seg) pinned against the
reference library's cft_reduce / cft_reduce_seg, built here from the
reference's own sources: every reduction opcode, format and rounding
attribute, lengths that exercise every tree shape near powers of two, and
the planted specials of IEEE 754-2019 9.4's infinity rule."""
import ctypes
from pathlib import Path

import numpy as np
import pytest

from cftgb import workload as wl

OPS = (24, 25, 28, 29, 31)
LENS = (0, 1, 2, 3, 5, 7, 8, 13, 64, 100, 1000, 2049)


def _ref():
    p = Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "libcft_ref.so"
    if not p.exists():
        pytest.skip("the reference library is built only where the reference tree is present")
    L = ctypes.CDLL(str(p))
    vp, i, sz, u32p = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.POINTER(ctypes.c_uint32)
    L.cft_open.argtypes = [ctypes.c_char_p, i, ctypes.POINTER(vp)]
    L.cft_reduce.argtypes = [vp, i, i, i, vp, vp, vp, sz, u32p, u32p]
    L.cft_reduce_seg.argtypes = [vp, i, i, i, vp, vp, vp, sz, sz, u32p, u32p]
    dev = ctypes.c_void_p()
    assert L.cft_open(None, 0, ctypes.byref(dev)) == 0
    return L, dev


def _bind(oracle):
    vp, i, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t
    u32p = ctypes.POINTER(ctypes.c_uint32)
    oracle.L.sfp_reduce.argtypes = [i, i, i, vp, vp, vp, sz, u32p]
    oracle.L.sfp_reduce_seg.argtypes = [i, i, i, vp, vp, vp, sz, sz, u32p]


def operands(fmt, n, seed, plant=None):
    a, b, _ = wl.gen_operands(fmt, max(n, 1), seed, special_frac=0.0, exp_range=12,
                              triples_frac=0.0)
    a, b = a[:n].copy(), b[:n].copy()
    W = wl.words(fmt)
    if plant and n:
        e_w, m_w = wl.GEOM[fmt]
        expmask = ((1 << e_w) - 1) << m_w
        vals = {"inf": expmask, "-inf": expmask | (1 << (e_w + m_w)),
                "qnan": expmask | (1 << (m_w - 1)), "snan": expmask | 1}
        rng = np.random.default_rng(seed)
        for name in plant:
            a[int(rng.integers(0, n))] = wl.from_int(vals[name], W)
    return a, b


def run_both(L, dev, oracle, fmt, op, rnd, a, b, n):
    W = wl.words(fmt)
    d_ref = np.zeros(W, np.uint32)
    d_or = np.zeros(W, np.uint32)
    f_ref, f_or = ctypes.c_uint32(), ctypes.c_uint32()
    st = L.cft_reduce(dev, op, fmt, rnd, a.ctypes.data if n else None,
                      b.ctypes.data if (n and op == 25) else None, d_ref.ctypes.data, n,
                      ctypes.byref(f_ref), None)
    assert st == 0, (op, fmt, rnd, n)
    assert oracle.L.sfp_reduce(fmt, op, rnd, a.ctypes.data if n else None,
                               b.ctypes.data if n else None, d_or.ctypes.data, n,
                               ctypes.byref(f_or)) == 0
    return d_ref, f_ref.value, d_or, f_or.value


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
def test_reductions_match_reference(oracle, fmt):
    L, dev = _ref()
    _bind(oracle)
    for op in OPS:
        for n in LENS:
            a, b = operands(fmt, n, 1000 * fmt + n)
            for rnd in range(5):
                d_ref, f_ref, d_or, f_or = run_both(L, dev, oracle, fmt, op, rnd, a, b, n)
                assert np.array_equal(d_ref, d_or) and f_ref == f_or, (op, n, rnd)


@pytest.mark.parametrize("plant", [["inf"], ["qnan"], ["snan"], ["inf", "qnan"], ["inf", "snan"],
                                   ["-inf", "inf"], ["snan", "-inf", "qnan"]])
def test_reduction_specials_match_reference(oracle, plant):
    L, dev = _ref()
    _bind(oracle)
    for fmt in (1, 3):
        for op in OPS:
            for n in (1, 2, 9, 300):
                a, b = operands(fmt, n, 7 + n, plant=plant)
                d_ref, f_ref, d_or, f_or = run_both(L, dev, oracle, fmt, op, 0, a, b, n)
                assert np.array_equal(d_ref, d_or) and f_ref == f_or, (op, n, plant)


def test_segmented_reductions_match_reference(oracle):
    L, dev = _ref()
    _bind(oracle)
    n = 96
    for fmt in (0, 2, 3):
        a, b = operands(fmt, n, 31 + fmt, plant=["inf", "qnan"])
        a2, b2 = operands(fmt, n, 41 + fmt)
        W = wl.words(fmt)
        for A, B in ((a, b), (a2, b2)):
            for op in OPS:
                for seg in (1, 3, 32, 96):
                    d_ref = np.zeros((n // seg, W), np.uint32)
                    d_or = np.zeros_like(d_ref)
                    f_ref, f_or = ctypes.c_uint32(), ctypes.c_uint32()
                    assert L.cft_reduce_seg(dev, op, fmt, 1, A.ctypes.data,
                                            B.ctypes.data if op == 25 else None, d_ref.ctypes.data,
                                            n, seg, ctypes.byref(f_ref), None) == 0
                    assert oracle.L.sfp_reduce_seg(fmt, op, 1, A.ctypes.data, B.ctypes.data,
                                                   d_or.ctypes.data, n, seg, ctypes.byref(f_or)) == 0
                    assert np.array_equal(d_ref, d_or) and f_ref.value == f_or.value, (fmt, op, seg)


def _wide(fmt, n, seed):
    """Raw random encodings (every exponent: NaN payloads, subnormals, huge
    alignment gaps) and values next to the overflow threshold (sums that
    overflow), half and half."""
    g = wl.geometry(fmt)
    W, es, expw = g["W"], g["es"], g["expw"]
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(2):
        x = rng.integers(0, 1 << 32, size=(n, W), dtype=np.uint64).astype(np.uint32)
        half = n // 2
        emax = (1 << expw) - 2
        top = x[half:, W - 1] & np.uint32(~(((1 << expw) - 1) << es) & 0xFFFFFFFF)
        near = rng.integers(emax - 4, emax + 1, size=n - half).astype(np.uint32)
        x[half:, W - 1] = top | (near << np.uint32(es))
        out.append(x)
    return out


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
def test_reductions_over_wide_encodings_match_reference(oracle, fmt):
    L, dev = _ref()
    _bind(oracle)
    for op in OPS:
        for n in (2, 7, 64, 513):
            a, b = _wide(fmt, n, 3000 * fmt + n)
            for rnd in range(5):
                d_ref, f_ref, d_or, f_or = run_both(L, dev, oracle, fmt, op, rnd, a, b, n)
                assert np.array_equal(d_ref, d_or) and f_ref == f_or, (op, n, rnd)
            # the tail alone: every value near the overflow threshold
            t = n - n // 2
            a2, b2 = a[n // 2:].copy(), b[n // 2:].copy()
            d_ref, f_ref, d_or, f_or = run_both(L, dev, oracle, fmt, op, 0, a2, b2, t)
            assert np.array_equal(d_ref, d_or) and f_ref == f_or, (op, t, "near max")
