"""The oracle pinned: its restatement (oracle/sfport.c) against the golden
vectors the reference's Python definition produced (tests/golden/), and -
where this machine holds the reference tree - against the reference
library built from its own sources (oracle/_ref/)."""
import ctypes
from pathlib import Path

import numpy as np
import pytest

from cftgb import workload as wl

GOLD = Path(__file__).resolve().parent / "golden"
DIV, SQRT = 1000, 1001


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
def test_oracle_matches_golden_vectors(oracle, fmt):
    g = np.load(GOLD / f"golden_{wl.geometry(fmt)['width']}.npz")
    bad = []
    for i in range(len(g["op"])):
        op, rnd = int(g["op"][i]), int(g["rnd"][i])
        kind = 1 if op == DIV else 2 if op == SQRT else 0
        a, b, c = (g[k][i:i + 1] for k in ("a", "b", "c"))
        d, lf, _ = oracle.run(kind, fmt, 0 if kind else op, rnd, a, b, c)
        if not (np.array_equal(d[0], g["d"][i]) and lf[0] == g["flags"][i]):
            bad.append((i, op, rnd))
    assert not bad, f"{len(bad)} golden mismatches, first {bad[:5]}"


def _ref():
    p = Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "libcft_ref.so"
    if not p.exists():
        pytest.skip("the reference library is built only where the reference tree is present")
    L = ctypes.CDLL(str(p))
    vp, i, sz, u32p = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.POINTER(ctypes.c_uint32)
    L.cft_open.argtypes = [ctypes.c_char_p, i, ctypes.POINTER(vp)]
    L.cft_run.argtypes = [vp, i, i, i, vp, vp, vp, vp, sz, u32p, u32p]
    L.cft_div.argtypes = [vp, i, i, vp, vp, vp, sz, u32p, u32p]
    L.cft_sqrt.argtypes = [vp, i, i, vp, vp, sz, u32p, u32p]
    dev = ctypes.c_void_p()
    assert L.cft_open(None, 0, ctypes.byref(dev)) == 0
    return L, dev


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
def test_oracle_matches_reference_library(oracle, fmt):
    """Whole arrays, every opcode and mode: values and the OR of the flags;
    then every element's own flags through n=1 calls."""
    L, dev = _ref()
    n = 2000
    a, b, c = wl.gen_operands(fmt, n, 77 + fmt, ties=True, triples_frac=0.05)
    for kind, ops in ((0, [o for o in range(32) if o not in (24, 25, 28, 29, 31)] + [77]),
                      (1, [0]), (2, [0])):
        for op in ops:
            for rnd in range(5) if (kind or op <= 3) else (0,):
                d, lf, acc = oracle.run(kind, fmt, op, rnd, a, b, c)
                ref = np.zeros_like(d)
                fl = ctypes.c_uint32()
                if kind == 0:
                    st = L.cft_run(dev, op, fmt, rnd, a.ctypes.data, b.ctypes.data, c.ctypes.data,
                                   ref.ctypes.data, ctypes.c_size_t(n), ctypes.byref(fl), None)
                elif kind == 1:
                    st = L.cft_div(dev, fmt, rnd, a.ctypes.data, b.ctypes.data, ref.ctypes.data,
                                   ctypes.c_size_t(n), ctypes.byref(fl), None)
                else:
                    st = L.cft_sqrt(dev, fmt, rnd, a.ctypes.data, ref.ctypes.data,
                                    ctypes.c_size_t(n), ctypes.byref(fl), None)
                assert st == 0
                assert np.array_equal(d, ref), (kind, op, rnd)
                assert acc == fl.value, (kind, op, rnd)
                # every element's flags through n=1 calls
                for i in range(n):
                    one = np.zeros((1, a.shape[1]), np.uint32)
                    f1 = ctypes.c_uint32()
                    if kind == 0:
                        L.cft_run(dev, op, fmt, rnd, a[i:].ctypes.data, b[i:].ctypes.data,
                                  c[i:].ctypes.data, one.ctypes.data, ctypes.c_size_t(1),
                                  ctypes.byref(f1), None)
                    elif kind == 1:
                        L.cft_div(dev, fmt, rnd, a[i:].ctypes.data, b[i:].ctypes.data,
                                  one.ctypes.data, ctypes.c_size_t(1), ctypes.byref(f1), None)
                    else:
                        L.cft_sqrt(dev, fmt, rnd, a[i:].ctypes.data, one.ctypes.data,
                                   ctypes.c_size_t(1), ctypes.byref(f1), None)
                    assert lf[i] == f1.value, (kind, op, rnd, i)


def test_oracle_planted_mistake_is_caught(oracle):
    """A mistake planted in the oracle's OUTPUT (on the CPU) must fail the
    golden comparison: the check is not vacuous."""
    g = np.load(GOLD / "golden_256.npz")
    i = int(np.nonzero(g["op"] == 0)[0][5])
    d, lf, _ = oracle.run(0, 3, 0, int(g["rnd"][i]), g["a"][i:i + 1], g["b"][i:i + 1],
                          g["c"][i:i + 1])
    d[0, 0] ^= 1
    assert not np.array_equal(d[0], g["d"][i])


def _raw_and_boundary(fmt, n, seed):
    """Operands drawn over the whole encoding space: uniform random words
    (every exponent, so far-apart alignments, NaN payloads and subnormals),
    then the same words with exponents moved next to the overflow and the
    underflow thresholds (products and sums that overflow, results that land
    in the subnormal range or round across its edges)."""
    g = wl.geometry(fmt)
    W, es, expw = g["W"], g["es"], g["expw"]
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(3):
        x = rng.integers(0, 1 << 32, size=(n, W), dtype=np.uint64).astype(np.uint32)
        third = n // 3
        emax = (1 << expw) - 2
        near = np.concatenate([rng.integers(max(1, emax - 3 * g["prec"]), emax + 1, size=third),
                               rng.integers(1, 3 * g["prec"], size=third)]).astype(np.uint32)
        top = x[n - 2 * third:, W - 1]
        top &= np.uint32(~(((1 << expw) - 1) << es) & 0xFFFFFFFF)
        top |= near << np.uint32(es)
        x[n - 2 * third:, W - 1] = top
        out.append(x)
    return out


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
def test_oracle_matches_reference_on_raw_encodings(oracle, fmt):
    """FMA/ADD/SUB/MUL, division and square root under every attribute over
    raw and boundary encodings: the same values and, element by element, the
    same flags as the reference library."""
    L, dev = _ref()
    n = 1500
    a, b, c = _raw_and_boundary(fmt, n, 31 + fmt)
    for kind, op in ((0, 0), (0, 1), (0, 2), (0, 3), (1, 0), (2, 0)):
        for rnd in range(5):
            d, lf, acc = oracle.run(kind, fmt, op, rnd, a, b, c)
            ref = np.zeros_like(d)
            fl = ctypes.c_uint32()
            if kind == 0:
                st = L.cft_run(dev, op, fmt, rnd, a.ctypes.data, b.ctypes.data, c.ctypes.data,
                               ref.ctypes.data, ctypes.c_size_t(n), ctypes.byref(fl), None)
            elif kind == 1:
                st = L.cft_div(dev, fmt, rnd, a.ctypes.data, b.ctypes.data, ref.ctypes.data,
                               ctypes.c_size_t(n), ctypes.byref(fl), None)
            else:
                st = L.cft_sqrt(dev, fmt, rnd, a.ctypes.data, ref.ctypes.data,
                                ctypes.c_size_t(n), ctypes.byref(fl), None)
            assert st == 0
            bad = np.nonzero((d != ref).any(1))[0]
            assert bad.size == 0, (kind, op, rnd, bad[:5])
            assert acc == fl.value, (kind, op, rnd)
            for i in range(n):
                one = np.zeros((1, a.shape[1]), np.uint32)
                f1 = ctypes.c_uint32()
                if kind == 0:
                    L.cft_run(dev, op, fmt, rnd, a[i:].ctypes.data, b[i:].ctypes.data,
                              c[i:].ctypes.data, one.ctypes.data, ctypes.c_size_t(1),
                              ctypes.byref(f1), None)
                elif kind == 1:
                    L.cft_div(dev, fmt, rnd, a[i:].ctypes.data, b[i:].ctypes.data,
                              one.ctypes.data, ctypes.c_size_t(1), ctypes.byref(f1), None)
                else:
                    L.cft_sqrt(dev, fmt, rnd, a[i:].ctypes.data, one.ctypes.data,
                               ctypes.c_size_t(1), ctypes.byref(f1), None)
                assert lf[i] == f1.value, (kind, op, rnd, i)
