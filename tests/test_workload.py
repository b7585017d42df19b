"""The seeded synthetic operands stand in for the benchmark configurations'
value mix; these CPU tests hold the generator to that mix: about 10 % of
each operand special, spread over the six kinds; normals with unbiased
exponents in [-64, 64]; exact-cancellation triples whose FMA the oracle
rounds to an exact zero; halfway cases that round as ties; the same arrays
for the same seed."""
import numpy as np
import pytest

from cftgb import workload as wl

N = 60000


def _fields(fmt, x):
    g = wl.geometry(fmt)
    W, es, expw = g["W"], g["es"], g["expw"]
    top = x[:, W - 1]
    e = (top >> np.uint32(es)) & np.uint32((1 << expw) - 1)
    frac_zero = ((top & np.uint32((1 << es) - 1)) == 0) & (x[:, :W - 1] == 0).all(1)
    return e.astype(np.int64), frac_zero, g


@pytest.mark.parametrize("fmt", [1, 2, 3])
def test_special_share_and_normal_exponents(fmt):
    a, b, c = wl.gen_operands(fmt, N, 7, triples_frac=0.0)
    for x in (a, b, c):
        e, fz, g = _fields(fmt, x)
        emax = (1 << g["expw"]) - 1
        zero = (e == 0) & fz
        sub = (e == 0) & ~fz
        inf = (e == emax) & fz
        nan = (e == emax) & ~fz
        near_top = e == emax - 1
        normal = (e > 0) & (e < emax - 1)
        share = {"zero": zero.mean(), "subnormal": sub.mean(), "inf": inf.mean(),
                 "nan": nan.mean(), "near_max": near_top.mean()}
        special = 1.0 - normal.mean()
        assert 0.09 < special < 0.11, special
        # six kinds, quiet and signalling NaNs counted together
        for k, v in share.items():
            want = 2 / 60 if k == "nan" else 1 / 60
            assert abs(v - want) < 0.006, (k, v)
        ue = e[normal] - g["bias"]
        assert ue.min() >= -64 and ue.max() <= 64
        assert abs(ue.mean()) < 1.5


@pytest.mark.parametrize("fmt", [2, 3])
def test_triples_cancel_exactly(oracle, fmt):
    n = 20000
    a, b, c = wl.gen_operands(fmt, n, 9, special_frac=0.0, triples_frac=0.02)
    d, lf, _ = oracle.run(0, fmt, 0, 0, a, b, c)          # FMA, RNE
    W = wl.words(fmt)
    exact_zero = ((d[:, W - 1] & np.uint32(0x7FFFFFFF)) == 0) & (d[:, :W - 1] == 0).all(1) & (lf == 0)
    # normals give an exact zero only by cancellation; the triples all do
    assert exact_zero.sum() >= int(n * 0.02)
    assert exact_zero.sum() <= int(n * 0.02) + 5


@pytest.mark.parametrize("fmt", [1, 3])
def test_halfway_cases_round_as_ties(oracle, fmt):
    """With ties=True, some MUL and ADD results are exact halfway cases:
    they round differently under roundTiesToEven and roundTiesToAway."""
    n = 8000
    a, b, c = wl.gen_operands(fmt, n, 13, special_frac=0.0, triples_frac=0.01, ties=True)
    for op in (3, 1):                                      # MUL, ADD
        rne, _, _ = oracle.run(0, fmt, op, 0, a, b, c)
        rna, _, _ = oracle.run(0, fmt, op, 4, a, b, c)
        differ = (rne != rna).any(1)
        assert differ.sum() >= 10, (fmt, op, int(differ.sum()))


def test_same_seed_same_operands():
    x = wl.gen_operands(3, 5000, 21, ties=True)
    y = wl.gen_operands(3, 5000, 21, ties=True)
    z = wl.gen_operands(3, 5000, 22, ties=True)
    assert all(np.array_equal(p, q) for p, q in zip(x, y))
    assert not np.array_equal(x[0], z[0])
