"""Binary128/256 FMA/ADD/SUB/MUL through the kernel that sorts special
elements out of the general path's warps (elem_q.cu) against the oracle
and against the one-element-a-thread kernel (CFTG_ELEM_SORT=0): every
element's value and flags, all five attributes, arrays spanning many tiles
with a ragged last one, and tiles that are all special, all general or
empty of either."""
import numpy as np
import pytest

from cftgb import workload as wl
from test_elem_gpu import device_run
from test_oracle import _raw_and_boundary

pytestmark = pytest.mark.gpu

KINDS = ((0, "fma"), (1, "add"), (2, "sub"), (3, "mul"))


@pytest.mark.parametrize("fmt", [2, 3])
def test_sorted_path_matches_oracle(gpu, oracle, fmt):
    n = 40000 + 13
    mixes = [wl.gen_operands(fmt, n, 700 + fmt, ties=True),
             _raw_and_boundary(fmt, 20000, 710 + fmt),
             wl.gen_operands(fmt, 5000, 720 + fmt, special_frac=1.0, triples_frac=0.0),
             wl.gen_operands(fmt, 5000, 730 + fmt, special_frac=0.0, triples_frac=0.0)]
    for mi, (a, b, c) in enumerate(mixes):
        for op, name in KINDS:
            for rnd in range(5):
                d, lf, acc = device_run(gpu, 0, fmt, op, rnd, a, b, c)
                rd, rlf, racc = oracle.run(0, fmt, op, rnd, a, b, c)
                vbad = np.nonzero((d != rd).any(1))[0]
                fbad = np.nonzero(lf != rlf)[0]
                assert vbad.size == 0 and fbad.size == 0, (mi, name, rnd, vbad[:4], fbad[:4])
                assert acc & 0x1F == racc, (mi, name, rnd)


@pytest.mark.parametrize("fmt", [2, 3])
def test_sorted_path_equals_unsorted(gpu, monkeypatch, fmt):
    n = (1 << 21) + 301
    a, b, c = wl.gen_operands(fmt, n, 740 + fmt, ties=True)
    for op, name in KINDS:
        for rnd in (0, 4):
            d1, lf1, acc1 = device_run(gpu, 0, fmt, op, rnd, a, b, c)
            monkeypatch.setenv("CFTG_ELEM_SORT", "0")
            d2, lf2, acc2 = device_run(gpu, 0, fmt, op, rnd, a, b, c)
            monkeypatch.delenv("CFTG_ELEM_SORT")
            assert np.array_equal(d1, d2) and np.array_equal(lf1, lf2) and acc1 == acc2, (name, rnd)
