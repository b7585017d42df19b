"""Binary32 FMA/ADD/SUB/MUL on the hardware's rounding (elem_hw.cu) against
the oracle and against the integer kernels, every element's value and
flags, under all five attributes (RMM always takes the integer path);
binary64 (the integer kernels) on the same edge operands.

Besides the benchmark's value mix and raw encodings, the operands aim at
the hardware path's own decision edges: exact results (short significands,
aligned addends), results a few ulps around 2^(emin+1) and 2^emin (the
lowest magnitudes the hardware path keeps, and tininess), around the
largest finite magnitude (overflow in every direction), and exact
cancellations (zero results)."""
import numpy as np
import pytest

from cftgb import workload as wl
from test_elem_gpu import device_run
from test_oracle import _raw_and_boundary

pytestmark = pytest.mark.gpu

KINDS = ((0, "fma"), (1, "add"), (2, "sub"), (3, "mul"))


def _bits(x, fmt):
    if fmt == 0:
        return x.astype(np.float32).view(np.uint32).reshape(-1, 1)
    return x.astype(np.float64).view(np.uint32).reshape(-1, 2)


def edge_operands(fmt, n, seed):
    """(a, b, c) aimed at the hardware path's edges (see the module text)."""
    with np.errstate(over="ignore", invalid="ignore", under="ignore"):
        return _edge_operands(fmt, n, seed)


def _edge_operands(fmt, n, seed):
    rng = np.random.default_rng(seed)
    p, emin, emax = (24, -126, 127) if fmt == 0 else (53, -1022, 1023)
    h = p // 2
    sig = lambda k: rng.integers(1 << (k - 1), 1 << k, size=n).astype(np.float64)  # noqa: E731
    sgn = lambda: np.where(rng.random(n) < 0.5, -1.0, 1.0)  # noqa: E731
    group = rng.integers(0, 5, size=n)
    ea = rng.integers(-20, 20, size=n)
    eb = rng.integers(-20, 20, size=n)
    # the product's target exponent by group: anywhere, near 2^(emin+1),
    # near 2^emin, near the top, anywhere (with c cancelling it)
    tgt = np.select([group == 1, group == 2, group == 3],
                    [emin + 1 + rng.integers(-2, 3, size=n), emin + rng.integers(-2, 2, size=n),
                     emax + rng.integers(-1, 1, size=n)], default=ea + eb)
    sa, sb = sig(h), sig(h)
    lead = np.floor(np.log2(sa * sb)).astype(np.int64)          # the exact product's top bit
    shift_b = tgt - lead - ea
    eb = np.where(group > 0, shift_b, eb)
    a = np.ldexp(sgn() * sa, ea - 0)
    b = np.ldexp(sgn() * sb, eb)
    # c: short significand near the product (exact sums), or its negation
    ec = tgt - (h - 1) + rng.integers(-3, 4, size=n)
    c = np.ldexp(sgn() * sig(h), ec)
    prod = a * b                                                 # exact in binary64 at fp32;
    c = np.where(group == 4, -prod, c)                           # zero results
    if fmt == 0:
        ok = np.isfinite(a.astype(np.float32)) & np.isfinite(b.astype(np.float32)) & \
            np.isfinite(c.astype(np.float32))
        a, b, c = (np.where(ok, x, 1.0) for x in (a, b, c))
    return _bits(a, fmt), _bits(b, fmt), _bits(c, fmt)


@pytest.mark.parametrize("fmt", [0, 1])
def test_hw_path_matches_oracle(gpu, oracle, fmt):
    sets = [wl.gen_operands(fmt, 1 << 17, 300 + fmt, ties=True),
            _raw_and_boundary(fmt, 30000, 400 + fmt),
            edge_operands(fmt, 1 << 17, 500 + fmt)]
    for si, (a, b, c) in enumerate(sets):
        for op, name in KINDS:
            for rnd in range(5):
                d, lf, acc = device_run(gpu, 0, fmt, op, rnd, a, b, c)
                rd, rlf, racc = oracle.run(0, fmt, op, rnd, a, b, c)
                vbad = np.nonzero((d != rd).any(1))[0]
                fbad = np.nonzero(lf != rlf)[0]
                assert vbad.size == 0, (si, name, rnd, "values", vbad[:4], a[vbad[:2]], b[vbad[:2]],
                                        c[vbad[:2]], d[vbad[:2]], rd[vbad[:2]])
                assert fbad.size == 0, (si, name, rnd, "flags", fbad[:4], lf[fbad[:4]], rlf[fbad[:4]])
                assert acc & 0x1F == racc


@pytest.mark.parametrize("fmt", [0])
def test_hw_path_equals_integer_path(gpu, monkeypatch, fmt):
    """The same launches with CFTG_ELEM_HW=0 (the integer kernels): every
    value and flag equal, on arrays large enough to span many tiles and
    blocks, with a ragged last tile."""
    n = (1 << 21) + 77
    a, b, c = wl.gen_operands(fmt, n, 600 + fmt, ties=True)
    for op, name in KINDS:
        for rnd in (0, 1, 2, 3):
            d1, lf1, acc1 = device_run(gpu, 0, fmt, op, rnd, a, b, c)
            monkeypatch.setenv("CFTG_ELEM_HW", "0")
            d2, lf2, acc2 = device_run(gpu, 0, fmt, op, rnd, a, b, c)
            monkeypatch.delenv("CFTG_ELEM_HW")
            assert np.array_equal(d1, d2) and np.array_equal(lf1, lf2) and acc1 == acc2, (name, rnd)
