"""Parity of the bulk-staged elementwise kernels (large arrays in device
memory: operands staged into shared memory by cp.async.bulk copies) with
the oracle and with the direct kernels, bit for bit in values and in every
element's flags, through cftg_run_device.

Under CFTG_ELEM_STAGING=bulk the staged kernels take calls of n >= 65,536
without index tables whose streamed operands are 16-byte aligned device
memory; otherwise the direct kernels take every call, which is how the two
are set side by side here. Sizes cover a ragged end (n mod 32 != 0, computed with
direct loads by one warp), an exact multiple of the 32-element warp tile,
one tile a warp and many (each warp's two-stage ring reused with its
barrier phases flipping), scalar and NULL operands (read directly, beside
staged ones), an output that is an input, and a misaligned operand (sent
to the direct kernel)."""
import os

import numpy as np
import pytest

import cftgb
from cftgb import workload as wl

pytestmark = pytest.mark.gpu

BULK_MIN = 1 << 16


class staging:
    """CFTG_ELEM_STAGING for the calls inside the block."""

    def __init__(self, mode):
        self.mode = mode

    def __enter__(self):
        self.old = os.environ.get("CFTG_ELEM_STAGING")
        if self.mode is None:
            os.environ.pop("CFTG_ELEM_STAGING", None)
        else:
            os.environ["CFTG_ELEM_STAGING"] = self.mode

    def __exit__(self, *a):
        if self.old is None:
            os.environ.pop("CFTG_ELEM_STAGING", None)
        else:
            os.environ["CFTG_ELEM_STAGING"] = self.old


def _dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x).view(np.int32)).cuda()


def to_dev(fmt, arrays, offset=0):
    """device copies of (n, W) operand arrays (None stays None), each with
    `offset` elements of padding before its first element; returns the
    tensors and the operands' device addresses"""
    import torch
    W = wl.words(fmt)
    ts, ptrs = [], []
    for x in arrays:
        if x is None:
            ts.append(None)
            ptrs.append(None)
            continue
        t = torch.zeros((x.shape[0] + offset, W), dtype=torch.int32, device="cuda")
        t[offset:] = _dev(x)
        ts.append(t)
        ptrs.append(t[offset:].data_ptr())
    return ts, ptrs


def run_ptrs(h, kind, fmt, op, rnd, ptrs, n, scalar_mask=0, lane_flags=True):
    """(values, lane flags or None, flag word) through cftg_run_device"""
    import torch
    W = wl.words(fmt)
    td = torch.zeros((n, W), dtype=torch.int32, device="cuda")
    tf = torch.zeros(1, dtype=torch.int32, device="cuda")
    tl = torch.zeros(n, dtype=torch.uint8, device="cuda") if lane_flags else None
    st = cftgb.lib().cftg_run_device(h, kind, op, fmt, rnd, ptrs[0], ptrs[1], ptrs[2],
                                     td.data_ptr(), n, scalar_mask,
                                     tl.data_ptr() if tl is not None else None, tf.data_ptr(),
                                     torch.cuda.current_stream().cuda_stream)
    cftgb._lib.check(st, "cftg_run_device")
    torch.cuda.synchronize()
    word = int(tf.item()) & 0xFFFFFFFF
    assert not word & 0x80000000, "a staged load timed out"
    return (td.cpu().numpy().view(np.uint32), tl.cpu().numpy() if tl is not None else None, word)


def run_dev(h, kind, fmt, op, rnd, a, b, c, n, scalar_mask=0, lane_flags=True, offset=0):
    """run_ptrs over device copies of a, b, c, with the staged kernels asked for"""
    ts, ptrs = to_dev(fmt, (a, b, c), offset)
    with staging("bulk"):
        return run_ptrs(h, kind, fmt, op, rnd, ptrs, n, scalar_mask, lane_flags)


# (kind, op): FMA, ADD, SUB, MUL, then DIV, SQRT, then two simple opcodes
KINDS = [(0, 0), (0, 1), (0, 2), (0, 3), (1, 0), (2, 0), (0, 5), (0, 20)]


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
def test_staged_matches_oracle_ragged(gpu, oracle, fmt):
    """every kind at n = 65,536 + 37 against the oracle, element by element"""
    n = BULK_MIN + 37
    a, b, c = wl.gen_operands(fmt, n, 40 + fmt, ties=True, triples_frac=0.02)
    for kind, op in KINDS:
        for rnd in ((0, 3) if kind == 0 and op < 4 else (0,)):
            d, lf, acc = run_dev(gpu, kind, fmt, op, rnd, a, b, c, n)
            rd, rlf, racc = oracle.run(kind, fmt, op, rnd, a, b, c)
            bad = np.nonzero((d != rd).any(1) | (lf != rlf))[0]
            assert bad.size == 0, (fmt, kind, op, rnd, bad[:5])
            assert acc == racc, (fmt, kind, op, rnd, hex(acc), hex(racc))


@pytest.mark.parametrize("fmt", [1, 2, 3])
@pytest.mark.parametrize("n", [BULK_MIN, BULK_MIN + 1, 3 * BULK_MIN + 31, (1 << 21) + 5])
def test_staged_equals_direct(gpu, fmt, n):
    """the staged and the direct kernels on the same operands, every rounding
    attribute, with and without per-element flags"""
    ts, ptrs = to_dev(fmt, wl.gen_operands(fmt, n, 50 + fmt + n % 7))
    for kind, op in KINDS[:6]:
        for rnd in range(5):
            lfl = rnd != 4
            with staging("direct"):
                want = run_ptrs(gpu, kind, fmt, op, rnd, ptrs, n, lane_flags=lfl)
            with staging("bulk"):
                got = run_ptrs(gpu, kind, fmt, op, rnd, ptrs, n, lane_flags=lfl)
            assert np.array_equal(got[0], want[0]), (fmt, n, kind, op, rnd)
            if lfl:
                assert np.array_equal(got[1], want[1]), (fmt, n, kind, op, rnd)
            assert got[2] == want[2], (fmt, n, kind, op, rnd)


def test_staged_scalar_and_null_operands(gpu, oracle):
    """a scalar addend (read directly) beside staged a and b; MUL with c NULL;
    ADD with b NULL; scalar a for every operand"""
    fmt, n = 3, BULK_MIN + 100
    a, b, c = wl.gen_operands(fmt, n, 61)
    for mask in (4, 1, 2, 5, 7):
        d, lf, acc = run_dev(gpu, 0, fmt, 0, 0, a, b, c, n, scalar_mask=mask)
        rd, rlf, racc = oracle.run(0, fmt, 0, 0, a, b, c, n=n, scalar_mask=mask)
        assert np.array_equal(d, rd) and np.array_equal(lf, rlf) and acc == racc, mask
    d, lf, acc = run_dev(gpu, 0, fmt, 3, 1, a, b, None, n)
    rd, rlf, racc = oracle.run(0, fmt, 3, 1, a, b, None)
    assert np.array_equal(d, rd) and np.array_equal(lf, rlf) and acc == racc
    d, lf, acc = run_dev(gpu, 0, fmt, 1, 2, a, None, c, n)
    rd, rlf, racc = oracle.run(0, fmt, 1, 2, a, None, c)
    assert np.array_equal(d, rd) and np.array_equal(lf, rlf) and acc == racc


def test_misaligned_operand_goes_direct(gpu, oracle):
    """binary64 operands 8 bytes off a 16-byte boundary cannot be bulk-copied;
    the call still computes every element"""
    fmt, n = 1, BULK_MIN + 3
    a, b, c = wl.gen_operands(fmt, n, 71)
    d, lf, acc = run_dev(gpu, 0, fmt, 0, 0, a, b, c, n, offset=1)
    rd, rlf, racc = oracle.run(0, fmt, 0, 0, a, b, c)
    assert np.array_equal(d, rd) and np.array_equal(lf, rlf) and acc == racc


def test_staged_output_aliases_input(gpu, oracle):
    """d == a: each warp reads its tile before it writes the same elements"""
    import torch
    fmt, n = 2, BULK_MIN + 9
    a, b, c = wl.gen_operands(fmt, n, 81)
    ta, tb, tc = _dev(a), _dev(b), _dev(c)
    tf = torch.zeros(1, dtype=torch.int32, device="cuda")
    with staging("bulk"):
        st = cftgb.lib().cftg_run_device(gpu, 0, 0, fmt, 0, ta.data_ptr(), tb.data_ptr(),
                                         tc.data_ptr(), ta.data_ptr(), n, 0, None, tf.data_ptr(),
                                         torch.cuda.current_stream().cuda_stream)
    cftgb._lib.check(st, "cftg_run_device")
    torch.cuda.synchronize()
    rd, _, racc = oracle.run(0, fmt, 0, 0, a, b, c)
    assert np.array_equal(ta.cpu().numpy().view(np.uint32), rd)
    assert int(tf.item()) == racc
