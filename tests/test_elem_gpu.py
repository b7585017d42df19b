"""Parity of the GPU elementwise path with the oracle, bit for bit in values
and in every element's flags, through the C ABI (cft_run / cft_div /
cft_sqrt with host buffers; cftg_run_device with device buffers and a
per-element flag byte)."""
import ctypes
from pathlib import Path

import numpy as np
import pytest

import cftgb
from cftgb import workload as wl

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
DIV, SQRT = 1000, 1001
ARITH = [0, 1, 2, 3]
SIMPLE = [o for o in range(32) if o not in (0, 1, 2, 3, 24, 25, 28, 29, 31)] + [40, 255]


def device_run(h, kind, fmt, op, rnd, a, b, c, n=None, scalar_mask=0):
    """values and per-element flags through cftg_run_device"""
    import torch
    n = a.shape[0] if n is None else n
    W = wl.words(fmt)
    ta = torch.from_numpy(a.view(np.int32)).cuda()
    tb = torch.from_numpy(b.view(np.int32)).cuda() if b is not None else None
    tc = torch.from_numpy(c.view(np.int32)).cuda() if c is not None else None
    td = torch.zeros((n, W), dtype=torch.int32, device="cuda")
    tf = torch.zeros(1, dtype=torch.int32, device="cuda")
    tl = torch.zeros(n, dtype=torch.uint8, device="cuda")
    st = cftgb.lib().cftg_run_device(
        h, kind, op, fmt, rnd, ta.data_ptr(), tb.data_ptr() if tb is not None else None,
        tc.data_ptr() if tc is not None else None, td.data_ptr(), n, scalar_mask, tl.data_ptr(),
        tf.data_ptr(), torch.cuda.current_stream().cuda_stream)
    cftgb._lib.check(st, "cftg_run_device")
    torch.cuda.synchronize()
    return td.cpu().numpy().view(np.uint32), tl.cpu().numpy(), int(tf.item())


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
def test_golden_vectors_on_gpu(gpu, fmt):
    g = np.load(GOLD / f"golden_{wl.geometry(fmt)['width']}.npz")
    ops = g["op"]
    for key in sorted(set(zip(ops.tolist(), g["rnd"].tolist()))):
        op, rnd = key
        sel = (ops == op) & (g["rnd"] == rnd)
        kind = 1 if op == DIV else 2 if op == SQRT else 0
        d, lf, acc = device_run(gpu, kind, fmt, 0 if kind else op, rnd, g["a"][sel], g["b"][sel],
                                g["c"][sel])
        assert np.array_equal(d, g["d"][sel]), (fmt, op, rnd)
        assert np.array_equal(lf, g["flags"][sel]), (fmt, op, rnd)


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
def test_arith_matches_oracle_per_element(gpu, oracle, fmt):
    n = 1 << 14
    a, b, c = wl.gen_operands(fmt, n, 11 + fmt, ties=True)
    for op in ARITH:
        for rnd in range(5):
            d, lf, acc = device_run(gpu, 0, fmt, op, rnd, a, b, c)
            rd, rlf, racc = oracle.run(0, fmt, op, rnd, a, b, c)
            bad = np.nonzero((d != rd).any(1) | (lf != rlf))[0]
            assert bad.size == 0, (fmt, op, rnd, bad[:5], d[bad[:1]], rd[bad[:1]], lf[bad[:1]], rlf[bad[:1]])
            assert acc == racc


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
def test_div_sqrt_match_oracle_per_element(gpu, oracle, fmt):
    n = 1 << 12
    a, b, c = wl.gen_operands(fmt, n, 21 + fmt, ties=True)
    for kind in (1, 2):
        for rnd in range(5):
            d, lf, acc = device_run(gpu, kind, fmt, 0, rnd, a, b, None)
            rd, rlf, racc = oracle.run(kind, fmt, 0, rnd, a, b, None)
            bad = np.nonzero((d != rd).any(1) | (lf != rlf))[0]
            assert bad.size == 0, (fmt, kind, rnd, bad[:5])


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
def test_simple_ops_match_oracle(gpu, oracle, fmt):
    n = 4096
    a, b, c = wl.gen_operands(fmt, n, 31 + fmt)
    for op in SIMPLE:
        d, lf, acc = device_run(gpu, 0, fmt, op, 0, a, b, c)
        rd, rlf, racc = oracle.run(0, fmt, op, 0, a, b, c)
        bad = np.nonzero((d != rd).any(1) | (lf != rlf))[0]
        assert bad.size == 0, (fmt, op, bad[:5])


@pytest.mark.parametrize("fmt", [0, 3])
def test_cft_run_host_buffers_and_chunks(gpu, oracle, fmt):
    """cft_run through host buffers, across several pipeline chunks, with
    odd sizes and the empty call."""
    esz = wl.words(fmt) * 4
    n = (40 << 20) // esz + 37               # > one 32 MiB chunk, ragged tail
    a, b, c = wl.gen_operands(fmt, n, 5, special_frac=0.1)
    d = np.zeros_like(a)
    fl = cftgb.run(gpu, 0, fmt, 0, a, b, c, d, n)
    rd, rlf, racc = oracle.run(0, fmt, 0, 0, a[:4096], b[:4096], c[:4096])
    assert np.array_equal(d[:4096], rd)
    tail = slice(n - 3000, n)
    rd2, _, _ = oracle.run(0, fmt, 0, 0, a[tail], b[tail], c[tail])
    assert np.array_equal(d[tail], rd2)
    # OR of flags equals the oracle's over the whole array (checked on a
    # sample: every flag the sample raises must be in the call's word)
    assert (racc & ~fl) == 0
    assert cftgb.run(gpu, 0, fmt, 0, a, b, c, d, 0) == 0


def test_aliasing_and_null_operands(gpu, oracle):
    fmt = 2
    n = 1000
    a, b, c = wl.gen_operands(fmt, n, 8)
    # ADD with b NULL; d aliasing a
    x = a.copy()
    fl = cftgb.run(gpu, 1, fmt, 3, x, None, c, x, n)
    rd, _, racc = oracle.run(0, fmt, 1, 3, a, None, c)
    assert np.array_equal(x, rd) and fl == racc
    # MUL with c NULL
    d = np.zeros_like(a)
    cftgb.run(gpu, 3, fmt, 0, a, b, None, d, n)
    rd, _, _ = oracle.run(0, fmt, 3, 0, a, b, None)
    assert np.array_equal(d, rd)
    # FMA with b NULL is an argument error
    with pytest.raises(cftgb.CftError) as e:
        cftgb.run(gpu, 0, fmt, 0, a, None, c, d, n)
    assert e.value.status == 1


@pytest.mark.parametrize("fmt", [0, 1, 3])
def test_run_ex_scalar_and_index_tables(gpu, oracle, fmt):
    n = 3000
    a, b, c = wl.gen_operands(fmt, n, 9)
    d = np.zeros_like(a)
    # scalar b: element 0 of b for every i
    cftgb.run_ex(gpu, 0, fmt, 0, a, b, c, d, n, scalar_mask=2)
    bb = np.repeat(b[:1], n, 0)
    rd, _, _ = oracle.run(0, fmt, 0, 0, a, bb, c)
    assert np.array_equal(d, rd)
    # gather a through a table with CFT_IDX_NONE entries
    src = a[:500].copy()
    idx = np.random.default_rng(3).integers(0, 500, n).astype(np.uint32)
    idx[::7] = 0xFFFFFFFF
    d2 = np.zeros_like(a)
    cftgb.run_ex(gpu, 0, fmt, 0, src, b, c, d2, n, idx=(idx, None, None), src=(500, 0, 0))
    ga = np.where((idx == 0xFFFFFFFF)[:, None], 0, src[np.minimum(idx, 499)]).astype(np.uint32)
    rd2, _, _ = oracle.run(0, fmt, 0, 0, ga, b, c)
    assert np.array_equal(d2, rd2)
    # an index past the source is refused before the run
    idx[5] = 500
    with pytest.raises(cftgb.CftError) as e:
        cftgb.run_ex(gpu, 0, fmt, 0, src, b, c, d2, n, idx=(idx, None, None), src=(500, 0, 0))
    assert e.value.status == 1 and "idx_a[5]" in e.value.detail


def test_unassigned_and_reduction_opcodes(gpu):
    fmt = 1
    a = np.zeros((4, 2), np.uint32)
    d = np.zeros_like(a)
    fl = cftgb.run(gpu, 200, fmt, 0, a, a, a, d, 4)
    assert fl == 1 and (d[:, 1] == 0x7FF80000).all() and (d[:, 0] == 0).all()
    for op in (24, 25, 28, 29, 31, 256, -1):
        with pytest.raises(cftgb.CftError) as e:
            cftgb.run(gpu, op, fmt, 0, a, a, a, d, 4)
        assert e.value.status == 1


def test_status_word_accumulates_and_mute_free(gpu):
    L = cftgb.lib()
    L.cft_lower_flags(gpu, 31)
    fmt = 0
    a = np.array([[0x7F800000]], np.uint32)      # +inf
    z = np.array([[0]], np.uint32)
    d = np.zeros_like(a)
    cftgb.run(gpu, 3, fmt, 0, a, z, None, d, 1)  # inf * 0 -> invalid
    assert L.cft_save_all_flags(gpu) & 1
    L.cft_lower_flags(gpu, 1)
    assert L.cft_save_all_flags(gpu) & 1 == 0
