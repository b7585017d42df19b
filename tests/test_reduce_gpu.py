"""Reductions on the GPU (cft_reduce, cft_reduce_seg, cftg_reduce_device)
against the oracle's restatement of the reference tree: every opcode,
format and rounding attribute; lengths around the chunk size (2048) and
its square, so every level of the multi-CTA tree and every fold of the
leftover blocks is exercised; IEEE 754-2019 9.4's infinity rule; the
identities of an empty reduction; segments on both paths."""
import ctypes

import numpy as np
import pytest

import cftgb
from cftgb import workload as wl

pytestmark = pytest.mark.gpu

OPS = (24, 25, 28, 29, 31)
vp, sz = ctypes.c_void_p, ctypes.c_size_t
u32p = ctypes.POINTER(ctypes.c_uint32)


def _bind(L, oracle):
    i = ctypes.c_int
    L.cft_reduce.argtypes = [vp, i, i, i, vp, vp, vp, sz, u32p, u32p]
    L.cft_reduce_seg.argtypes = [vp, i, i, i, vp, vp, vp, sz, sz, u32p, u32p]
    L.cftg_reduce_device.argtypes = [vp, i, i, i, vp, vp, vp, sz, sz, vp, vp, vp]
    L.cftg_reduce_partial_bytes.argtypes = [i, sz]
    L.cftg_reduce_partial_bytes.restype = sz
    oracle.L.sfp_reduce.argtypes = [i, i, i, vp, vp, vp, sz, u32p]
    oracle.L.sfp_reduce_seg.argtypes = [i, i, i, vp, vp, vp, sz, sz, u32p]


def operands(fmt, n, seed, plant=()):
    a, b, _ = wl.gen_operands(fmt, max(n, 1), seed, special_frac=0.0, exp_range=12,
                              triples_frac=0.0)
    a, b = a[:n].copy(), b[:n].copy()
    if plant and n:
        e_w, m_w = wl.GEOM[fmt]
        expmask = ((1 << e_w) - 1) << m_w
        vals = {"inf": expmask, "-inf": expmask | (1 << (e_w + m_w)),
                "qnan": expmask | (1 << (m_w - 1)), "snan": expmask | 1}
        rng = np.random.default_rng(seed)
        for name in plant:
            a[int(rng.integers(0, n))] = wl.from_int(vals[name], wl.words(fmt))
    return a, b


def gpu_reduce(L, h, op, fmt, rnd, a, b, n):
    d = np.zeros(wl.words(fmt), np.uint32)
    fl = ctypes.c_uint32()
    st = L.cft_reduce(h, op, fmt, rnd, a.ctypes.data if n else None,
                      b.ctypes.data if (n and op == 25) else None, d.ctypes.data, n,
                      ctypes.byref(fl), None)
    assert st == 0, (op, fmt, rnd, n)
    return d, fl.value


def oracle_reduce(oracle, op, fmt, rnd, a, b, n):
    d = np.zeros(wl.words(fmt), np.uint32)
    fl = ctypes.c_uint32()
    assert oracle.L.sfp_reduce(fmt, op, rnd, a.ctypes.data if n else None,
                               b.ctypes.data if n else None, d.ctypes.data, n,
                               ctypes.byref(fl)) == 0
    return d, fl.value


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
def test_reduce_matches_oracle(gpu, oracle, fmt):
    L = cftgb.lib()
    _bind(L, oracle)
    for n in (0, 1, 2, 3, 7, 8, 255, 256, 257, 2047, 2048, 2049, 6147, 2048 * 5 + 1000):
        a, b = operands(fmt, n, 100 * fmt + n)
        for op in OPS:
            for rnd in range(5):
                g = gpu_reduce(L, gpu, op, fmt, rnd, a, b, n)
                o = oracle_reduce(oracle, op, fmt, rnd, a, b, n)
                assert np.array_equal(g[0], o[0]) and g[1] == o[1], (op, n, rnd)


@pytest.mark.parametrize("fmt,n", [(1, 2048 * 2048 + 2048 * 3 + 5), (3, 2048 * 2048 + 7)])
def test_reduce_two_chunk_levels(gpu, oracle, fmt, n):
    L = cftgb.lib()
    _bind(L, oracle)
    a, b = operands(fmt, n, 9)
    for op in (24, 25):
        g = gpu_reduce(L, gpu, op, fmt, 2, a, b, n)
        o = oracle_reduce(oracle, op, fmt, 2, a, b, n)
        assert np.array_equal(g[0], o[0]) and g[1] == o[1], op


@pytest.mark.parametrize("plant", [["inf"], ["qnan"], ["snan"], ["inf", "qnan"], ["inf", "snan"],
                                   ["-inf", "inf"], ["snan", "-inf", "qnan"]])
def test_reduce_specials(gpu, oracle, plant):
    L = cftgb.lib()
    _bind(L, oracle)
    for fmt in (0, 1, 3):
        for n in (1, 2, 9, 3000):
            a, b = operands(fmt, n, 7 + n, plant=plant)
            for op in OPS:
                g = gpu_reduce(L, gpu, op, fmt, 0, a, b, n)
                o = oracle_reduce(oracle, op, fmt, 0, a, b, n)
                assert np.array_equal(g[0], o[0]) and g[1] == o[1], (op, n, plant)


def test_reduce_seg_both_paths(gpu, oracle):
    L = cftgb.lib()
    _bind(L, oracle)
    for fmt, n, segs in ((0, 6000, (1, 3, 100, 2000, 3000)), (2, 4096 * 3, (2048, 4096, 6144)),
                         (1, 2 * 70000, (70000,)), (3, 2049 * 4, (2049,))):
        a, b = operands(fmt, n, 55, plant=["inf", "qnan"] if fmt == 0 else [])
        W = wl.words(fmt)
        for op in OPS:
            for seg in segs:
                g = np.zeros((n // seg, W), np.uint32)
                o = np.zeros_like(g)
                gf, of = ctypes.c_uint32(), ctypes.c_uint32()
                assert L.cft_reduce_seg(gpu, op, fmt, 3, a.ctypes.data,
                                        b.ctypes.data if op == 25 else None, g.ctypes.data, n, seg,
                                        ctypes.byref(gf), None) == 0
                assert oracle.L.sfp_reduce_seg(fmt, op, 3, a.ctypes.data, b.ctypes.data,
                                               o.ctypes.data, n, seg, ctypes.byref(of)) == 0
                assert np.array_equal(g, o) and gf.value == of.value, (fmt, op, seg)


def test_reduce_device_entry_and_refusals(gpu, oracle):
    import torch
    L = cftgb.lib()
    _bind(L, oracle)
    fmt, n = 3, 10000
    a, b = operands(fmt, n, 3)
    ta, tb = (torch.from_numpy(x.view(np.int32)).cuda() for x in (a, b))
    out = torch.zeros(8, dtype=torch.int32, device="cuda")
    word = torch.zeros(2, dtype=torch.int32, device="cuda")
    part = torch.zeros(max(1, L.cftg_reduce_partial_bytes(fmt, n)) // 4 + 1, dtype=torch.int32,
                       device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    for op in OPS:
        assert L.cftg_reduce_device(gpu, op, fmt, 1, ta.data_ptr(), tb.data_ptr(), out.data_ptr(),
                                    n, n, part.data_ptr(), word.data_ptr(), s) == 0
        torch.cuda.synchronize()
        o = oracle_reduce(oracle, op, fmt, 1, a, b, n)
        assert np.array_equal(out.cpu().numpy().view(np.uint32), o[0])
        assert (int(word[0].item()) & 0x1F) == o[1]
    d = np.zeros(8, np.uint32)
    fl = ctypes.c_uint32()
    assert L.cft_reduce(gpu, 1, fmt, 0, a.ctypes.data, None, d.ctypes.data, n, ctypes.byref(fl),
                        None) == 1                     # ADD is elementwise: refused
    assert L.cft_reduce(gpu, 25, fmt, 0, a.ctypes.data, None, d.ctypes.data, n, ctypes.byref(fl),
                        None) == 1                     # DOT reads b
    assert L.cft_reduce_seg(gpu, 24, fmt, 0, a.ctypes.data, None, d.ctypes.data, 10, 3,
                            ctypes.byref(fl), None) == 1   # 10 is not whole segments of 3
    assert L.cft_reduce_seg(gpu, 24, fmt, 0, a.ctypes.data, None, d.ctypes.data, 10, 0,
                            ctypes.byref(fl), None) == 1
    # MAXALL of nothing is -inf; one signalling NaN comes back verbatim, no flags
    assert L.cft_reduce(gpu, 31, fmt, 0, None, None, d.ctypes.data, 0, ctypes.byref(fl), None) == 0
    assert d[-1] == 0xFFFFF000 and not d[:-1].any() and fl.value == 0
    sn = operands(fmt, 1, 1, plant=["snan"])[0]
    for op in (24, 31):
        assert L.cft_reduce(gpu, op, fmt, 0, sn.ctypes.data, None, d.ctypes.data, 1,
                            ctypes.byref(fl), None) == 0
        assert np.array_equal(d, sn[0]) and fl.value == 0
