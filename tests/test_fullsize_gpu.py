"""Parity at the configurations' full size: binary256 FMA over 2^24
device-generated operands (the benchmark's value mix), through
cftg_run_device with per-element flag bytes. Elements sampled from the
whole array (not only its start) equal the oracle in value and flags, and
a size-independent property holds for every element: a*b+c and b*a+c are
the same bits with the same flags."""
import ctypes

import numpy as np
import pytest

import cftgb

pytestmark = pytest.mark.gpu


def test_fma_fp256_full_size(gpu, oracle):
    import torch
    L = cftgb.lib()
    vp = ctypes.c_void_p
    L.cftg_fill_operands.argtypes = [ctypes.c_int, vp, ctypes.c_size_t, ctypes.c_uint64,
                                     ctypes.c_int, ctypes.c_uint32, vp]
    fmt, W, n = 3, 8, 1 << 24
    s = torch.cuda.current_stream().cuda_stream
    ops = [torch.empty((n, W), dtype=torch.int32, device="cuda") for _ in range(3)]
    for j, t in enumerate(ops):
        cftgb._lib.check(L.cftg_fill_operands(fmt, t.data_ptr(), n, 77 + j, 64, 100000, s),
                         "cftg_fill_operands")
    a, b, c = ops

    def fma(x, y):
        d = torch.empty((n, W), dtype=torch.int32, device="cuda")
        lf = torch.empty(n, dtype=torch.uint8, device="cuda")
        w = torch.zeros(1, dtype=torch.int32, device="cuda")
        cftgb._lib.check(L.cftg_run_device(gpu, 0, 0, fmt, 0, x.data_ptr(), y.data_ptr(),
                                           c.data_ptr(), d.data_ptr(), n, 0, lf.data_ptr(),
                                           w.data_ptr(), s), "cftg_run_device")
        return d, lf, w

    d1, lf1, w1 = fma(a, b)
    d2, lf2, w2 = fma(b, a)
    torch.cuda.synchronize()
    assert torch.equal(d1, d2) and torch.equal(lf1, lf2) and torch.equal(w1, w2)

    rng = np.random.default_rng(5)
    idx = np.sort(rng.choice(n, size=8192, replace=False))
    idx[-1] = n - 1                                    # the last element too
    ti = torch.from_numpy(idx).cuda()
    host = [t.index_select(0, ti).cpu().numpy().view(np.uint32) for t in (a, b, c, d1)]
    lfs = lf1.index_select(0, ti).cpu().numpy()
    rd, rlf, _ = oracle.run(0, fmt, 0, 0, host[0], host[1], host[2])
    bad = np.nonzero((host[3] != rd).any(1) | (lfs != rlf))[0]
    assert bad.size == 0, idx[bad[:5]]
    # the call's flag word covers every flag the sample raised
    raised = int(np.bitwise_or.reduce(rlf.astype(np.uint32)))
    assert raised & ~(int(w1.item()) & 0xFFFFFFFF) == 0
