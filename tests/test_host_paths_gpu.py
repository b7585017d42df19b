"""The ways host data reaches the kernels, each against the oracle: the
direct route (pinned or page-table-visible host memory read in place), the
staged pipeline, misaligned host pointers, and resident buffers (cft_alloc)
with the reference's authority rule, aliasing and interior pointers."""
import ctypes
import os

import numpy as np
import pytest

import cftgb
from cftgb import workload as wl

pytestmark = pytest.mark.gpu


@pytest.fixture
def staged():
    os.environ["CFTG_HOST_ACCESS"] = "stage"
    yield
    del os.environ["CFTG_HOST_ACCESS"]


def _ref(oracle, fmt, op, rnd, a, b, c):
    return oracle.run(0, fmt, op, rnd, a, b, c)


@pytest.mark.parametrize("fmt", [1, 3])
def test_direct_and_staged_routes_agree(gpu, oracle, fmt):
    import torch
    n = 70001
    a, b, c = wl.gen_operands(fmt, n, 12)
    rd, _, racc = _ref(oracle, fmt, 0, 2, a, b, c)
    # pinned host buffers (the direct route where the GPU can map them)
    ta, tb, tc = (torch.from_numpy(x.view(np.int32)).pin_memory() for x in (a, b, c))
    td = torch.zeros_like(ta).pin_memory()
    fl = ctypes.c_uint32()
    L = cftgb.lib()
    cftgb._lib.check(L.cft_run(gpu, 0, fmt, 2, ta.data_ptr(), tb.data_ptr(), tc.data_ptr(),
                               td.data_ptr(), n, ctypes.byref(fl), None), "cft_run")
    assert np.array_equal(td.numpy().view(np.uint32), rd) and fl.value == racc
    # pageable numpy buffers
    d = np.zeros_like(a)
    assert cftgb.run(gpu, 0, fmt, 2, a, b, c, d, n) == racc
    assert np.array_equal(d, rd)


def test_staged_route(gpu, oracle, staged):
    fmt, n = 2, 50000
    a, b, c = wl.gen_operands(fmt, n, 13)
    d = np.zeros_like(a)
    fl = cftgb.run(gpu, 0, fmt, 0, a, b, c, d, n)
    rd, _, racc = _ref(oracle, fmt, 0, 0, a, b, c)
    assert np.array_equal(d, rd) and fl == racc


def test_misaligned_host_pointers(gpu, oracle):
    """Operands that start 4 bytes into a buffer: staged, never handed to a
    vector load."""
    fmt, n = 3, 3000
    a, b, c = wl.gen_operands(fmt, n, 14)
    rd, _, racc = _ref(oracle, fmt, 0, 0, a, b, c)
    views = []                                            # 4 bytes past a 16-byte boundary
    for k, x in enumerate((a, b, c)):
        v = np.zeros(x.size * 4 + 64, np.uint8)
        o = (-v.ctypes.data) % 16 + 4
        v[o:o + x.size * 4] = x.view(np.uint8).ravel()
        views.append((v, o))
    out = np.zeros(a.size * 4 + 64, np.uint8)
    oo = (-out.ctypes.data) % 16 + 4
    L = cftgb.lib()
    fl = ctypes.c_uint32()
    p = [v.ctypes.data + o for v, o in views]
    cftgb._lib.check(L.cft_run(gpu, 0, fmt, 0, p[0], p[1], p[2], out.ctypes.data + oo, n,
                               ctypes.byref(fl), None), "cft_run")
    got = out[oo:oo + a.size * 4].view(np.uint32).reshape(a.shape)
    assert np.array_equal(got, rd) and fl.value == racc


def test_resident_buffers_authority_and_aliasing(gpu, oracle):
    L = cftgb.lib()
    fmt, n = 3, 4096
    esz = 32
    a, b, c = wl.gen_operands(fmt, n, 15)
    bufs = []
    for x in (a, b, c):
        h = ctypes.c_void_p()
        cftgb._lib.check(L.cft_alloc(gpu, x.nbytes, ctypes.byref(h)), "cft_alloc")
        ctypes.memmove(L.cft_buffer_data(h), x.ctypes.data, x.nbytes)
        cftgb._lib.check(L.cft_buffer_to_device(h), "publish")
        bufs.append(h)
    pa, pb, pc = (L.cft_buffer_data(h) for h in bufs)
    fl = ctypes.c_uint32()
    # d aliases a, in place on the device copy
    cftgb._lib.check(L.cft_run(gpu, 0, fmt, 0, pa, pb, pc, pa, n, ctypes.byref(fl), None), "run")
    rd, _, racc = _ref(oracle, fmt, 0, 0, a, b, c)
    # the mirror is stale until read back; a publish is refused meanwhile
    assert L.cft_buffer_to_device(bufs[0]) == 1
    cftgb._lib.check(L.cft_buffer_from_device(bufs[0]), "read back")
    got = np.ctypeslib.as_array((ctypes.c_uint32 * (n * 8)).from_address(pa)).reshape(n, 8)
    assert np.array_equal(got, rd) and fl.value == racc
    # an interior window, fed back as an input without a read-back first
    half = n // 2
    cftgb._lib.check(L.cft_run(gpu, 1, fmt, 0, pa + half * esz, None, pc, pb, half,
                               ctypes.byref(fl), None), "run interior")
    cftgb._lib.check(L.cft_buffer_from_device(bufs[1]), "read back b")
    rd2, _, _ = _ref(oracle, fmt, 1, 0, rd[half:], None, c[:half])
    gotb = np.ctypeslib.as_array((ctypes.c_uint32 * (half * 8)).from_address(pb)).reshape(half, 8)
    assert np.array_equal(gotb, rd2)
    for h in bufs:
        L.cft_buffer_free(h)
