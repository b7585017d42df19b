"""The C ABI's struct and empty-call conventions on a GPU handle (the
reference's host/include/cft.h:244-303 and the struct_size handshake of
cft_get_caps, cft_program_get_info, cft_run_ex and cft_program_run_ex): an
input struct of the wrong struct_size is refused with an argument error and
a sentence, an output struct is filled up to the caller's struct_size and no
further, and a call over zero elements writes nothing and raises nothing."""
import ctypes

import numpy as np
import pytest

import cftgb
import seq_util as su
from cftgb import _lib
from cftgb import workload as wl

pytestmark = pytest.mark.gpu

ERR_ARG = 1


def _filled(size, byte=0xAB):
    buf = (ctypes.c_uint8 * size)()
    ctypes.memset(buf, byte, size)
    return buf


def test_caps_fill_up_to_the_callers_size(gpu):
    L = cftgb.lib()
    full = ctypes.sizeof(_lib.Caps)
    caps = lambda buf: ctypes.cast(buf, ctypes.POINTER(_lib.Caps))  # noqa: E731
    # a caller that knows only struct_size and format_mask
    small = 8 + 4
    buf = _filled(full)
    ctypes.c_size_t.from_buffer(buf, 0).value = small
    assert L.cft_get_caps(gpu, caps(buf)) == 0
    assert ctypes.c_size_t.from_buffer(buf, 0).value == small
    assert ctypes.c_uint32.from_buffer(buf, 8).value == 0xF
    assert bytes(buf[small:]) == b"\xab" * (full - small)
    # a caller whose struct is larger than this library's: only the known part
    buf = _filled(full + 64)
    ctypes.c_size_t.from_buffer(buf, 0).value = full + 64
    assert L.cft_get_caps(gpu, caps(buf)) == 0
    assert ctypes.c_size_t.from_buffer(buf, 0).value == full
    assert bytes(buf[full:]) == b"\xab" * 64
    # smaller than the struct_size field itself
    buf = _filled(full)
    ctypes.c_size_t.from_buffer(buf, 0).value = 4
    assert L.cft_get_caps(gpu, caps(buf)) == ERR_ARG
    assert b"struct_size" in L.cft_last_error()


def test_run_ex_refuses_a_wrong_struct_size(gpu):
    L = cftgb.lib()
    fmt, n = 3, 64
    a, b, c = wl.gen_operands(fmt, n, 3)
    d = np.full_like(a, 0x5A5A5A5A)
    fl = ctypes.c_uint32(0)
    e = _lib.ElemArgs()
    e.a, e.b, e.c, e.d, e.n = a.ctypes.data, b.ctypes.data, c.ctypes.data, d.ctypes.data, n
    e.flags_out = ctypes.pointer(fl)
    for size in (ctypes.sizeof(e) - 8, ctypes.sizeof(e) + 8, 0):
        e.struct_size = size
        assert L.cft_run_ex(gpu, 0, fmt, 0, ctypes.byref(e)) == ERR_ARG, size
        assert b"cft_elem_args" in L.cft_last_error()
    assert (d == 0x5A5A5A5A).all() and fl.value == 0
    e.struct_size = ctypes.sizeof(e)
    assert L.cft_run_ex(gpu, 0, fmt, 0, ctypes.byref(e)) == 0
    assert not (d == 0x5A5A5A5A).all()


def _program(gpu):
    case = next(c for c in map(su.load, su.cases()) if not su.uses_augadd(c["image"]))
    prog = ctypes.c_void_p()
    img = case["image"]
    _lib.check(cftgb.lib().cft_program_load(gpu, img.ctypes.data, img.size, ctypes.byref(prog)),
               "cft_program_load")
    return prog, case


def test_program_info_fills_up_to_the_callers_size(gpu):
    L = cftgb.lib()
    prog, case = _program(gpu)
    try:
        full = ctypes.sizeof(_lib.ProgramInfo)
        small = 8 + 4                                 # struct_size and format
        buf = _filled(full)
        ctypes.c_size_t.from_buffer(buf, 0).value = small
        assert L.cft_program_get_info(prog, ctypes.cast(buf, ctypes.POINTER(_lib.ProgramInfo))) == 0
        assert ctypes.c_size_t.from_buffer(buf, 0).value == small
        assert ctypes.c_int.from_buffer(buf, 8).value == su.header(case["image"])["prec"]
        assert bytes(buf[small:]) == b"\xab" * (full - small)
    finally:
        L.cft_program_free(prog)


def test_program_run_ex_refuses_a_wrong_struct_size(gpu):
    L = cftgb.lib()
    prog, case = _program(gpu)
    try:
        A = _lib.RunArgs()
        A.n = 0
        for size in (ctypes.sizeof(A) - 8, ctypes.sizeof(A) + 8):
            A.struct_size = size
            assert L.cft_program_run_ex(prog, ctypes.byref(A)) == ERR_ARG, size
            assert b"cft_run_args" in L.cft_last_error()
    finally:
        L.cft_program_free(prog)


@pytest.mark.parametrize("fmt", [0, 3])
def test_empty_call_writes_and_raises_nothing(gpu, fmt):
    L = cftgb.lib()
    a, b, c = wl.gen_operands(fmt, 8, 5)
    d = np.full_like(a, 0x5A5A5A5A)
    fl = ctypes.c_uint32(0)
    for op in (0, 1, 3, 15):
        assert L.cft_run(gpu, op, fmt, 0, a.ctypes.data, b.ctypes.data, c.ctypes.data,
                         d.ctypes.data, 0, ctypes.byref(fl), None) == 0
    assert L.cft_div(gpu, fmt, 0, a.ctypes.data, b.ctypes.data, d.ctypes.data, 0,
                     ctypes.byref(fl), None) == 0
    assert L.cft_sqrt(gpu, fmt, 0, a.ctypes.data, d.ctypes.data, 0, ctypes.byref(fl), None) == 0
    assert fl.value == 0
    assert (d == 0x5A5A5A5A).all()
