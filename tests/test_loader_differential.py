"""The program loader's decision against the reference's own (CPU tests).

Every image the reference ships (tests/golden/programs, assembled by the
reference's cft-asm) is mutated - header fields out of range, a wrong
length, reserved bits, and seeded random bit flips in instruction words -
and for every mutant the status of this library's cftg_program_check (the
whole of cft_program_load's decision, no device needed) must equal the
status of the reference library's cft_program_load on its software device
(host/src/program.c:601-800 and :1325-1420 define the refusals). The
reference library is the one oracle/Makefile compiles from the reference's
sources; where it is absent the test is skipped."""
import ctypes
from pathlib import Path

import numpy as np
import pytest

import cftgb
import seq_util as su
from cftgb import _lib

REF = Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "libcft_ref.so"
pytestmark = pytest.mark.skipif(not REF.exists(),
                                reason="the reference library (oracle/_ref) is not built here")


@pytest.fixture(scope="module")
def ref():
    R = ctypes.CDLL(str(REF))
    vp = ctypes.c_void_p
    R.cft_open.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(vp)]
    R.cft_close.argtypes = [vp]
    R.cft_get_caps.argtypes = [vp, ctypes.POINTER(_lib.Caps)]
    R.cft_program_load.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(vp)]
    R.cft_program_free.argtypes = [vp]
    R.cft_last_error.restype = ctypes.c_char_p
    h = vp()
    assert R.cft_open(None, 0, ctypes.byref(h)) == 0
    caps = _lib.Caps()
    caps.struct_size = ctypes.sizeof(caps)
    assert R.cft_get_caps(h, ctypes.byref(caps)) == 0
    yield R, h, caps
    R.cft_close(h)


def _ref_status(R, h, img):
    prog = ctypes.c_void_p()
    st = R.cft_program_load(h, img, len(img), ctypes.byref(prog))
    if st == 0:
        R.cft_program_free(prog)
    return st


def _ours(img, depth):
    L = cftgb.lib()
    L.cftg_program_check.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_uint32]
    return L.cftg_program_check(img, len(img), depth)


def _word(img, k, v):
    b = bytearray(img)
    b[4 * k:4 * k + 4] = int(v & 0xFFFFFFFF).to_bytes(4, "little")
    return bytes(b)


def _mutants(img, rng, flips):
    h = su.header(np.frombuffer(img, np.uint8))
    esz = (4, 8, 16, 32)[h["prec"]]
    base = 32 + (0 if h["flags"] & 1 else h["n_consts"] * esz)
    out = [
        ("short header", img[:31]),
        ("one instruction short", img[:-8]),
        ("one word long", img + b"\0\0\0\0"),
        ("magic", _word(img, 0, 0x50544644)),           # "DFTP"
        ("version 2", _word(img, 1, 2)),
        ("unknown header flag", _word(img, 6, h["flags"] | 0x80000000)),
        ("precision 4", _word(img, 5, 4)),
        ("more instructions than bytes", _word(img, 2, h["n_insns"] + 1)),
    ]
    if not h["flags"] & 2:
        out.append(("scratch_io without SCRATCH_IO", _word(img, 7, 0x00010001)))
    n = h["n_insns"]
    for j in range(flips):
        i = int(rng.integers(0, n))
        bit = int(rng.integers(0, 64))
        b = bytearray(img)
        off = base + 8 * i + bit // 8
        b[off] ^= 1 << (bit % 8)
        out.append((f"instruction {i} bit {bit}", bytes(b)))
    return out


def test_loader_refuses_what_the_reference_refuses(ref):
    R, h, caps = ref
    rng = np.random.default_rng(2024)
    checked = refused = 0
    mismatches = []
    for path in su.cases():
        img = bytes(su.load(path)["image"])
        assert _ours(img, caps.max_scratch) == _ref_status(R, h, img) == 0, path.name
        for what, m in _mutants(img, rng, 60):
            want = _ref_status(R, h, m)
            got = _ours(m, caps.max_scratch)
            checked += 1
            refused += want != 0
            if got != want:
                mismatches.append((path.name, what, got, want,
                                   cftgb.lib().cft_last_error(), R.cft_last_error()))
    assert not mismatches, mismatches[:5]
    assert checked > 2000 and refused > 500, (checked, refused)
