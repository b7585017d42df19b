"""Programs as source, and the batch character conversions, on a device
handle: a certificate's program submitted as `.cfta` text (its
disassembly) and run on the GPU gives the certificate's boundary hashes;
cft_from_decimal_char / cft_from_hex_char convert a batch as the
reference's chars.py does, with the flag OR and the bad index."""
import ctypes
import gzip
import hashlib
import json

import numpy as np
import pytest

import cftgb
from cftgb import asm
from cftgb._lib import RunArgs

import seq_util as su

pytestmark = pytest.mark.gpu
CORPUS = json.load(gzip.open(su.GOLD / "asm_corpus.json.gz", "rt"))


@pytest.mark.parametrize("cert", ["lorenz63", "henonheiles"])
def test_certificate_from_source(gpu, cert):
    z = np.load(su.GOLD / f"{cert}_cert.npz")
    src = asm.disassemble(z["image"].tobytes())
    prog = asm.load_source(gpu, src, f"{cert}.cfta")
    L = cftgb.lib()
    bank = z["bank"].copy()
    slots = su.header(z["image"])["sout"]
    state = z["state0"].copy().view(np.uint32).reshape(-1, 8)
    n = state.shape[0] // slots
    a = np.zeros((n, 8), np.uint32)
    tag = b"cft-certificate 1 state\0"
    try:
        for k, end in enumerate(z["ends"][:3]):
            out = np.zeros_like(state)
            fl, bus = ctypes.c_uint32(), ctypes.c_uint32()
            A = RunArgs()
            A.struct_size = ctypes.sizeof(RunArgs)
            A.a, A.n = a.ctypes.data, n
            A.bank, A.bank_bytes = bank.ctypes.data, bank.size
            A.scratch_in, A.scratch_in_bytes = state.ctypes.data, state.nbytes
            A.scratch_out, A.scratch_out_bytes = out.ctypes.data, out.nbytes
            A.flags_out, A.bus_out = ctypes.pointer(fl), ctypes.pointer(bus)
            cftgb._lib.check(L.cft_program_run_ex(prog, ctypes.byref(A)), "run")
            assert hashlib.sha256(tag + out.tobytes()).hexdigest() == str(end), f"segment {k}"
            assert fl.value == int(z["flags"][k]) and bus.value == int(z["status"][k])
            state = out
    finally:
        L.cft_program_free(prog)


def test_source_refusal_through_the_device_call(gpu):
    with pytest.raises(asm.AsmError) as e:
        asm.load_source(gpu, ".format fp64\n.deposits 1\nrepeat 0\nendrep\n", "k.cfta")
    assert "k.cfta:3:" in str(e.value)


def _batch(h, fn, fmt, rnd, strings):
    L = cftgb.lib()
    getattr(L, fn).argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                               ctypes.POINTER(ctypes.c_char_p), ctypes.c_void_p, ctypes.c_size_t,
                               ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_uint32)]
    arr = (ctypes.c_char_p * max(1, len(strings)))(*[s.encode() for s in strings])
    esz = 4 << fmt
    d = ctypes.create_string_buffer(esz * max(1, len(strings)))
    bad = ctypes.c_size_t(99)
    fl = ctypes.c_uint32(0)
    st = getattr(L, fn)(h, fmt, rnd, arr, d, len(strings), ctypes.byref(bad), ctypes.byref(fl))
    vals = [int.from_bytes(d.raw[i * esz:(i + 1) * esz], "little") for i in range(len(strings))]
    return st, vals, bad.value, fl.value


@pytest.mark.parametrize("key,fn", [("dec", "cft_from_decimal_char"), ("hex", "cft_from_hex_char")])
def test_batch_conversions(gpu, key, fn):
    for fmt in range(4):
        for rnd in range(5):
            ok = [r for r in CORPUS["sequences"] if r["fmt"] == fmt and r[key][rnd] is not None]
            bad = [r for r in CORPUS["sequences"] if r["fmt"] == fmt and r[key][rnd] is None]
            if not ok:
                continue
            st, vals, _, fl = _batch(gpu, fn, fmt, rnd, [r["s"] for r in ok])
            assert st == 0
            assert [format(v, "x") for v in vals] == [r[key][rnd][0] for r in ok]
            acc = 0
            for r in ok:
                acc |= r[key][rnd][1]
            assert fl == acc
            if bad:
                strings = [r["s"] for r in ok[:3]] + [bad[0]["s"]] + [r["s"] for r in ok[3:6]]
                st, _, where, _ = _batch(gpu, fn, fmt, rnd, strings)
                assert st == 1 and where == min(3, len(ok))
    st, _, where, fl = _batch(gpu, fn, 3, 0, [])
    assert st == 0 and fl == 0
