"""Programs as source: the `.cfta` assembler, the character conversions it
reads literals with, and the ODE programs' default banks - libcft_gb300's
cftg_asm_* / cftg_from_char / cftg_ode_bank calls, with the names of the
reference's python/cft_golden/asm.py (`assemble`, `disassemble`, `info`)
and chars.py (`from_decimal`, `from_hex`). No device is needed.
"""
import ctypes

from ._lib import CftError, lib

_BOUND = False


def _L():
    global _BOUND
    L = lib()
    if not _BOUND:
        vp, sz = ctypes.c_void_p, ctypes.c_size_t
        L.cftg_asm_assemble.argtypes = [ctypes.c_char_p, sz, ctypes.c_char_p,
                                        ctypes.POINTER(vp), ctypes.POINTER(sz)]
        L.cftg_asm_assemble.restype = ctypes.c_int
        for f in ("cftg_asm_disassemble", "cftg_asm_info"):
            getattr(L, f).argtypes = [ctypes.c_char_p, sz, ctypes.POINTER(vp)]
            getattr(L, f).restype = ctypes.c_int
        L.cftg_asm_free.argtypes = [vp]
        L.cftg_asm_free.restype = None
        L.cftg_ode_bank.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p, vp, sz,
                                    ctypes.POINTER(sz)]
        L.cftg_ode_bank.restype = ctypes.c_int
        L.cftg_from_char.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_char_p,
                                     vp, ctypes.POINTER(ctypes.c_uint32)]
        L.cftg_from_char.restype = ctypes.c_int
        L.cftg_program_load_source.argtypes = [vp, ctypes.c_char_p, sz, ctypes.c_char_p,
                                               ctypes.POINTER(vp)]
        L.cftg_program_load_source.restype = ctypes.c_int
        _BOUND = True
    return L


class AsmError(CftError):
    """A source the assembler refuses or an image it cannot read; the
    message is the library's ("source:line: reason")."""


def _raise(st, where):
    L = lib()
    raise AsmError(st, where, L.cft_strerror(st).decode(), L.cft_last_error().decode())


def _bytes(text):
    return text if isinstance(text, (bytes, bytearray)) else text.encode("utf-8")


def assemble(text, source="<text>"):
    """`.cfta` source (str, or the bytes of a file) -> the `.cftp` image bytes."""
    L = _L()
    data = bytes(_bytes(text))
    p, n = ctypes.c_void_p(), ctypes.c_size_t()
    st = L.cftg_asm_assemble(data, len(data), source.encode(), ctypes.byref(p), ctypes.byref(n))
    if st:
        _raise(st, "cftg_asm_assemble")
    try:
        return ctypes.string_at(p, n.value)
    finally:
        L.cftg_asm_free(p)


def _text_call(fn, image, where):
    p = ctypes.c_void_p()
    img = bytes(image)
    st = fn(img, len(img), ctypes.byref(p))
    if st:
        _raise(st, where)
    try:
        return ctypes.string_at(p).decode()
    finally:
        _L().cftg_asm_free(p)


def disassemble(image):
    """An image -> `.cfta` text that assembles back to the same bytes."""
    return _text_call(_L().cftg_asm_disassemble, image, "cftg_asm_disassemble")


def info(image):
    """The header report `cft-asm -i` prints, with the image's SHA-256."""
    return _text_call(_L().cftg_asm_info, image, "cftg_asm_info")


def ode_bank(system, fmt, h):
    """The default bank of an ODE segment program ("lorenz63-rk4",
    "lorenz96-rk4", "henonheiles-lf") at format fmt (0..3) for step h (a
    decimal string), as programs/gen_odes.py:bank_values derives it."""
    L = _L()
    need = ctypes.c_size_t()
    st = L.cftg_ode_bank(system.encode(), fmt, h.encode(), None, 0, ctypes.byref(need))
    if st:
        _raise(st, "cftg_ode_bank")
    buf = ctypes.create_string_buffer(need.value)
    st = L.cftg_ode_bank(system.encode(), fmt, h.encode(), buf, need.value, ctypes.byref(need))
    if st:
        _raise(st, "cftg_ode_bank")
    return buf.raw[:need.value]


def _from_char(hexf, fmt, s, rnd):
    L = _L()
    buf = ctypes.create_string_buffer(32)
    fl = ctypes.c_uint32()
    st = L.cftg_from_char(hexf, fmt, rnd, _bytes(s), buf, ctypes.byref(fl))
    if st:
        _raise(st, "cftg_from_char")
    return int.from_bytes(buf.raw[:4 << fmt], "little"), fl.value


def from_decimal(fmt, s, rnd=0):
    """A decimal sequence -> (encoding as an int, flags), correctly rounded."""
    return _from_char(0, fmt, s, rnd)


def from_hex(fmt, s, rnd=0):
    """A hexadecimal-significand sequence -> (encoding as an int, flags)."""
    return _from_char(1, fmt, s, rnd)


def load_source(dev, text, source="<text>"):
    """Assemble and cft_program_load in one call; returns the program handle."""
    L = _L()
    data = bytes(_bytes(text))
    prog = ctypes.c_void_p()
    st = L.cftg_program_load_source(dev, data, len(data), source.encode(), ctypes.byref(prog))
    if st:
        _raise(st, "cftg_program_load_source")
    return prog
