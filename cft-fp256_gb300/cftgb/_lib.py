"""ctypes binding of libcft_gb300's C ABI (include/cft.h, include/cft_gb300.h).

Mirrors the reference binding's calls (bindings/python/cftmpfr/_lib.py:
open_device, run, div, sqrt, get_caps, supports, check) so that code
written against it reads the same here. Loading fails loudly when the
library has not been built: there is no CPU path behind these calls.
"""
import ctypes
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent.parent
LIB_PATH = _PKG / "lib" / "libcft_gb300.so"

FMT_NAMES = ("fp32", "fp64", "fp128", "fp256")
ESZ = (4, 8, 16, 32)
OPS = {"fma": 0, "add": 1, "sub": 2, "mul": 3, "abs": 4, "neg": 5, "copysign": 6, "min": 7,
       "max": 8, "minnum": 9, "maxnum": 10, "select": 11, "cmplt": 12, "cmple": 13, "cmpeq": 14,
       "iand": 16, "ior": 17, "ixor": 18, "iadd": 19, "isub": 20, "ishl": 21, "ishr": 22,
       "icmplt": 23, "recip_seed": 26, "rsqrt_seed": 27, "imul": 30}
RND = {"rne": 0, "rtz": 1, "rdn": 2, "rup": 3, "rmm": 4}
KIND_OP, KIND_DIV, KIND_SQRT = 0, 1, 2

_LIB = None


class CftError(RuntimeError):
    def __init__(self, status, where, what, detail):
        super().__init__(f"{where}: {what} ({status}): {detail}")
        self.status = status
        self.where = where
        self.detail = detail


class Caps(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("format_mask", ctypes.c_uint32),
                ("tiles", ctypes.c_uint32), ("abi_version", ctypes.c_uint32),
                ("device_version", ctypes.c_uint32), ("flags_readable", ctypes.c_int),
                ("backend", ctypes.c_char * 32), ("max_deposits", ctypes.c_uint32),
                ("max_insns", ctypes.c_uint32), ("max_consts", ctypes.c_uint32),
                ("seq_features", ctypes.c_uint32), ("max_scratch", ctypes.c_uint32),
                ("buffers_resident", ctypes.c_int)]


class ElemArgs(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("a", ctypes.c_void_p), ("b", ctypes.c_void_p),
                ("c", ctypes.c_void_p), ("d", ctypes.c_void_p), ("n", ctypes.c_size_t),
                ("scalar_mask", ctypes.c_uint32), ("flags_out", ctypes.POINTER(ctypes.c_uint32)),
                ("bus_out", ctypes.POINTER(ctypes.c_uint32)), ("idx_a", ctypes.c_void_p),
                ("idx_b", ctypes.c_void_p), ("idx_c", ctypes.c_void_p),
                ("idx_a_src", ctypes.c_size_t), ("idx_b_src", ctypes.c_size_t),
                ("idx_c_src", ctypes.c_size_t)]


class RunArgs(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("a", ctypes.c_void_p), ("b", ctypes.c_void_p),
                ("c", ctypes.c_void_p), ("n", ctypes.c_size_t), ("bank", ctypes.c_void_p),
                ("bank_bytes", ctypes.c_size_t), ("scratch_in", ctypes.c_void_p),
                ("scratch_in_bytes", ctypes.c_size_t), ("scratch_out", ctypes.c_void_p),
                ("scratch_out_bytes", ctypes.c_size_t), ("deposits", ctypes.c_void_p),
                ("counts", ctypes.c_void_p), ("flags_out", ctypes.POINTER(ctypes.c_uint32)),
                ("bus_out", ctypes.POINTER(ctypes.c_uint32)), ("idx_a", ctypes.c_void_p),
                ("idx_b", ctypes.c_void_p), ("idx_c", ctypes.c_void_p),
                ("idx_a_src", ctypes.c_size_t), ("idx_b_src", ctypes.c_size_t),
                ("idx_c_src", ctypes.c_size_t), ("idx_scratch_in", ctypes.c_void_p),
                ("idx_scratch_src", ctypes.c_size_t), ("lane_mask", ctypes.c_void_p),
                ("lane_mask_bytes", ctypes.c_size_t), ("lane_flags", ctypes.c_void_p),
                ("lane_flags_bytes", ctypes.c_size_t)]


class ProgramInfo(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("format", ctypes.c_int),
                ("max_deposits", ctypes.c_uint32), ("n_insns", ctypes.c_uint32),
                ("n_consts", ctypes.c_uint32), ("flags", ctypes.c_uint32),
                ("n_scratch_in", ctypes.c_uint32), ("n_scratch_out", ctypes.c_uint32),
                ("scratch_used", ctypes.c_uint32)]


def _bind(L):
    c_int, u32, sz, vp, cp = ctypes.c_int, ctypes.c_uint32, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_char_p
    u32p = ctypes.POINTER(u32)
    L.cft_abi_version.restype = u32
    L.cft_strerror.argtypes = [c_int]
    L.cft_strerror.restype = cp
    L.cft_last_error.restype = cp
    L.cft_format_size.argtypes = [c_int]
    L.cft_format_size.restype = sz
    L.cft_format_name.argtypes = [c_int]
    L.cft_format_name.restype = cp
    L.cft_op_name.argtypes = [c_int]
    L.cft_op_name.restype = cp
    L.cft_open.argtypes = [cp, c_int, ctypes.POINTER(vp)]
    L.cft_open.restype = c_int
    L.cft_close.argtypes = [vp]
    L.cft_close.restype = None
    L.cft_get_caps.argtypes = [vp, ctypes.POINTER(Caps)]
    L.cft_get_caps.restype = c_int
    L.cft_supports.argtypes = [vp, c_int, c_int]
    L.cft_supports.restype = c_int
    L.cft_run.argtypes = [vp, c_int, c_int, c_int, vp, vp, vp, vp, sz, u32p, u32p]
    L.cft_run.restype = c_int
    L.cft_run_ex.argtypes = [vp, c_int, c_int, c_int, ctypes.POINTER(ElemArgs)]
    L.cft_run_ex.restype = c_int
    L.cft_div.argtypes = [vp, c_int, c_int, vp, vp, vp, sz, u32p, u32p]
    L.cft_div.restype = c_int
    L.cft_sqrt.argtypes = [vp, c_int, c_int, vp, vp, sz, u32p, u32p]
    L.cft_sqrt.restype = c_int
    L.cft_alloc.argtypes = [vp, sz, ctypes.POINTER(vp)]
    L.cft_alloc.restype = c_int
    L.cft_buffer_data.argtypes = [vp]
    L.cft_buffer_data.restype = vp
    for f in ("cft_buffer_to_device", "cft_buffer_from_device"):
        getattr(L, f).argtypes = [vp]
        getattr(L, f).restype = c_int
    L.cft_buffer_free.argtypes = [vp]
    L.cft_buffer_free.restype = None
    L.cft_program_load.argtypes = [vp, vp, sz, ctypes.POINTER(vp)]
    L.cft_program_load.restype = c_int
    L.cft_program_free.argtypes = [vp]
    L.cft_program_free.restype = None
    L.cft_program_get_info.argtypes = [vp, ctypes.POINTER(ProgramInfo)]
    L.cft_program_get_info.restype = c_int
    L.cft_program_run_ex.argtypes = [vp, ctypes.POINTER(RunArgs)]
    L.cft_program_run_ex.restype = c_int
    L.cft_sha256.argtypes = [vp, sz, vp]
    L.cft_sha256.restype = c_int
    L.cft_save_all_flags.argtypes = [vp]
    L.cft_save_all_flags.restype = u32
    L.cft_lower_flags.argtypes = [vp, u32]
    L.cft_lower_flags.restype = None
    L.cftg_run_device.argtypes = [vp, c_int, c_int, c_int, c_int, vp, vp, vp, vp, sz, u32, vp, vp, vp]
    L.cftg_run_device.restype = c_int
    L.cftg_seq_features.restype = u32
    return L


def lib():
    """The process-wide bound library. Raises if it has not been built."""
    global _LIB
    if _LIB is None:
        path = Path(os.environ.get("CFTG_LIB", LIB_PATH))
        if not path.exists():
            raise OSError(f"libcft_gb300 not found at {path}; build it first "
                          f"(python -c 'import __graft_entry__ as g; g.build()')")
        _LIB = _bind(ctypes.CDLL(str(path)))
    return _LIB


def check(status, where):
    if status != 0:
        L = lib()
        raise CftError(status, where, L.cft_strerror(status).decode(), L.cft_last_error().decode())


def open_device(artifact=None, index=0):
    h = ctypes.c_void_p()
    art = artifact.encode() if isinstance(artifact, str) else artifact
    check(lib().cft_open(art, index, ctypes.byref(h)), "cft_open")
    return h


def close_device(h):
    if h:
        lib().cft_close(h)


def get_caps(h):
    c = Caps()
    c.struct_size = ctypes.sizeof(Caps)
    check(lib().cft_get_caps(h, ctypes.byref(c)), "cft_get_caps")
    return c


def supports(h, op, fmt):
    return bool(lib().cft_supports(h, op, fmt))


def _ptr(x):
    """A C pointer for bytes, bytearray, ctypes buffers, numpy arrays or None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "ctypes"):           # numpy
        return x.ctypes.data
    if isinstance(x, (bytes,)):
        return ctypes.cast(ctypes.c_char_p(x), ctypes.c_void_p).value
    return ctypes.addressof(ctypes.c_char.from_buffer(x))


def run(h, op, fmt, rnd, a, b, c, d, n):
    """cft_run over n elements into d (a writable buffer). Returns flags."""
    fl = ctypes.c_uint32(0)
    check(lib().cft_run(h, op, fmt, rnd, _ptr(a), _ptr(b), _ptr(c), _ptr(d), n,
                        ctypes.byref(fl), None), "cft_run")
    return fl.value


def div(h, fmt, rnd, a, b, d, n):
    fl = ctypes.c_uint32(0)
    check(lib().cft_div(h, fmt, rnd, _ptr(a), _ptr(b), _ptr(d), n, ctypes.byref(fl), None),
          "cft_div")
    return fl.value


def sqrt(h, fmt, rnd, a, d, n):
    fl = ctypes.c_uint32(0)
    check(lib().cft_sqrt(h, fmt, rnd, _ptr(a), _ptr(d), n, ctypes.byref(fl), None), "cft_sqrt")
    return fl.value


def run_ex(h, op, fmt, rnd, a, b, c, d, n, scalar_mask=0, idx=(None, None, None), src=(0, 0, 0)):
    fl = ctypes.c_uint32(0)
    e = ElemArgs()
    e.struct_size = ctypes.sizeof(ElemArgs)
    e.a, e.b, e.c, e.d = _ptr(a), _ptr(b), _ptr(c), _ptr(d)
    e.n = n
    e.scalar_mask = scalar_mask
    e.flags_out = ctypes.pointer(fl)
    e.idx_a, e.idx_b, e.idx_c = (_ptr(i) for i in idx)
    e.idx_a_src, e.idx_b_src, e.idx_c_src = src
    check(lib().cft_run_ex(h, op, fmt, rnd, ctypes.byref(e)), "cft_run_ex")
    return fl.value
