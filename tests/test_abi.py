"""The C ABI without a GPU: the library loads, exports every symbol the
headers declare (so the reference's ctypes binding can bind it), and
answers the calls that need no device as the reference does."""
import ctypes
import re
from pathlib import Path

import pytest

import cftgb
from cftgb import _lib

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        for m in re.finditer(r"CFT_API\s+[^;(]*?\b((?:cft|cftg)_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_headers_declare_the_hot_path():
    names = declared_symbols()
    for must in ("cft_open", "cft_run", "cft_run_ex", "cft_div", "cft_sqrt", "cft_program_load",
                 "cft_program_run_ex", "cft_alloc", "cft_get_caps", "cftg_run_device"):
        assert must in names


def test_library_exports_every_declared_symbol():
    L = cftgb.lib()
    missing = [n for n in sorted(declared_symbols()) if not hasattr(L, n)]
    assert not missing, missing


def test_reference_binding_symbols_are_exported():
    """Every symbol the reference's cftmpfr._bind touches (its _lib.py:181-372)."""
    binding = ("cft_abi_version cft_strerror cft_last_error cft_format_size cft_format_name "
               "cft_op_name cft_open cft_close cft_get_caps cft_supports cft_run cft_reduce "
               "cft_div cft_sqrt cft_exp cft_expm1 cft_exp2 cft_log cft_log1p cft_log2 cft_log10 "
               "cft_sinpi cft_cospi cft_tanpi cft_asin cft_acos cft_atan cft_asinpi cft_acospi "
               "cft_atanpi cft_sin cft_cos cft_tan cft_sinh cft_cosh cft_tanh cft_asinh cft_acosh "
               "cft_atanh cft_exp2m1 cft_exp10 cft_exp10m1 cft_log2p1 cft_log10p1 cft_rsqrt "
               "cft_pow cft_hypot cft_atan2 cft_atan2pi cft_powr cft_pown cft_compound cft_rootn "
               "cft_augmented_add cft_augmented_sub cft_augmented_mul cft_scaled_prod "
               "cft_scaled_prod_sum cft_scaled_prod_diff cft_formatof_add cft_formatof_sub "
               "cft_formatof_mul cft_formatof_div cft_formatof_sqrt cft_formatof_fma "
               "cft_format_decimal_digits cft_from_decimal_char cft_from_hex_char "
               "cft_to_decimal_char cft_to_hex_char cft_get_payload cft_set_payload "
               "cft_set_payload_signaling cft_min_mag cft_max_mag cft_minnum_mag cft_maxnum_mag "
               "cft_lower_flags cft_raise_flags cft_test_flags cft_save_all_flags "
               "cft_restore_flags cft_test_saved_flags cft_is754version1985 "
               "cft_is754version2008 cft_is754version2019").split()
    L = cftgb.lib()
    assert [s for s in binding if not hasattr(L, s)] == []


def test_names_and_sizes_match_the_reference_tables():
    L = cftgb.lib()
    assert L.cft_abi_version() >> 16 == 0 and L.cft_abi_version() & 0xFFFF == 18
    assert [L.cft_format_name(f).decode() for f in range(4)] == ["fp32", "fp64", "fp128", "fp256"]
    assert L.cft_format_name(4) == b"invalid" and L.cft_format_size(7) == 0
    assert [L.cft_format_size(f) for f in range(4)] == [4, 8, 16, 32]
    for name, op in _lib.OPS.items():
        assert L.cft_op_name(op).decode() == name
    assert L.cft_op_name(15) == b"reserved" and L.cft_op_name(200) == b"reserved"
    assert L.cft_op_name(31) == b"maxall" and L.cft_op_name(24) == b"sum"
    assert L.cft_strerror(0) == b"ok" and L.cft_strerror(99) == b"unknown status"


def test_flag_operations_tolerate_a_null_device():
    L = cftgb.lib()
    L.cft_raise_flags(None, 31)
    assert L.cft_test_flags(None, 31) == 0
    assert L.cft_save_all_flags(None) == 0
    assert L.cft_test_saved_flags(0b10100, 0b00100) == 1
    assert L.cft_test_saved_flags(0b10100, 0b01000) == 0
    assert (L.cft_is754version2019(), L.cft_is754version2008(), L.cft_is754version1985()) == (1, 0, 0)


def test_null_device_is_an_argument_error():
    L = cftgb.lib()
    fl = ctypes.c_uint32(7)
    assert L.cft_run(None, 0, 3, 0, None, None, None, None, 1, ctypes.byref(fl), None) == 1
    assert b"dev is NULL" in L.cft_last_error()
    assert L.cft_div(None, 3, 0, None, None, None, 1, None, None) == 1
    # the sentence belongs to the call that just returned
    assert L.cft_format_size(3) == 32
    assert L.cft_get_caps(None, None) == 1


def test_out_of_scope_calls_refuse_by_name():
    L = cftgb.lib()
    L.cft_exp.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                          ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    assert L.cft_exp(None, 3, 0, None, None, 0, None) == 2
    assert b"cft_exp" in L.cft_last_error()
    L.cft_format_decimal_digits.restype = ctypes.c_size_t
    assert [L.cft_format_decimal_digits(f) for f in range(4)] == [9, 17, 36, 73]


def test_open_without_a_gpu_fails_loudly():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = cftgb.lib()
    h = ctypes.c_void_p()
    st = L.cft_open(None, 0, ctypes.byref(h))
    assert st == 3                                  # CFT_ERR_NO_DEVICE, no CPU fallback
    assert b"no CPU fallback" in L.cft_last_error()
    assert L.cft_open(b"xclbin/tile.xclbin", 0, ctypes.byref(h)) == 3


def test_queue_block_shape_setter_checks_its_argument():
    """the batched form's block shape: multiples of 32 in 32..256 only"""
    L = _lib.lib()
    L.cftg_set_queue_block_threads.argtypes = [ctypes.c_int]
    L.cftg_queue_block_threads.restype = ctypes.c_int
    before = L.cftg_queue_block_threads()
    try:
        for bad in (0, 16, 100, 288, 512, -32):
            assert L.cftg_set_queue_block_threads(bad) == 1, bad
            assert L.cftg_queue_block_threads() == before
        assert L.cftg_set_queue_block_threads(128) == 0
        assert L.cftg_queue_block_threads() == 128
    finally:
        L.cftg_set_queue_block_threads(before)

# every function the reference's public header exports (host/include/cft.h,
# its CFT_API declarations): the link-level interface a C caller binds
REFERENCE_CFT_API = (
    "cft_abi_version cft_acos cft_acosh cft_acospi cft_alloc cft_asin cft_asinh cft_asinpi "
    "cft_atan cft_atan2 cft_atan2pi cft_atanh cft_atanpi cft_augmented_add cft_augmented_mul "
    "cft_augmented_sub cft_buffer_data cft_buffer_free cft_buffer_from_device "
    "cft_buffer_get_info cft_buffer_to_device cft_build_id cft_class cft_close cft_cmp_sig "
    "cft_compound cft_conformance cft_convert cft_cos cft_cosh cft_cospi cft_cvt_from_i32 "
    "cft_cvt_from_i64 cft_cvt_from_u32 cft_cvt_from_u64 cft_cvt_to_i32 cft_cvt_to_i64 "
    "cft_cvt_to_u32 cft_cvt_to_u64 cft_div cft_exp cft_exp10 cft_exp10m1 cft_exp2 cft_exp2m1 "
    "cft_expm1 cft_format_decimal_digits cft_format_name cft_format_size cft_formatof_add "
    "cft_formatof_div cft_formatof_fma cft_formatof_mul cft_formatof_sqrt cft_formatof_sub "
    "cft_from_decimal_char cft_from_hex_char cft_get_caps cft_get_image_id cft_get_payload "
    "cft_hypot cft_is754version1985 cft_is754version2008 cft_is754version2019 cft_last_error "
    "cft_log cft_log10 cft_log10p1 cft_log1p cft_log2 cft_log2p1 cft_logb cft_lower_flags "
    "cft_max_mag cft_maxnum_mag cft_min_mag cft_minnum_mag cft_next_down cft_next_up "
    "cft_op_name cft_open cft_open_ex cft_pow cft_pown cft_powr cft_program_digest "
    "cft_program_free cft_program_get_info cft_program_load cft_program_run "
    "cft_program_run_bank cft_program_run_ex cft_raise_flags cft_reduce cft_reduce_seg "
    "cft_rem cft_restore_flags cft_rint cft_rootn cft_rsqrt cft_run cft_run_ex "
    "cft_save_all_flags cft_scaleb cft_scaled_prod cft_scaled_prod_diff cft_scaled_prod_sum "
    "cft_set_payload cft_set_payload_signaling cft_sha256 cft_sin cft_sinh cft_sinpi "
    "cft_sqrt cft_strerror cft_supports cft_tan cft_tanh cft_tanpi cft_test_flags "
    "cft_test_saved_flags cft_to_decimal_char cft_to_hex_char cft_total_order "
    "cft_total_order_mag").split()


def _public_names(text):
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"CFT_API\s+[^;(]*?\b(cft_[a-z0-9_]+)\s*\(", text))


def test_every_reference_entry_point_is_declared_and_exported():
    """cft.h here (with the refusals it includes) declares, and the library
    exports, every function the reference's cft.h exports."""
    assert len(REFERENCE_CFT_API) == 125
    ours = declared_symbols()
    assert [n for n in REFERENCE_CFT_API if n not in ours] == []
    L = cftgb.lib()
    assert [n for n in REFERENCE_CFT_API if not hasattr(L, n)] == []


def test_reference_header_names_are_the_frozen_list():
    """Where the reference tree is present, its header still exports
    exactly the names above (so the list is not stale)."""
    from refpath import reference_root
    ref = reference_root()
    if ref is None:
        pytest.skip("the reference tree is not present")
    assert _public_names((ref / "host" / "include" / "cft.h").read_text()) == set(REFERENCE_CFT_API)


def test_a_c_caller_of_every_entry_point_compiles_and_links(tmp_path):
    """A C program that names every reference entry point, including cft.h
    only, compiles against include/ and links against libcft_gb300.so."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "caller.c"
    body = ",\n".join(f"    (void (*)(void)){n}" for n in REFERENCE_CFT_API)
    src.write_text('#include "cft.h"\n#include <stdio.h>\n'
                   f"static void (*const table[])(void) = {{\n{body}\n}};\n"
                   "int main(void) { printf(\"%zu %s\\n\", sizeof table / sizeof table[0], "
                   "cft_strerror(CFT_OK)); return 0; }\n")
    so = Path(cftgb.lib()._name)
    exe = tmp_path / "caller"
    p = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", str(ROOT / "include"), str(src),
                        "-o", str(exe), "-L", str(so.parent), "-lcft_gb300",
                        f"-Wl,-rpath,{so.parent}"], capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.split() == ["125", "ok"], (r.stdout, r.stderr)


def test_new_refusals_name_themselves():
    L = cftgb.lib()
    for name in ("cft_rint", "cft_convert", "cft_class", "cft_rem", "cft_cvt_to_u64",
                 "cft_total_order_mag"):
        fn = getattr(L, name)
        fn.restype = ctypes.c_int
        assert fn(None, 0, 0, 0, None, None, None, None, None) == 2, name
        assert name.encode() in L.cft_last_error()
    L.cft_conformance.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p,
                                  ctypes.c_size_t, ctypes.POINTER(ctypes.c_uint64)]
    rep = ctypes.create_string_buffer(b"x" * 16)
    cases = ctypes.c_uint64(99)
    assert L.cft_conformance(None, None, rep, 16, ctypes.byref(cases)) == 2
    assert rep.value == b"" and cases.value == 0
