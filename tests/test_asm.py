"""The `.cfta` assembler, the character conversions and the ODE banks,
held to the reference's Python definitions through committed fixtures
(tests/golden/make_asm_corpus.py) - host code, no GPU.

* every generated source: the same image as asm.py, or a refusal where it
  refuses; the same disassembly and header report (by SHA-256);
* every image the reference's cft-asm built from its own programs
  (tests/golden/programs, odes.npz): the disassembly and report digests,
  and assemble(disassemble(image)) == image;
* decimal and hexadecimal-significand sequences under all five attributes:
  encoding and flags as chars.py gives them, refusals where it refuses;
* the ODE banks as gen_odes.py's derivation gives them;
* where the reference tree is present, every `.cfta` it ships against its
  own asm.py and MANIFEST.
"""
import gzip
import hashlib
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from cftgb import asm
from refpath import reference_root

GOLDEN = Path(__file__).resolve().parent / "golden"
CORPUS = json.load(gzip.open(GOLDEN / "asm_corpus.json.gz", "rt"))
# the reference tree, where it is present (this checks against its own
# definitions; the fixtures above carry the same checks everywhere else)
REF = reference_root() or Path("/nonexistent-reference-tree")
REF_TOOL = Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "cft-asm"


def sha(t):
    return hashlib.sha256(t.encode()).hexdigest()


def test_generated_sources_assemble_as_the_reference_does():
    accepted = refused = 0
    for i, rec in enumerate(CORPUS["programs"]):
        data = rec["src"].encode("utf-8")
        if rec["image"] is None:
            with pytest.raises(asm.AsmError):
                asm.assemble(data, "src")
            refused += 1
            continue
        img = asm.assemble(data, "src")
        assert img.hex() == rec["image"], f"source {i}"
        assert sha(asm.disassemble(img)) == rec["disasm_sha"], f"source {i}"
        assert sha(asm.info(img)) == rec["info_sha"], f"source {i}"
        assert asm.assemble(asm.disassemble(img)) == img, f"source {i} round trip"
        accepted += 1
    assert accepted > 200 and refused > 200


def shipped_images():
    out = {}
    for f in sorted((GOLDEN / "programs").glob("*.npz")):
        z = np.load(f)
        if "image" in z.files:
            out[f.stem] = z["image"].tobytes()
    z = np.load(GOLDEN / "odes.npz")
    for k in ("l63", "l96", "hh"):
        out["odes_" + k] = z[k + "_image"].tobytes()
    return out


def test_reference_images_read_back_and_round_trip():
    imgs = shipped_images()
    assert set(imgs) == set(CORPUS["images"])
    for name, img in imgs.items():
        text = asm.disassemble(img)
        assert sha(text) == CORPUS["images"][name]["disasm_sha"], name
        assert sha(asm.info(img)) == CORPUS["images"][name]["info_sha"], name
        assert asm.assemble(text, name) == img, name


def test_info_names_the_image_digest():
    img = shipped_images()["odes_l63"]
    rep = asm.info(img)
    assert f"sha256        {hashlib.sha256(img).hexdigest()}" in rep
    assert "features      REGS32 BANK_PTR SCRATCH SCRATCH_IO" in rep


def test_sequences_convert_as_chars_py():
    n = 0
    for rec in CORPUS["sequences"]:
        for key, fn in (("dec", asm.from_decimal), ("hex", asm.from_hex)):
            for rnd, want in enumerate(rec[key]):
                if want is None:
                    with pytest.raises(asm.AsmError):
                        fn(rec["fmt"], rec["s"], rnd)
                    continue
                bits, fl = fn(rec["fmt"], rec["s"], rnd)
                assert (format(bits, "x"), fl) == (want[0], want[1]), (rec["s"], rec["fmt"], key, rnd)
                n += 1
    assert n > 5000


def test_ode_banks_as_gen_odes_derives_them():
    for rec in CORPUS["banks"]:
        got = asm.ode_bank(rec["system"], rec["fmt"], rec["h"])
        assert got.hex() == rec["bank"], (rec["system"], rec["fmt"], rec["h"])
    z = np.load(GOLDEN / "odes.npz")
    assert asm.ode_bank("lorenz63-rk4", 3, "0.01") == z["l63_bank"].tobytes()
    assert asm.ode_bank("lorenz96-rk4", 2, "0.005") == z["l96_bank"].tobytes()
    assert asm.ode_bank("henonheiles-lf", 3, "0.001") == z["hh_bank"].tobytes()


def test_ode_bank_refusals():
    with pytest.raises(asm.AsmError):
        asm.ode_bank("rossler", 3, "0.01")
    with pytest.raises(asm.AsmError):
        asm.ode_bank("lorenz63-rk4", 0, "1e-300")      # rounds to zero at binary32
    with pytest.raises(asm.AsmError):
        asm.ode_bank("lorenz63-rk4", 3, "0.0.1")


def test_refusals_carry_the_source_line():
    src = ".format fp64\n.deposits 1\n\nfma r1, r2\nhalt\n"
    with pytest.raises(asm.AsmError) as e:
        asm.assemble(src, "k.cfta")
    assert "k.cfta:4:" in str(e.value)
    with pytest.raises(asm.AsmError) as e:
        asm.assemble(".format fp64\n.deposits 1\nhalt\r", "k.cfta")
    assert "carriage return" in str(e.value)


def test_hand_written_example():
    """The text form's worked example (a Newton step for 1/x)."""
    src = """; newton step for 1/x
.format   fp64
.deposits 2
.const    TWO = 2.0
.reg      y = r3
.reg      e = r4

recip_seed y, r0
repeat 4
  neg   e, r0
  fma   e, e, y, TWO
  mul   y, y, e
endrep
deposit y
halt
"""
    img = asm.assemble(src)
    assert img[:4] == b"CFTP"
    text = asm.disassemble(img)
    assert "fma r4, r4, r3, k0" in text and ".const    k0 = 0x4000000000000000" in text
    assert asm.assemble(text) == img


def test_command_line_tool(tmp_path):
    from cftgb import build
    tool = build.TOOL
    if not tool.exists():
        pytest.skip("cftg-asm not built")
    src = tmp_path / "k.cfta"
    src.write_text(".format fp32\n.deposits 1\ndeposit r0\nhalt\n")
    out = tmp_path / "k.cftp"
    assert subprocess.run([str(tool), str(src), "-o", str(out)]).returncode == 0
    assert out.read_bytes() == asm.assemble(src.read_text())
    p = subprocess.run([str(tool), "-d", str(out)], capture_output=True, text=True)
    assert p.returncode == 0 and asm.assemble(p.stdout) == out.read_bytes()
    p = subprocess.run([str(tool), "-i", str(out)], capture_output=True, text=True)
    assert p.returncode == 0 and p.stdout == asm.info(out.read_bytes())
    bank = tmp_path / "b.bank"
    assert subprocess.run([str(tool), "--bank", "henonheiles-lf", "fp256", "0.001", "-o",
                           str(bank)]).returncode == 0
    assert bank.read_bytes() == np.load(GOLDEN / "odes.npz")["hh_bank"].tobytes()
    bad = tmp_path / "bad.cfta"
    bad.write_text(".format fp32\n.deposits 1\nrepeat 0\nendrep\n")
    p = subprocess.run([str(tool), str(bad)], capture_output=True, text=True)
    assert p.returncode == 1 and "repeat 0" in p.stderr


@pytest.mark.skipif(not (REF / "python" / "cft_golden" / "asm.py").exists(),
                    reason="the reference tree is not present")
def test_every_shipped_source_against_the_reference():
    sys.path.insert(0, str(REF / "python"))
    from cft_golden import asm as ref_asm
    manifest = {}
    for line in (REF / "programs" / "MANIFEST").read_text().splitlines():
        parts = line.split()
        if len(parts) == 2:
            manifest[parts[1]] = parts[0]
    files = sorted(set(REF.glob("programs/**/*.cfta")) | set(REF.glob("certificates/**/*.cfta")))
    assert len(files) > 40
    for f in files:
        data = f.read_bytes()
        try:
            want = ref_asm.assemble(data, str(f))
        except ref_asm.AsmError:
            with pytest.raises(asm.AsmError):
                asm.assemble(data, str(f))
            continue
        got = asm.assemble(data, str(f))
        assert got == want, f
        assert asm.disassemble(got) == ref_asm.disassemble(want), f
        assert asm.info(got) == ref_asm.info(want), f
        name = f.stem + ".cftp"
        if f.parent.name == "programs" and name in manifest:
            assert hashlib.sha256(got).hexdigest() == manifest[name], f


@pytest.mark.skipif(not REF_TOOL.exists() or not (REF / "programs").exists(),
                    reason="the reference's cft-asm (oracle/_ref) or its tree is not present")
def test_shipped_sources_against_the_reference_c_tool(tmp_path):
    """The reference's C assembler, built from its sources by oracle/Makefile."""
    for f in sorted(REF.glob("programs/*.cfta")):
        out = tmp_path / "o.cftp"
        p = subprocess.run([str(REF_TOOL), str(f), "-o", str(out)], capture_output=True)
        if p.returncode != 0:
            with pytest.raises(asm.AsmError):
                asm.assemble(f.read_bytes(), str(f))
            continue
        img = asm.assemble(f.read_bytes(), str(f))
        assert img == out.read_bytes(), f
        q = subprocess.run([str(REF_TOOL), "-i", str(out)], capture_output=True, text=True)
        assert q.returncode == 0 and q.stdout == asm.info(img), f


def test_c_abi_argument_checks():
    """The C calls refuse NULL outputs and unreadable images by name, and
    the bank call answers a size query (NULL bank, cap 0)."""
    import ctypes
    L = asm._L()
    vp, sz = ctypes.c_void_p, ctypes.c_size_t
    assert L.cftg_asm_assemble(b".format fp32\n.deposits 1\nhalt\n", 30, b"k", None, None) == 1
    p = vp()
    assert L.cftg_asm_disassemble(b"CFTP", 4, ctypes.byref(p)) == 1
    assert b"header" in L.cft_last_error()
    assert L.cftg_asm_info(b"XXXX" + bytes(28), 32, ctypes.byref(p)) == 1
    assert b"magic" in L.cft_last_error()
    need = sz()
    assert L.cftg_ode_bank(b"lorenz96-rk4", 2, b"0.005", None, 0, ctypes.byref(need)) == 0
    assert need.value == 5 * 16
    small = ctypes.create_string_buffer(16)
    assert L.cftg_ode_bank(b"lorenz96-rk4", 2, b"0.005", small, 16, ctypes.byref(need)) == 1
    assert L.cftg_ode_bank(b"lorenz96-rk4", 7, b"0.005", None, 0, ctypes.byref(need)) == 1


def test_images_the_loader_takes():
    """Every image the assembler writes is one the library's own loader
    takes (cftg_program_check, no device; scratch depth 2^15, the deepest
    a tile publishes)."""
    import ctypes
    L = asm._L()
    L.cftg_program_check.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint32]
    n = 0
    for rec in CORPUS["programs"]:
        if rec["image"] is None:
            continue
        img = bytes.fromhex(rec["image"])
        assert L.cftg_program_check(img, len(img), 1 << 15) == 0, L.cft_last_error()
        n += 1
    assert n > 200
