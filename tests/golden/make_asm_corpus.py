"""Fixtures for the `.cfta` assembler, the character conversions and the
ODE banks, generated with the reference's own Python definitions.

    python tests/golden/make_asm_corpus.py /path/to/reference

The inputs are this file's: seeded synthetic `.cfta` sources (valid
programs over every directive, operand form, rounding suffix and control
code, plus character-level mutations that make most of them refusals),
seeded decimal and hexadecimal-significand sequences (midpoints, long
digit strings, band-edge exponents, NaN payloads, syntax errors) and a
table of ODE steps. The outputs are the reference's:

  * python/cft_golden/asm.py - `assemble` (the image, or a refusal), and
    for each accepted source the SHA-256 of its `disassemble` text and of
    its `info` report; the same two digests for every image under
    tests/golden/programs/ and odes.npz (images the reference's cft-asm
    built from its own programs);
  * python/cft_golden/chars.py - `from_decimal` / `from_hex` under all five
    attributes: the encoding and the flags, or a refusal;
  * programs/gen_odes.py's `bank_values` derivation - the same exact
    operations in the golden model - for each (system, format, step).

Written to tests/golden/asm_corpus.json.gz.
"""
import gzip
import hashlib
import json
import random
import sys
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent / "asm_corpus.json.gz"

OPS = ["fma", "add", "sub", "mul", "abs", "neg", "copysign", "min", "max", "minnum", "maxnum",
       "select", "cmplt", "cmple", "cmpeq", "iand", "ior", "ixor", "iadd", "isub", "ishl",
       "ishr", "icmplt", "recip_seed", "rsqrt_seed", "imul"]
ARITY = {"fma": 3, "select": 3, "add": 2, "sub": 2, "abs": 1, "neg": 1, "recip_seed": 1,
         "rsqrt_seed": 1}
GOOD_LITS = ["2.0", "-0.0", "1e-320", "inf", "-inf", "nan", "snan", "nan(0x5)", "snan(7)",
             "-0x1.8p-3", "1.5e30", "0.1", "-1e-45", "0x1p-149", "3", "0.001", "8", "-7.25e-3",
             "0x3f800000", "0x1P3"]
ODD_LITS = ["0x1p237", "0x7ff0000000000000", "0x3ff0_0000_0000_0000", "1.5e300", "1e400",
            "123456789012345678901234567890", "0x1.fffffffffffffp1023", "+3", "0x 12", "0x+5",
            "0x0x10", "0X1p3", "1.", ".", "e5", "1e", "0x1.8", "nan()", "NaN(0x)", "Infinity",
            "-0x0p0", "-0x10", "0x-0", "4.9e-324", "0x1p-1074", "snan(0)", "nan(0x7fffffff)"]
MUT_CHARS = list(",;.=_+-xpPX0123456789 \tabrkK") + ["\r", "\r\n", "\x0b", "\x00", "é",
                                                      " ", "r31", "r32", "fma", ".kx", "\n"]


def gen_source(rng):
    L = []
    fmt = rng.choice(["fp32", "fp64", "fp128", "fp256"])
    L.append(f".format {fmt}")
    L.append(f".deposits {rng.choice([0, 1, 2, 16, '0x10', 1048576, '1_0'])}")
    ext = rng.random() < 0.3
    if ext:
        L.append(".bank external")
    if rng.random() < 0.3:
        L.append(f".scratch {rng.choice([256, 512, 2048, '0x100', 1])}")
    if rng.random() < 0.3:
        L.append(f".scratch in {rng.randint(0, 20)}")
    if rng.random() < 0.3:
        L.append(f".scratch out {rng.randint(0, 20)}")
    if rng.random() < 0.1:
        L.append(".scratch strict")
    names = []
    odd = rng.random() < 0.15                    # this source may carry an odd literal
    for i in range(rng.choice([0, 1, 3, 20, 300])):
        nm = f"K{i}"
        names.append(nm)
        if ext and rng.random() < 0.7:
            L.append(f".const {nm}")
        else:
            lit = rng.choice(ODD_LITS if odd and rng.random() < 0.05 else GOOD_LITS)
            L.append(f".const {nm} = {lit}")
    regs = [f"r{i}" for i in range(32)] + ["R3", "r07"]
    for i in range(rng.randint(0, 3)):
        a = f"A{i}"
        L.append(f".reg {a} = r{rng.randint(0, 31)}")
        regs.append(a)
    slots = []
    for i in range(rng.randint(0, 2)):
        s = f"S{i}"
        L.append(f".slot {s} = {rng.randint(0, 255)}")
        slots.append(s)
    stack = []                                   # open loops ("r") and quiet regions ("q")
    sloppy = rng.random() < 0.15                 # may break the structural rules

    def opnd():
        if names and rng.random() < 0.35:
            return rng.choice(names)
        return rng.choice(regs)

    for _ in range(rng.randint(1, 40)):
        r = rng.random()
        pad = "  " * len(stack)
        depth = stack.count("r")
        if r < 0.5:
            op = rng.choice(OPS + ["op24", "op15", "op200"])
            suf = ""
            if rng.random() < 0.3:
                suf += "." + rng.choice(["rne", "rtz", "rdn", "rup", "rmm"])
            n = ARITY.get(op, 2)
            if op.startswith("op") or rng.random() < 0.15:
                n = 3
            ops = [opnd() for _ in range(n)]
            if rng.random() < 0.1 and (sloppy or any(o in names for o in ops)):
                suf += ".kx"
            L.append(pad + f"{op}{suf} {rng.choice(regs)}, " + ", ".join(ops))
        elif r < 0.6 and depth < 4:
            L.append(pad + f"repeat {rng.choice([1, 2, 3, 1000, '0x10', 4294967295])}")
            stack.append("r")
        elif r < 0.7 and stack and (stack[-1] == "r" or sloppy):
            stack.pop()
            L.append("  " * len(stack) + "endrep")
        elif r < 0.75:
            top = 600 if sloppy else 255
            L.append(pad + f"{rng.choice(['stl', 'ldl'])} {rng.choice(regs)}, "
                     f"{rng.choice(slots + [str(rng.randint(0, top))])}")
        elif r < 0.8:
            st = rng.choice(["", ", +1", ", -1", ", 2047", ", -2048", ", 0x10", ", -0x10"])
            L.append(pad + f"{rng.choice(['stx', 'ldx'])} {rng.choice(regs)}, {rng.choice(regs)}{st}")
        elif r < 0.85:
            L.append(pad + f"{rng.choice(['augadd', 'augerr'])} {rng.choice(regs)}, "
                     f"{rng.choice(regs)}, {rng.choice(regs)}")
        elif r < 0.9:
            L.append(pad + f"{rng.choice(['deposit', 'setact', 'raise'])} {rng.choice(regs)}")
        elif r < 0.93 and stack.count("q") < 4:
            L.append(pad + "quiet")
            stack.append("q")
        elif r < 0.96 and stack and (stack[-1] == "q" or sloppy):
            stack.pop()
            L.append("  " * len(stack) + "endquiet")
        elif not stack or sloppy:
            L.append(pad + rng.choice(["actall", "halt"]))
    while stack:
        k = stack.pop()
        L.append("  " * len(stack) + ("endrep" if k == "r" else "endquiet"))
    if rng.random() < 0.7:
        L.append("halt  ; done")
    return "\n".join(L) + ("\n" if rng.random() < 0.9 else "")


def mutate(rng, s):
    s = list(s)
    for _ in range(rng.randint(1, 4)):
        k = rng.random()
        i = rng.randint(0, max(0, len(s) - 1))
        if k < 0.33 and s:
            del s[i]
        elif k < 0.66:
            s.insert(i, rng.choice(MUT_CHARS))
        elif s:
            s[i] = rng.choice(MUT_CHARS)
    return "".join(s)


def exact_decimal(m, e):
    """The exact decimal of m * 2^e."""
    if e >= 0:
        return str(m << e)
    d = str(m * 5 ** (-e))
    k = -e
    if len(d) <= k:
        d = "0" * (k - len(d) + 1) + d
    return d[:-k] + "." + d[-k:]


def gen_sequence(rng, F):
    r = rng.random()
    if r < 0.25:
        nd = rng.randint(1, rng.choice([5, 20, 80, 300]))
        ds = "".join(rng.choice("0123456789") for _ in range(nd))
        if rng.random() < 0.5:
            ds = ds[:rng.randint(0, len(ds))] + "." + ds[rng.randint(0, len(ds)):]
        ex = rng.choice(["", f"e{rng.randint(-400, 400)}", f"E+{rng.randint(0, 80000)}",
                         f"e-{rng.randint(0, 80000)}", f"e{F.emax // 3}", f"e{F.emin // 3}",
                         "e99999999999999999999", "e-99999999999999999999"])
        return rng.choice(["", "-", "+"]) + ds + ex
    if r < 0.55:                 # at or beside a rounding midpoint
        p = F.prec
        e = rng.randint(F.emin - p - 2, F.emax - p + 2) if F.width <= 64 else rng.randint(-700, 700)
        m = rng.randint(1 << (p - 1), (1 << p) - 1) if rng.random() < 0.8 else rng.randint(1, 1 << p)
        val = exact_decimal(2 * m + 1, e - 1)
        if rng.random() < 0.3:
            val = val + rng.choice(["1", "0001", "9"]) if "." in val else val + ".0001"
        elif rng.random() < 0.3 and len(val) > 2:
            val = val[:-1]
        return rng.choice(["", "-"]) + val
    if r < 0.7:
        nd = rng.randint(1, 80)
        hs = "".join(rng.choice("0123456789abcdefABCDEF") for _ in range(nd))
        if rng.random() < 0.5:
            hs = hs[:rng.randint(0, len(hs))] + "." + hs[rng.randint(0, len(hs)):]
        return (rng.choice(["", "-"]) + rng.choice(["0x", "0X"]) + hs + rng.choice(["p", "P"])
                + rng.choice(["", "+", "-"]) + str(rng.randint(0, 300000)))
    if r < 0.85:
        w = rng.choice(["inf", "Infinity", "INF", "nan", "NaN", "snan", "sNaN", "nan(0)",
                        "nan(123)", "snan(0)", "snan(0x1f)", "nan(0x)", "nan()", "nan(" + "9" * 80 + ")",
                        "infinit", "nan(x1)", "snan(1)"])
        return rng.choice(["", "-", "+"]) + w
    return rng.choice(["1.5", "0x1p3", "12e5", "inf", ".", "e3", "1e", "1e+", "--1", "+-1", " 1",
                       "1 ", "0x1.8", "1_000", "١", "0x", "0xp1", "1.2.3", "1e5.5"])


ODE_STEPS = ["0.01", "0.005", "0.001", "0.1", "1e-5", "-0.01", "0.0625",
             "0.33333333333333333333333333333333333333333333333333333333333333333333333333333",
             "1e-40"]


def main(ref):
    ref = Path(ref)
    sys.path.insert(0, str(ref / "python"))
    sys.set_int_max_str_digits(0)
    from cft_golden import asm, chars, formats, softfloat as sf

    sha = lambda t: hashlib.sha256(t.encode()).hexdigest()
    rng = random.Random(20261203)
    programs = []
    while len(programs) < 700:
        src = gen_source(rng)
        if rng.random() < 0.4:
            src = mutate(rng, src)
        try:
            img = asm.assemble(src.encode("utf-8"), "src")
        except asm.AsmError:
            img = None
        rec = {"src": src, "image": img.hex() if img is not None else None}
        if img is not None:
            rec["disasm_sha"] = sha(asm.disassemble(img))
            rec["info_sha"] = sha(asm.info(img))
        programs.append(rec)

    images = {}
    golden = Path(__file__).resolve().parent
    for f in sorted((golden / "programs").glob("*.npz")):
        z = np.load(f)
        if "image" in z.files:
            images[f.stem] = z["image"].tobytes()
    z = np.load(golden / "odes.npz")
    for k in ("l63", "l96", "hh"):
        images["odes_" + k] = z[k + "_image"].tobytes()
    image_digests = {}
    for name, img in images.items():
        image_digests[name] = {"disasm_sha": sha(asm.disassemble(img)), "info_sha": sha(asm.info(img))}

    F = [formats.FORMATS[n] for n in ("fp32", "fp64", "fp128", "fp256")]
    seqs = []
    for i in range(1500):
        f = rng.randint(0, 3)
        s = gen_sequence(rng, F[f])
        rec = {"s": s, "fmt": f, "dec": [], "hex": []}
        for key, fn in (("dec", chars.from_decimal), ("hex", chars.from_hex)):
            for rnd in range(5):
                try:
                    bits, fl = fn(F[f], s, rnd)
                    rec[key].append([format(bits, "x"), fl])
                except chars.CharacterSyntaxError:
                    rec[key].append(None)
        seqs.append(rec)

    def dec(fmt, text):
        return chars.from_decimal(fmt, text, sf.RND_RNE)[0]

    banks = []
    for system in ("lorenz63-rk4", "lorenz96-rk4", "henonheiles-lf"):
        for f in range(4):
            fmt = F[f]
            for h in ODE_STEPS:
                hv = dec(fmt, h)
                two = dec(fmt, "2")
                h2, _ = sf.mul(fmt, hv, dec(fmt, "0.5"))
                h6, _ = sf.div(fmt, hv, dec(fmt, "6"))
                if system == "lorenz63-rk4":
                    beta, _ = sf.div(fmt, dec(fmt, "8"), dec(fmt, "3"))
                    vals = [hv, h2, h6, two, dec(fmt, "10"), dec(fmt, "28"), beta]
                elif system == "lorenz96-rk4":
                    vals = [hv, h2, h6, two, dec(fmt, "8")]
                else:
                    mh, _ = sf.neg(fmt, hv)
                    vals = [hv, h2, mh, dec(fmt, "1"), two]
                esz = fmt.width // 8
                if hv & ((1 << (fmt.width - 1)) - 1) == 0:
                    continue                       # the step rounds to zero in this format
                banks.append({"system": system, "fmt": f, "h": h,
                              "bank": b"".join(v.to_bytes(esz, "little") for v in vals).hex()})
        # the derivation reproduces the shipped h = 0.01 banks
        assert next(b for b in banks if b["system"] == system and b["fmt"] == 3 and b["h"] == "0.01")[
            "bank"] == (ref / "programs" / f"{system}-fp256.classic.bank").read_bytes().hex()

    with gzip.open(OUT, "wt") as fh:
        json.dump({"programs": programs, "images": image_digests, "sequences": seqs,
                   "banks": banks}, fh, separators=(",", ":"))
    acc = sum(p["image"] is not None for p in programs)
    print(f"{len(programs)} sources ({acc} accepted), {len(image_digests)} images, "
          f"{len(seqs)} sequences, {len(banks)} banks -> {OUT}")


if __name__ == "__main__":
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    from refpath import require_reference
    main(require_reference(sys.argv))
