"""Generate the sequencer fixtures under tests/golden/programs/ from the
reference itself, run here where its tree is present:

    make -C oracle ref                       # the reference library + cft-asm
    python tests/golden/make_programs.py [REFERENCE_TREE]        # or CFT_REFERENCE
    python tests/golden/make_programs.py REFERENCE_TREE odes

For every program source the reference ships (programs/*.cfta and
certificates/programs/*.cfta) it writes one .npz holding:
  * the image, assembled by the reference's own assembler (cft-asm);
  * seeded input streams, a bank (the program's own .bank where one
    exists, else seeded values) and a scratch-in block;
  * the outputs the reference library (software backend) produced for
    them through cft_program_run_ex: deposits, counts, lane flags, the
    run's flags and STATUS, scratch-out;
and, for a subset, a second run with a lane mask and index tables.

It also writes:
  * loader_cases.npz: valid and mutated images with the status the
    reference's cft_program_load returns for each on a software handle;
  * photograph/: the reference's known-answer case (host/tests/photograph/
    hopf): the camera image, its four banks and the SHA-256 of each pass's
    deposit buffer as an NVIDIA GPU recorded it;
  * lorenz63_cert.npz: the fp256 Lorenz-63 certificate's boundary states
    and segment hashes (certificates/lorenz63-rk4-fp256).
"""
import ctypes
import hashlib
import re
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
OUT = ROOT / "tests" / "golden" / "programs"
sys.path.insert(0, str(ROOT / "cft-fp256_gb300"))
from cftgb import workload as wl  # noqa: E402

ASM = ROOT / "oracle" / "_ref" / "cft-asm"
LIB = ROOT / "oracle" / "_ref" / "libcft_ref.so"


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


def lib():
    L = ctypes.CDLL(str(LIB))
    vp = ctypes.c_void_p
    L.cft_open.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(vp)]
    L.cft_program_load.argtypes = [vp, vp, ctypes.c_size_t, ctypes.POINTER(vp)]
    L.cft_program_run_ex.argtypes = [vp, ctypes.POINTER(RunArgs)]
    L.cft_program_free.argtypes = [vp]
    L.cft_last_error.restype = ctypes.c_char_p
    return L


def header(img):
    w = np.frombuffer(img[:32], "<u4")
    return dict(n_insns=int(w[2]), n_consts=int(w[3]), maxdep=int(w[4]), prec=int(w[5]),
                flags=int(w[6]), sin=int(w[7]) & 0xFFFF if w[6] & 2 else 0,
                sout=int(w[7]) >> 16 if w[6] & 2 else 0)


def ptr(x):
    return None if x is None else x.ctypes.data


def run_ref(L, dev, img, n, a, b, c, bank, sin, mask=None, idx=None, src=None, want_lf=True):
    h = header(img)
    esz = wl.words(h["prec"]) * 4
    prog = ctypes.c_void_p()
    buf = np.frombuffer(img, np.uint8).copy()
    st = L.cft_program_load(dev, buf.ctypes.data, len(img), ctypes.byref(prog))
    if st:
        return None, st
    W = esz // 4
    dep = np.zeros((max(1, n * h["maxdep"]), W), np.uint32)
    cnt = np.zeros(n, np.uint32)
    lf = np.zeros(n, np.uint8)
    sout = np.zeros((max(1, n * h["sout"]), W), np.uint32)
    fl, bus = ctypes.c_uint32(), ctypes.c_uint32()
    A = RunArgs()
    A.struct_size = ctypes.sizeof(RunArgs)
    A.a, A.b, A.c, A.n = ptr(a), ptr(b), ptr(c), n
    if h["flags"] & 1:
        A.bank, A.bank_bytes = ptr(bank), bank.nbytes
    if h["flags"] & 2:
        if h["sin"]:
            A.scratch_in, A.scratch_in_bytes = ptr(sin), sin.nbytes
        if h["sout"]:
            A.scratch_out, A.scratch_out_bytes = ptr(sout), n * h["sout"] * esz
    A.deposits = ptr(dep) if h["maxdep"] else None
    A.counts = ptr(cnt)
    A.flags_out = ctypes.pointer(fl)
    A.bus_out = ctypes.pointer(bus)
    if mask is not None:
        A.lane_mask, A.lane_mask_bytes = ptr(mask), mask.nbytes
    if idx is not None:
        A.idx_a, A.idx_a_src = ptr(idx), src
    if want_lf:
        A.lane_flags, A.lane_flags_bytes = ptr(lf), n
    st = L.cft_program_run_ex(prog, ctypes.byref(A))
    L.cft_program_free(prog)
    if st:
        return None, st
    return dict(deposits=dep[: n * h["maxdep"]], counts=cnt, lane_flags=lf, flags=fl.value,
                status=bus.value, scratch_out=sout[: n * h["sout"]]), 0


def assemble(src):
    with tempfile.TemporaryDirectory() as t:
        out = Path(t) / "p.cftp"
        p = subprocess.run([str(ASM), str(src), "-o", str(out)], capture_output=True, text=True)
        if p.returncode != 0:
            return None
        return out.read_bytes()


def main(ref):
    ref = Path(ref)
    OUT.mkdir(parents=True, exist_ok=True)
    L = lib()
    dev = ctypes.c_void_p()
    assert L.cft_open(None, 0, ctypes.byref(dev)) == 0
    sources = sorted((ref / "programs").glob("*.cfta")) + \
        sorted((ref / "certificates" / "programs").glob("*.cfta"))
    written = 0
    for k, src in enumerate(sources):
        img = assemble(src)
        if img is None:
            print("skip (does not assemble):", src.name)
            continue
        h = header(img)
        fmt, W = h["prec"], wl.words(h["prec"])
        n = 70
        a, b, c = wl.gen_operands(fmt, n, 500 + k, special_frac=0.05)
        if "collatz" in src.name or "lowbias" in src.name or "zoom" in src.name:
            # integer-driven programs: small non-negative integer bit patterns
            a = np.zeros((n, W), np.uint32)
            a[:, 0] = np.arange(1, n + 1)
        bank = None
        if h["flags"] & 1:
            bk = ref / "programs" / (src.stem + ".classic.bank")
            cand = sorted((ref / "programs").glob(src.stem + ".*.bank"))
            if bk.exists():
                bank = np.frombuffer(bk.read_bytes(), np.uint32).reshape(-1, W).copy()
            elif cand:
                bank = np.frombuffer(cand[0].read_bytes(), np.uint32).reshape(-1, W).copy()
            else:
                bank = wl.gen_operands(fmt, max(1, h["n_consts"]), 900 + k, special_frac=0)[0]
                bank = bank[: h["n_consts"]]
            if bank.shape[0] != h["n_consts"]:
                bank = wl.gen_operands(fmt, max(1, h["n_consts"]), 900 + k, special_frac=0)[0][: h["n_consts"]]
        sin = None
        if h["sin"]:
            sin = wl.gen_operands(fmt, n * h["sin"], 700 + k, special_frac=0.02)[0]
        res, st = run_ref(L, dev, img, n, a, b, c, bank, sin)
        if res is None:
            print("skip (reference refuses the run):", src.name, st, L.cft_last_error())
            continue
        case = dict(image=np.frombuffer(img, np.uint8), a=a, b=b, c=c, n=np.int64(n),
                    bank=bank if bank is not None else np.zeros((0, W), np.uint32),
                    scratch_in=sin if sin is not None else np.zeros((0, W), np.uint32))
        for key, v in res.items():
            case["exp_" + key] = np.asarray(v)
        # a masked, gathered variant
        rng = np.random.default_rng(k)
        mask = rng.integers(0, 256, (n + 7) // 8).astype(np.uint8)
        srcn = 40
        idx = rng.integers(0, srcn, n).astype(np.uint32)
        idx[::9] = 0xFFFFFFFF
        pool = a[:srcn].copy()
        res2, st2 = run_ref(L, dev, img, n, pool, b, c, bank, sin, mask=mask, idx=idx, src=srcn)
        if res2 is not None:
            case["mask"] = mask
            case["idx_a"] = idx
            case["idx_a_src"] = np.int64(srcn)
            for key, v in res2.items():
                case["exp2_" + key] = np.asarray(v)
        np.savez_compressed(OUT / (src.stem + ".npz"), **case)
        written += 1
    print("program cases:", written)

    # ---- loader accept/refuse cases ---------------------------------------
    imgs = []
    for src in sources:
        img = assemble(src)
        if img is not None:
            imgs.append(img)
    rng = np.random.default_rng(7)
    rows = []
    for img in imgs:
        rows.append(img)
        for _ in range(24):
            m = bytearray(img)
            kind = rng.integers(0, 6)
            if kind == 0 and len(m) > 33:
                del m[int(rng.integers(0, len(m))):]                     # truncate
            elif kind == 1:
                i = int(rng.integers(0, 32))                            # header byte
                m[i] ^= 1 << int(rng.integers(0, 8))
            elif kind == 2 and len(m) > 32:
                i = int(rng.integers(32, len(m)))                       # any body byte
                m[i] ^= 1 << int(rng.integers(0, 8))
            elif kind == 3 and len(m) >= 40:
                # an instruction's high word (imm) or control bits
                h = header(img)
                esz = wl.words(h["prec"]) * 4
                base = 32 + (0 if h["flags"] & 1 else h["n_consts"] * esz)
                if h["n_insns"]:
                    j = base + 8 * int(rng.integers(0, h["n_insns"])) + int(rng.integers(3, 8))
                    if j < len(m):
                        m[j] = int(rng.integers(0, 256))
            elif kind == 4 and len(m) >= 40:
                h = header(img)
                esz = wl.words(h["prec"]) * 4
                base = 32 + (0 if h["flags"] & 1 else h["n_consts"] * esz)
                if h["n_insns"]:
                    j = base + 8 * int(rng.integers(0, h["n_insns"]))
                    m[j:j + 8] = rng.integers(0, 256, 8).astype(np.uint8).tobytes()
            else:
                h = header(img)                                         # header word
                i = int(rng.integers(2, 8))
                val = int(rng.choice([0, 1, 2, 3, 4, 5, 255, 511, 512, 513, 1 << 20, (1 << 20) + 1,
                                      0xFFFFFFFF, 0x00030003, 0x01000001]))
                m[4 * i:4 * i + 4] = np.uint32(val).tobytes()
            rows.append(bytes(m))
    statuses = []
    for m in rows:
        prog = ctypes.c_void_p()
        buf = np.frombuffer(m, np.uint8).copy() if len(m) else np.zeros(1, np.uint8)
        st = L.cft_program_load(dev, buf.ctypes.data, len(m), ctypes.byref(prog))
        if st == 0:
            L.cft_program_free(prog)
        statuses.append(st)
    lens = np.array([len(m) for m in rows], np.int64)
    blob = np.frombuffer(b"".join(rows), np.uint8)
    np.savez_compressed(OUT.parent / "loader_cases.npz", blob=blob, lens=lens,
                        status=np.array(statuses, np.int32))
    print("loader cases:", len(rows), "accepted:", statuses.count(0))

    # ---- the photograph known answer ------------------------------------
    ph = ref / "host" / "tests" / "photograph" / "hopf"
    pd = OUT.parent / "photograph"
    pd.mkdir(exist_ok=True)
    (pd / "camera.cftp").write_bytes((ph / "camera.cftp").read_bytes())
    for i in range(4):
        (pd / f"camera.p{i:04d}.bank").write_bytes((ph / f"camera.p{i:04d}.bank").read_bytes())
    hashes = [ln.split()[0] for ln in (ph / "deposits.SHA256").read_text().splitlines() if ln.strip()]
    (pd / "deposits.SHA256").write_text("\n".join(hashes) + "\n")

    # ---- the Lorenz-63 fp256 certificate ----------------------------------
    cd = ref / "certificates" / "lorenz63-rk4-fp256"
    cert = (cd / "lorenz63-rk4-fp256.cert").read_text()
    run0 = cert.split("run 1 ")[0]
    segs = re.findall(r"segment (\d+) start ([0-9a-f]{64}) end ([0-9a-f]{64}) flags (\d+) status (\d+)", run0)
    states = [np.frombuffer((cd / "states" / f"run-0-boundary-{i}.bin").read_bytes(), np.uint8)
              for i in range(len(segs) + 1)]
    # an open certificate's state hash: SHA-256 of the tag
    # "cft-certificate 1 state" with its NUL, then the lane-major state
    tag = b"cft-certificate 1 state\0"
    for i, s in enumerate(segs):
        assert hashlib.sha256(tag + states[i].tobytes()).hexdigest() == s[1]
        assert hashlib.sha256(tag + states[i + 1].tobytes()).hexdigest() == s[2]
    img = assemble(ref / "programs" / "lorenz63-rk4-fp256.cfta")
    bank = (ref / "programs" / "lorenz63-rk4-fp256.classic.bank").read_bytes()
    np.savez_compressed(OUT.parent / "lorenz63_cert.npz", image=np.frombuffer(img, np.uint8),
                        bank=np.frombuffer(bank, np.uint8), state0=states[0],
                        ends=np.array([s[2] for s in segs]), flags=np.array([int(s[3]) for s in segs]),
                        status=np.array([int(s[4]) for s in segs]))
    print("certificate segments:", len(segs))


if __name__ == "__main__" and len(sys.argv) <= 2:
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    from refpath import require_reference
    main(require_reference(sys.argv))


def ode_banks(ref):
    """The ODE workloads' images and constant banks, with the step sizes the
    benchmark configurations name: Lorenz-63 RK4 binary256 at h = 0.01 (its
    classic bank), Lorenz-96 RK4 binary128 at h = 0.005 and Henon-Heiles
    leapfrog binary256 at h = 0.001, each bank derived as the reference's
    programs/gen_odes.py:bank_values derives it (h from decimal under RNE,
    h/2 exact, h/6 one rounding) with the golden model's own arithmetic."""
    ref = Path(ref)
    sys.path.insert(0, str(ref / "python"))
    from cft_golden import chars, formats, softfloat as sf

    def dec(fmt, text):
        return chars.from_decimal(fmt, text, sf.RND_RNE)[0]

    def bank(kind, fmt, htext):
        h = dec(fmt, htext)
        two = dec(fmt, "2")
        h2, _ = sf.mul(fmt, h, dec(fmt, "0.5"))
        h6, _ = sf.div(fmt, h, dec(fmt, "6"))
        if kind == "l63":
            beta, _ = sf.div(fmt, dec(fmt, "8"), dec(fmt, "3"))
            vals = [h, h2, h6, two, dec(fmt, "10"), dec(fmt, "28"), beta]
        elif kind == "l96":
            vals = [h, h2, h6, two, dec(fmt, "8")]
        else:
            mh, _ = sf.neg(fmt, h)
            vals = [h, h2, mh, dec(fmt, "1"), two]
        esz = fmt.width // 8
        return np.frombuffer(b"".join(v.to_bytes(esz, "little") for v in vals), np.uint8)

    l63 = assemble(ref / "programs" / "lorenz63-rk4-fp256.cfta")
    l63_bank = bank("l63", formats.FP256, "0.01")
    for kind, name in (("l63", "lorenz63-rk4"), ("l96", "lorenz96-rk4"), ("hh", "henonheiles-lf")):
        # the derivation reproduces the shipped h = 0.01 banks
        assert bank(kind, formats.FP256, "0.01").tobytes() == \
            (ref / "programs" / f"{name}-fp256.classic.bank").read_bytes(), name
    l96 = (ref / "certificates" / "images" / "lorenz96-rk4-fp128.cftp").read_bytes()
    hh = assemble(ref / "programs" / "henonheiles-lf-fp256.cfta")
    np.savez_compressed(OUT.parent / "odes.npz",
                        l63_image=np.frombuffer(l63, np.uint8), l63_bank=l63_bank,
                        l96_image=np.frombuffer(l96, np.uint8),
                        l96_bank=bank("l96", formats.FP128, "0.005"),
                        hh_image=np.frombuffer(hh, np.uint8),
                        hh_bank=bank("hh", formats.FP256, "0.001"))
    print("ode images and banks written")


def certificate(ref, name):
    """Run 0 of certificates/<name>: the image, the classic bank, the lane-major
    boundary states and each segment's end hash, flags and status - every
    boundary re-derived here by the reference library from the one before it,
    so the fixture's bank and image are the ones the certificate ran."""
    ref = Path(ref)
    cd = ref / "certificates" / name
    run0 = (cd / f"{name}.cert").read_text().split("run 1 ")[0]
    segs = re.findall(r"segment (\d+) start ([0-9a-f]{64}) end ([0-9a-f]{64}) flags (\d+) status (\d+)", run0)
    lanes = int(re.search(r"^lanes (\d+)$", run0, re.M).group(1))
    img = (ref / "certificates" / "images" / f"{name}.cftp").read_bytes()
    assert hashlib.sha256(img).hexdigest() == re.search(r"program-image ([0-9a-f]{64})", run0).group(1)
    bank = np.frombuffer((ref / "programs" / f"{name}.classic.bank").read_bytes(), np.uint8).copy()
    tag = b"cft-certificate 1 state\0"
    h = header(img)
    W = wl.words(h["prec"])
    states = [np.frombuffer((cd / "states" / f"run-0-boundary-{i}.bin").read_bytes(), np.uint32)
              .reshape(-1, W) for i in range(len(segs) + 1)]
    L = lib()
    dev = ctypes.c_void_p()
    assert L.cft_open(None, 0, ctypes.byref(dev)) == 0
    for i, s in enumerate(segs):
        assert hashlib.sha256(tag + states[i].tobytes()).hexdigest() == s[1]
        assert hashlib.sha256(tag + states[i + 1].tobytes()).hexdigest() == s[2]
        a = np.zeros((lanes, W), np.uint32)
        out, st = run_ref(L, dev, img, lanes, a, None, None, bank, states[i].copy())
        assert st == 0 and np.array_equal(out["scratch_out"], states[i + 1]), (name, i)
        assert out["flags"] == int(s[3]) and out["status"] == int(s[4]), (name, i)
    np.savez_compressed(OUT.parent / f"{name.split('-')[0]}_cert.npz",
                        image=np.frombuffer(img, np.uint8), bank=bank, state0=states[0].view(np.uint8),
                        ends=np.array([s[2] for s in segs]), flags=np.array([int(s[3]) for s in segs]),
                        status=np.array([int(s[4]) for s in segs]))
    print(name, "segments:", len(segs), "lanes:", lanes)


if __name__ == "__main__" and len(sys.argv) > 2 and sys.argv[2] == "odes":
    ode_banks(sys.argv[1])
    certificate(sys.argv[1], "lorenz96-rk4-fp256")
    certificate(sys.argv[1], "henonheiles-lf-fp256")
