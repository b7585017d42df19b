"""Generate the golden fixtures (tests/golden/golden_<fmt>.npz) from the
reference's own Python definition of the arithmetic,
python/cft_golden/softfloat.py (its compute(), div() and sqrt()).

Run where the reference tree is present:

    python tests/golden/make_golden.py [REFERENCE_TREE]     # or CFT_REFERENCE

The fixtures are committed; nothing at test time imports the reference.
Cases: the seeded operand mix of cftgb.workload (specials, cancellation
triples, halfway cases) for fma/add/sub/mul/div/sqrt under all five
rounding attributes, plus every opcode 0..31 and two unassigned ones
under RNE.
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "cft-fp256_gb300"))
from cftgb import workload as wl  # noqa: E402

# op codes for the two contract operations that are not opcodes
DIV, SQRT = 1000, 1001


def main(ref):
    sys.path.insert(0, str(Path(ref) / "python"))
    from cft_golden import formats, softfloat as sf  # noqa: E402
    fmts = [formats.FP32, formats.FP64, formats.FP128, formats.FP256]
    for fi, F in enumerate(fmts):
        W = wl.words(fi)
        rows = []
        cases = []
        for op in (0, 1, 2, 3, DIV, SQRT):
            for rnd in range(5):
                cases.append((op, rnd, 48))
        for op in list(range(0, 32)) + [40, 255]:
            if op in (24, 25, 28, 29, 31):
                continue                      # reductions are not elementwise
            cases.append((op, 0, 16))
        seed = 1000 + fi
        for k, (op, rnd, cnt) in enumerate(cases):
            a, b, c = wl.gen_operands(fi, cnt, seed * 100 + k, special_frac=0.25,
                                      triples_frac=0.1, ties=True)
            for i in range(cnt):
                xa, xb, xc = wl.to_int(a[i]), wl.to_int(b[i]), wl.to_int(c[i])
                if op == DIV:
                    d, fl = sf.div(F, xa, xb, rnd)
                elif op == SQRT:
                    d, fl = sf.sqrt(F, xa, rnd)
                else:
                    d, fl = sf.compute(F, op, xa, xb, xc, rnd)
                rows.append((op, rnd, wl.from_int(xa, W), wl.from_int(xb, W), wl.from_int(xc, W),
                             wl.from_int(d, W), fl))
        out = ROOT / "tests" / "golden" / f"golden_{wl.geometry(fi)['width']}.npz"
        np.savez_compressed(
            out,
            op=np.array([r[0] for r in rows], np.int32),
            rnd=np.array([r[1] for r in rows], np.int32),
            a=np.array([r[2] for r in rows], np.uint32),
            b=np.array([r[3] for r in rows], np.uint32),
            c=np.array([r[4] for r in rows], np.uint32),
            d=np.array([r[5] for r in rows], np.uint32),
            flags=np.array([r[6] for r in rows], np.uint8))
        print(out, len(rows))


if __name__ == "__main__":
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    from refpath import require_reference
    main(require_reference(sys.argv))
