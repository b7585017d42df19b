"""Generate the reference's own fixture families as committed fixtures, for
the GPU tests to replay (tests/test_reference_sets_gpu.py). Run where the
reference tree is present:

    python tests/golden/make_reference_sets.py [REFERENCE_TREE]   # or CFT_REFERENCE

Nothing here restates the reference's case families: each one is produced
by the reference's own code, and every expected value by its own golden
model (python/cft_golden).

  * tests/golden/vectors/<fmt>.npz - the published conformance vector
    sets, made by the reference's vectors/gen_vectors.py for all four
    formats under all five attributes: the elementwise sets (directed and
    random cases of fma/add/sub/mul and 400 cases of every other opcode,
    vectors/gen_vectors.py:849-870 `--directed 4000 --random 6000`) and
    the same-format formatOf sets, which carry div and sqrt. The operand
    pool is the same under every attribute; each attribute has its own
    results.
  * tests/golden/divsqrt/<fmt>.npz - host/tests/divsqrt_check.py's
    families (check_div, check_sqrt, check_lanes, check_seeds at every
    attribute, and check_chunk_crossing's 5,000-element fp32 division):
    its functions are run with a recording device in place of the library,
    so the operands are exactly the ones it sends, and the recording
    device answers with the golden model, as its own comparison expects.
  * tests/golden/edge/edge-<fmt>.bin.gz and .expect - the FMA edge corpus
    of host/tests/fma_edge_corpus.py (its five hard classes at every
    attribute) at binary256 and binary128, COUNT cases each, in the
    corpus's own layout, with its expected-output SHA-256.
"""
import gzip
import json
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
OUT = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT / "cft-fp256_gb300"))
from cftgb import _lib  # noqa: E402  (opcode numbers by name)

FMTS = {"fp32": 0, "fp64": 1, "fp128": 2, "fp256": 3}
WORDS = {0: 1, 1: 2, 2: 4, 3: 8}
RNDS = ("rne", "rtz", "rdn", "rup", "rmm")
EDGE_COUNT = 10000


def words(v, W):
    return [(v >> (32 * i)) & 0xFFFFFFFF for i in range(W)]


def opcode(name):
    if name.startswith("reserved"):
        return int(name[len("reserved"):])
    return _lib.OPS[name]


def vector_sets(ref, tmp):
    out = tmp / "vec"
    subprocess.run([sys.executable, str(ref / "vectors" / "gen_vectors.py"), "--out", str(out),
                    "--rounding", *RNDS, "--transcend", "0", "--augmented", "0",
                    "--minmaxmag", "0", "--jobs", "8"], check=True, capture_output=True)
    (OUT / "vectors").mkdir(exist_ok=True)
    for name, fmt in FMTS.items():
        W = WORDS[fmt]
        res = {}
        ops = None
        for rnd in RNDS:
            suf = "" if rnd == "rne" else f"-{rnd}"
            rows = [json.loads(x) for x in open(out / f"{name}{suf}.jsonl")]
            for j in map(json.loads, open(out / f"{name}-to-{name}-formatof{suf}.jsonl")):
                # formatOf's add and sub take (a, b); cft_run's ADD and SUB
                # steer a*1 + c, so the second operand goes to c
                r = dict(op=j["fn"], a=j["a"], b=j.get("b", "0x0"), c=j.get("c", "0x0"),
                         d=j["d"], flags=j["flags"])
                if j["fn"] in ("add", "sub"):
                    r["b"], r["c"] = "0x0", j["b"]
                rows.append(r)
            key = [(r["op"], r["a"], r.get("b", "0x0"), r.get("c", "0x0")) for r in rows]
            if ops is None:
                ops = key
            assert key == ops, f"{name}: the operand pool differs between attributes"
            res[rnd] = (np.array([words(int(r["d"], 16), W) for r in rows], np.uint32),
                        np.array([int(r["flags"]) for r in rows], np.uint8))
        kind = np.array([1 if o == "div" else 2 if o == "sqrt" else 0 for o, *_ in ops], np.int32)
        op = np.array([0 if o in ("div", "sqrt") else opcode(o) for o, *_ in ops], np.int32)
        arrs = {k: np.array([words(int(x[i], 16), W) for x in ops], np.uint32)
                for k, i in (("a", 1), ("b", 2), ("c", 3))}
        np.savez_compressed(OUT / "vectors" / f"{name}.npz", kind=kind, op=op, **arrs,
                            **{f"d_{r}": res[r][0] for r in RNDS},
                            **{f"flags_{r}": res[r][1] for r in RNDS})
        print(f"vectors/{name}.npz: {len(ops)} cases x 5 attributes")


class Recorder:
    """Stands where divsqrt_check's Device stands: answers each call with
    the golden model and records it element by element."""

    def __init__(self, sf, compute):
        self.sf, self.compute = sf, compute
        self.rows = {}

    def _rec(self, fmt, kind, op, rnd, a, b, d, f):
        self.rows.setdefault(fmt.name, []).append((kind, op, rnd, a, b, d, f))

    def div(self, fmt, rnd, avals, bvals):
        acc, out = 0, []
        for a, b in zip(avals, bvals):
            d, f = self.sf.div(fmt, a, b, rnd)
            self._rec(fmt, 1, 0, rnd, a, b, d, f)
            acc |= f
            out.append(d)
        return out, acc

    def sqrt(self, fmt, rnd, avals):
        acc, out = 0, []
        for a in avals:
            d, f = self.sf.sqrt(fmt, a, rnd)
            self._rec(fmt, 2, 0, rnd, a, 0, d, f)
            acc |= f
            out.append(d)
        return out, acc

    def run1(self, fmt, op, rnd, xa):
        d, f = self.compute(fmt, op, xa, 0, 0, rnd)
        self._rec(fmt, 0, op, rnd, xa, 0, d, f)
        return d, f


def divsqrt_sets(ref):
    sys.path.insert(0, str(ref / "python"))
    sys.path.insert(0, str(ref / "host" / "tests"))
    import divsqrt_check as dc
    rec = Recorder(dc.sf, dc.compute)
    rnds = [dc.RND_BY_NAME[r] for r in RNDS]
    for name in FMTS:
        fmt = dc.FORMATS[name]
        trials = 30 if fmt.width <= 64 else 8
        assert dc.check_div(rec, fmt, rnds, trials)[0] == 0
        assert dc.check_sqrt(rec, fmt, rnds, 2 * trials)[0] == 0
        assert dc.check_lanes(rec, fmt, rnds)[0] == 0
        assert dc.check_seeds(rec, fmt, 2 * trials)[0] == 0
    for rnd in rnds:
        assert dc.check_chunk_crossing(rec, dc.FORMATS["fp32"], rnd)[0] == 0
    (OUT / "divsqrt").mkdir(exist_ok=True)
    for name, fmt in FMTS.items():
        rows = rec.rows[name]
        W = WORDS[fmt]
        np.savez_compressed(
            OUT / "divsqrt" / f"{name}.npz",
            kind=np.array([r[0] for r in rows], np.int32), op=np.array([r[1] for r in rows], np.int32),
            rnd=np.array([r[2] for r in rows], np.int32),
            a=np.array([words(r[3], W) for r in rows], np.uint32),
            b=np.array([words(r[4], W) for r in rows], np.uint32),
            d=np.array([words(r[5], W) for r in rows], np.uint32),
            flags=np.array([r[6] for r in rows], np.uint8))
        print(f"divsqrt/{name}.npz: {len(rows)} cases")


def edge_corpus(ref, tmp):
    (OUT / "edge").mkdir(exist_ok=True)
    for name in ("fp256", "fp128"):
        d = tmp / f"edge-{name}"
        subprocess.run([sys.executable, "-B", str(ref / "host" / "tests" / "fma_edge_corpus.py"),
                        str(d), "--format", name, "--count", str(EDGE_COUNT), "--jobs", "2"],
                       check=True, capture_output=True)
        with open(d / f"edge-{name}.bin", "rb") as src, \
                gzip.GzipFile(OUT / "edge" / f"edge-{name}.bin.gz", "wb", mtime=0) as dst:
            shutil.copyfileobj(src, dst)
        shutil.copy(d / f"edge-{name}.expect", OUT / "edge" / f"edge-{name}.expect")
        print(f"edge/edge-{name}.bin.gz: {EDGE_COUNT} cases")


def main(ref):
    ref = Path(ref)
    with tempfile.TemporaryDirectory() as t:
        tmp = Path(t)
        vector_sets(ref, tmp)
        divsqrt_sets(ref)
        edge_corpus(ref, tmp)


if __name__ == "__main__":
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    from refpath import require_reference
    main(require_reference(sys.argv))
