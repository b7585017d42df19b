"""The reference's own fixture families, as committed by
tests/golden/make_reference_sets.py, grouped for replay: every group is one
(format, kind, opcode, rounding attribute) with its operands and the
golden model's expected values and per-element flags.

kind 0 = an opcode through cft_run's element loop, 1 = division,
2 = square root (the oracle's and cftg_run_device's numbering)."""
import gzip
import hashlib
import struct
from pathlib import Path

import numpy as np

GOLD = Path(__file__).resolve().parent / "golden"
NAMES = ("fp32", "fp64", "fp128", "fp256")
RNDS = ("rne", "rtz", "rdn", "rup", "rmm")


def vector_groups(fmt):
    """The conformance vector sets (vectors/gen_vectors.py): elementwise
    and same-format formatOf cases, each under all five attributes."""
    z = np.load(GOLD / "vectors" / f"{NAMES[fmt]}.npz")
    kind, op = z["kind"], z["op"]
    for k, o in sorted(set(zip(kind.tolist(), op.tolist()))):
        sel = np.nonzero((kind == k) & (op == o))[0]
        for r, rn in enumerate(RNDS):
            yield dict(fmt=fmt, kind=k, op=o, rnd=r, idx=sel, a=z["a"][sel], b=z["b"][sel],
                       c=z["c"][sel], d=z[f"d_{rn}"][sel], flags=z[f"flags_{rn}"][sel])


def divsqrt_groups(fmt):
    """host/tests/divsqrt_check.py's families, element by element."""
    z = np.load(GOLD / "divsqrt" / f"{NAMES[fmt]}.npz")
    key = np.stack([z["kind"], z["op"], z["rnd"]], 1)
    for k, o, r in sorted(set(map(tuple, key.tolist()))):
        sel = np.nonzero((z["kind"] == k) & (z["op"] == o) & (z["rnd"] == r))[0]
        yield dict(fmt=fmt, kind=k, op=o, rnd=r, idx=sel, a=z["a"][sel], b=z["b"][sel],
                   c=np.zeros_like(z["a"][sel]), d=z["d"][sel], flags=z["flags"][sel])


def edge_corpus(fmt):
    """host/tests/fma_edge_corpus.py's corpus in its own layout: b"CFTGPUA1",
    u32 format code, u32 element bytes, u64 n; then a, b, c, the attribute
    bytes, the expected d and flags. Returns (dict of arrays, expected
    SHA-256 of d || flags)."""
    raw = gzip.open(GOLD / "edge" / f"edge-{NAMES[fmt]}.bin.gz").read()
    assert raw[:8] == b"CFTGPUA1"
    code, esz, n = struct.unpack("<IIQ", raw[8:24])
    assert code == fmt and esz == (4, 8, 16, 32)[fmt]
    W = esz // 4
    off = 24
    out = {}
    for k in ("a", "b", "c"):
        out[k] = np.frombuffer(raw[off:off + n * esz], "<u4").reshape(n, W).copy()
        off += n * esz
    out["rnd"] = np.frombuffer(raw[off:off + n], np.uint8).copy()
    off += n
    out["d"] = np.frombuffer(raw[off:off + n * esz], "<u4").reshape(n, W).copy()
    off += n * esz
    out["flags"] = np.frombuffer(raw[off:off + n], np.uint8).copy()
    expect = (GOLD / "edge" / f"edge-{NAMES[fmt]}.expect").read_text().split()[0]
    assert hashlib.sha256(out["d"].tobytes() + out["flags"].tobytes()).hexdigest() == expect
    return out, expect


def edge_groups(fmt):
    z, _ = edge_corpus(fmt)
    for r in range(5):
        sel = np.nonzero(z["rnd"] == r)[0]
        yield dict(fmt=fmt, kind=0, op=0, rnd=r, idx=sel, a=z["a"][sel], b=z["b"][sel],
                   c=z["c"][sel], d=z["d"][sel], flags=z["flags"][sel])
