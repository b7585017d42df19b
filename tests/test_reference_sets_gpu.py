"""The GPU kernels against the reference's own fixture families: the
conformance vector sets of vectors/gen_vectors.py (every opcode's
elementwise cases and the same-format formatOf cases carrying div and sqrt,
all four formats, all five attributes), the div/sqrt families of
host/tests/divsqrt_check.py (exact-tie divisors around 1 and min_normal,
max_subnormal, every special pairing one element a call, the seed opcodes,
the 5,000-element chunk-crossing division) and the FMA edge corpus of
host/tests/fma_edge_corpus.py at binary256 and binary128 (cancellation near
EMIN and EMAX, the normal boundary, overflow by a rounding carry, the
alignment edges). Expected values are the reference's golden model's
(tests/golden/make_reference_sets.py). Through cftg_run_device with a flag
byte per element, and through the reference-facing cft_run / cft_div /
cft_sqrt on host buffers: every value and every flag, bit for bit."""
import hashlib

import numpy as np
import pytest

import cftgb
import refsets
from test_elem_gpu import device_run

pytestmark = pytest.mark.gpu

CASES = [(f, m) for f in ("vectors", "divsqrt") for m in range(4)] + [("edge", 2), ("edge", 3)]
GROUPS = {"vectors": refsets.vector_groups, "divsqrt": refsets.divsqrt_groups,
          "edge": refsets.edge_groups}


def _host_run(h, g):
    d = np.zeros_like(g["a"])
    n = len(g["idx"])
    if g["kind"] == 1:
        fl = cftgb._lib.div(h, g["fmt"], g["rnd"], g["a"], g["b"], d, n)
    elif g["kind"] == 2:
        fl = cftgb._lib.sqrt(h, g["fmt"], g["rnd"], g["a"], d, n)
    else:
        fl = cftgb.run(h, g["op"], g["fmt"], g["rnd"], g["a"], g["b"], g["c"], d, n)
    return d, fl


@pytest.mark.parametrize("family,fmt", CASES)
def test_gpu_matches_reference_families(gpu, family, fmt):
    total = 0
    for g in GROUPS[family](fmt):
        d, lf, acc = device_run(gpu, g["kind"], fmt, g["op"], g["rnd"], g["a"], g["b"], g["c"])
        vbad = np.nonzero((d != g["d"]).any(1))[0]
        fbad = np.nonzero(lf != g["flags"])[0]
        where = (family, fmt, g["kind"], g["op"], g["rnd"])
        assert vbad.size == 0, (where, "values", g["idx"][vbad[:4]])
        assert fbad.size == 0, (where, "flags", g["idx"][fbad[:4]])
        want_acc = int(np.bitwise_or.reduce(g["flags"].astype(np.uint32)))
        assert acc & 0x1F == want_acc, where
        hd, hfl = _host_run(gpu, g)
        assert np.array_equal(hd, g["d"]) and hfl == want_acc, (where, "host path")
        total += len(g["idx"])
    assert total > 1000


@pytest.mark.parametrize("fmt", [3, 2])
def test_edge_corpus_digest(gpu, fmt):
    """The corpus's own acceptance check: the SHA-256 of the computed
    d || flags, in the corpus's order, equals its recorded expectation."""
    z, expect = refsets.edge_corpus(fmt)
    d = np.zeros_like(z["d"])
    fl = np.zeros_like(z["flags"])
    for r in range(5):
        sel = np.nonzero(z["rnd"] == r)[0]
        dd, lf, _ = device_run(gpu, 0, fmt, 0, r, z["a"][sel], z["b"][sel], z["c"][sel])
        d[sel], fl[sel] = dd, lf
    assert hashlib.sha256(d.tobytes() + fl.tobytes()).hexdigest() == expect
