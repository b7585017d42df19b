"""The oracle against the reference's own fixture families (CPU): the
conformance vector sets of vectors/gen_vectors.py (every opcode's
elementwise cases and the same-format formatOf cases that carry div and
sqrt, all four formats, all five attributes), the div/sqrt families of
host/tests/divsqrt_check.py and the FMA edge corpus of
host/tests/fma_edge_corpus.py - every expected value from the reference's
golden model (tests/golden/make_reference_sets.py). Values and every
element's flags, bit for bit."""
import numpy as np
import pytest

import refsets


def _check(oracle, g):
    d, lf, _ = oracle.run(g["kind"], g["fmt"], g["op"], g["rnd"], g["a"], g["b"], g["c"])
    vbad = np.nonzero((d != g["d"]).any(1))[0]
    fbad = np.nonzero(lf != g["flags"])[0]
    return vbad, fbad


CASES = [(f, m) for f in ("vectors", "divsqrt") for m in range(4)] + [("edge", 2), ("edge", 3)]


@pytest.mark.parametrize("family,fmt", CASES)
def test_oracle_matches_reference_families(oracle, family, fmt):
    groups = {"vectors": refsets.vector_groups, "divsqrt": refsets.divsqrt_groups,
              "edge": refsets.edge_groups}[family](fmt)
    total = 0
    for g in groups:
        vbad, fbad = _check(oracle, g)
        assert vbad.size == 0 and fbad.size == 0, (g["kind"], g["op"], g["rnd"], g["idx"][vbad[:3]],
                                                   g["idx"][fbad[:3]])
        total += len(g["idx"])
    assert total > 1000
