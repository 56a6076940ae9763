"""The oracle against the recorded answers of Reffine's own compile path
(tests/golden/ref_pipeline.json, made by tests/golden/make_ref_pipeline_golden.py from a Reffine
checkout): the four benchmark query shapes on seeded tables, in both vectorize modes.

Against the ``exact`` build of Reffine's emitted code (no contraction) the oracle is
bit-identical; against the ``fma`` build (a*b + c fused, as Reffine's JIT gives on a CPU with
FMA) its FP64 results are within the 1e-12 relative tolerance.  Needs no Reffine checkout.
"""
import json
import os
import sys

import numpy as np
import pytest

from parity import assert_same, assert_table_same
from test_oracle_ref import assert_identical

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
from make_ref_pipeline_golden import cases, decode, table_digest  # noqa: E402


def load():
    with open(os.path.join(GOLDEN, "ref_pipeline.json")) as f:
        js = json.load(f)["cases"]
    arrays = np.load(os.path.join(GOLDEN, "ref_pipeline_hashgroup.npz"))
    out = {}
    for name, entry in js.items():
        res = {}
        for key, r in entry["results"].items():
            if isinstance(r, dict) and "cols" in r:
                res[key] = {"len": r["len"], "null_count": 0, "valid": None,
                            "cols": [arrays[c] for c in r["cols"]]}
            else:
                res[key] = decode(r)
        out[name] = (entry["sha256"], res)
    return out


GOLD = load()
CASES = cases()


@pytest.mark.parametrize("vectorize", [False, True])
@pytest.mark.parametrize("name", sorted(GOLD))
def test_oracle_matches_recorded_reffine_answers(name, vectorize):
    from oracle import loopgen
    digest, res = GOLD[name]
    _, fn, tables, _ = CASES[name]
    assert table_digest(tables) == digest, "the seeded tables changed since the answers were recorded"
    got = loopgen.Query(fn, vectorize)(*tables)
    mode = "vectorize" if vectorize else "scalar"
    assert_identical(got, res[mode + "_exact"])
    if isinstance(got, dict):
        assert_table_same(got, res[mode + "_fma"])
    else:
        assert_same(got, res[mode + "_fma"])
