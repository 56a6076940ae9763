"""Reffine's emitted code for the four benchmark shapes (oracle/ref/generated, run through
oracle/ref_generated.py without a Reffine checkout: the CPU reference arm of bench.py).

Compiled without contraction it gives the recorded answers of Reffine's pipeline
(tests/golden/ref_pipeline.json) and the oracle's, bit for bit, on every one of several threads
running it at once; compiled with the compiler's default contraction (as bench.py times it) its
FP64 results stay within 1e-12 of them.  Where a Reffine checkout is present, the committed code
is checked to be what Reffine's pipeline emits today.
"""
import os
import sys

import pytest

from parity import assert_same, assert_table_same
from test_oracle_ref import assert_identical
from test_ref_golden import CASES, GOLD

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NAMES = ["filter_sum", "groupby", "join_agg", "hashgroup_ree"]


@pytest.mark.parametrize("name", NAMES)
def test_generated_code_gives_reffines_and_the_oracles_bits(name):
    from oracle import loopgen, ref_generated
    _, res = GOLD[name]
    _, fn, tables, _ = CASES[name]
    q = ref_generated.GeneratedQuery(name, fn, contract=False)
    q.prepare(*tables)
    _, outs = q.run(3)
    q.release()
    ref = loopgen.Query(fn)(*tables)
    for out in outs:
        assert_identical(out, res["scalar_exact"])
        assert_identical(out, ref)


@pytest.mark.parametrize("name", NAMES)
def test_generated_code_default_build_within_tolerance(name):
    from oracle import ref_generated
    _, res = GOLD[name]
    _, fn, tables, _ = CASES[name]
    q = ref_generated.GeneratedQuery(name, fn)
    q.prepare(*tables)
    _, (out,) = q.run(1)
    q.release()
    if isinstance(out, dict):
        assert_table_same(out, res["scalar_exact"])
    else:
        assert_same(out, res["scalar_exact"])


@pytest.mark.parametrize("name", NAMES)
def test_committed_code_is_what_reffine_emits(name):
    from oracle import ref_pipeline
    if not ref_pipeline.available():
        sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))
        from build_ref import build
        try:
            build(quiet=True)
        except FileNotFoundError as e:
            pytest.skip("no Reffine checkout (%s)" % e)
    sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))
    from emit_generated import GEN_DIR, generate
    with open(os.path.join(GEN_DIR, name + ".cpp")) as f:
        assert f.read() == generate(name)
