"""The oracle (oracle/loopgen.py) against Reffine's own compile path (oracle/ref_pipeline.py).

Every query of oracle/ref/ref_queries.h (Reffine's gtest queries and the four benchmark shapes,
built with Reffine's own builder) is lowered by Reffine's LoopGen, CanonPass, ReadWritePass,
ScalarPass and CEmitter, compiled with g++ and run on the same tables as the oracle's restatement
of the same query built with the Python builder.  Both are serial loops in row order, so the
results must be bit-identical, FP64 sums included, in both vectorize modes: this pins the oracle's
loop structure, accumulation order, struct stores and constant printing to Reffine's code.

A second build of Reffine's emitted code lets the C++ compiler fuse a*b + c (as clang's default
contraction does in Reffine's JIT on a CPU with FMA); its FP64 results stay within the 1e-12
relative tolerance of the oracle.

Needs a Reffine checkout: the pipeline library is built from it on first use
(oracle/ref/build_ref.py); without one the tests are skipped.  tests/test_ref_golden.py holds the
recorded answers for where there is none.
"""
import os
import struct
import sys

import numpy as np
import pytest

import refqueries as rq
from parity import assert_same, assert_table_same
from reffine_gb300 import workloads as W
from reffine_gb300.table import Table

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def RP():
    from oracle import ref_pipeline
    if not ref_pipeline.available():
        sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))
        from build_ref import build
        try:
            build(quiet=True)
        except FileNotFoundError as e:
            pytest.skip("no Reffine checkout to build Reffine's pipeline from (%s)" % e)
    return ref_pipeline


def _gen(lo, hi, step=1):
    t = np.arange(lo, hi, step, dtype=np.int64)
    return Table.from_arrays(1, {"t": t, "v": t * 3 + 1})


def _with_nulls(t: Table, col: int, seed: int, frac: float = 0.1) -> Table:
    rng = np.random.default_rng(seed)
    cols = {c.name: c.data for c in t.columns}
    types = {c.name: c.dtype for c in t.columns}
    valid = {t.columns[col].name: rng.random(len(t.columns[col].data)) >= frac}
    return Table.from_arrays(t.dim, cols, name=t.name, valid=valid, types=types)


def _cases():
    st = rq.students_table()
    ga, gb, gc = _gen(0, 40), _gen(5, 30), _gen(10, 50, 2)
    fs = W.filter_sum_table(200_003, seed=21)
    gbt = W.groupby_table(300_007, seed=22)
    b, p = W.join_tables(20_000, 100_003, seed=23)
    hg = W.ree_sorted(W.hashgroup_table(100_003, 10_000, 1.1, seed=24))
    return {
        "vector_op": ("vector_op", rq.vector_op(st), [st]),
        "transform_op": ("transform_op", rq.transform_op(st, 5, 10), [st]),
        "multidim_op": ("multidim_op", rq.multidim_op(rq.runend_table()), [rq.runend_table()]),
        "gen_table_op": ("gen_table_op", rq.gen_table_op(), [3, 17]),
        "gen_table_op_negative": ("gen_table_op", rq.gen_table_op(), [-5, 7]),
        "gen_table_op_one_row": ("gen_table_op", rq.gen_table_op(), [9, 10]),
        "join_op": ("join_op", rq.join_op(ga, gb, gc), [ga, gb, gc]),
        "nested_op": ("nested_op", rq.nested_op(10, 10), []),
        "filter_sum": ("filter_sum", W.filter_sum_query(fs.get_data_type()), [fs]),
        "filter_sum_one_row": ("filter_sum", W.filter_sum_query(fs.get_data_type()), [fs.rows(7, 8)]),
        "filter_sum_empty": ("filter_sum", W.filter_sum_query(fs.get_data_type()), [fs.rows(0, 0)]),
        "filter_sum_nulls": ("filter_sum", W.filter_sum_query(fs.get_data_type()), [_with_nulls(fs, 2, 25)]),
        "groupby": ("groupby", W.groupby_query(gbt.get_data_type()), [gbt]),
        "groupby_iter_nulls": ("groupby", W.groupby_query(gbt.get_data_type()), [_with_nulls(gbt, 0, 26)]),
        "join_agg": ("join_agg", W.join_query(b.get_data_type(), p.get_data_type()), [b, p]),
        "hashgroup_ree": ("hashgroup_ree", W.hashgroup_query(hg.get_data_type()), [hg]),
    }


CASES = _cases()
FP_CASES = ["filter_sum", "groupby", "join_agg", "hashgroup_ree"]


def _bits(x):
    return struct.pack("<d", x) if isinstance(x, float) else x


def assert_identical(got, ref, path="out"):
    """Bit-identical results: floats compared by their bits, tables column by column."""
    if isinstance(ref, dict):
        assert got["len"] == ref["len"], (path, got["len"], ref["len"])
        n = ref["len"]
        for c, (g, r) in enumerate(zip(got["cols"], ref["cols"])):
            assert g.dtype == r.dtype, (path, c, g.dtype, r.dtype)
            assert g[:n].tobytes() == r[:n].tobytes(), "%s column %d differs" % (path, c)
        assert got["null_count"] == ref["null_count"], (path, got["null_count"], ref["null_count"])
        if ref["null_count"]:
            np.testing.assert_array_equal(got["valid"][:n], ref["valid"][:n])
        return
    if isinstance(ref, (tuple, list)):
        assert len(got) == len(ref), path
        for i, (g, r) in enumerate(zip(got, ref)):
            assert_identical(g, r, "%s[%d]" % (path, i))
        return
    assert _bits(got) == _bits(ref), "%s: %r vs %r" % (path, got, ref)


@pytest.mark.parametrize("vectorize", [False, True])
@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_is_bit_identical_to_reffines_pipeline(RP, case, vectorize):
    from oracle import loopgen
    qname, fn, args = CASES[case]
    ref = RP.RefQuery(qname, fn, vectorize)(*args)
    got = loopgen.Query(fn, vectorize)(*args)
    assert_identical(got, ref)


@pytest.mark.parametrize("case", FP_CASES)
def test_oracle_within_tolerance_of_reffines_fma_build(RP, case):
    from oracle import loopgen
    qname, fn, args = CASES[case]
    ref = RP.RefQuery(qname, fn, False, contract=True)(*args)
    got = loopgen.Query(fn, False)(*args)
    if isinstance(ref, dict):
        assert_table_same(got, ref)
    else:
        assert_same(got, ref)


def test_known_answers_through_reffines_pipeline(RP):
    # the gtest suite's own answers (test_reduce.cpp:121, test_multidim.cpp:47-54), here from
    # Reffine's code run on the fixtures regenerated from its data files
    st = rq.students_table()
    assert RP.RefQuery("vector_op", rq.vector_op(st))(st) == 696
    re = rq.runend_table()
    out = RP.RefQuery("multidim_op", rq.multidim_op(re))(re)
    assert out["cols"][0].tolist() == [1, 2, 3, 4]
    assert out["cols"][1].tolist() == [3, 7, 26, 9]
