"""Queries built with Reffine's own IR builder, printed by the binding (reffine_gb300::func_text;
tests/golden/ref_func_text.tsv), compiled with rf_plan_compile and run on the GPU: the same
answers as the oracle running the same query, and the reference's gtest goldens (696)."""
import ctypes

import numpy as np
import pytest

import refqueries as rq
from oracle import loopgen
from parity import assert_same, assert_table_same
from reffine_gb300 import engine
from reffine_gb300 import workloads as W
from reffine_gb300.table import Table
from test_gpu_materialize import plan_run_table
from test_ref_binding import fixture

pytestmark = pytest.mark.gpu


def compile_text(eng, name, py_fn, vectorize=False):
    """A plan compiled from the reference-built text; the equivalent Python Func gives the
    argument and result layout."""
    h = ctypes.c_void_p()
    eng.check(eng.lib.rf_plan_compile(eng.h, fixture()[name].encode(), int(vectorize), ctypes.byref(h)))
    return engine.Plan(eng, h, py_fn, vectorize)


@pytest.mark.parametrize("vectorize", [False, True])
def test_reduce_op_golden_from_reference_builder(eng, vectorize):
    st = rq.students_table()
    plan = compile_text(eng, "vector_op", rq.vector_op(st), vectorize)
    assert plan.run(eng.upload(st)) == 696


@pytest.mark.parametrize("name", ["filter_sum", "groupby", "join_agg"])
def test_benchmark_queries_from_reference_builder(eng, name):
    if name == "filter_sum":
        t = W.filter_sum_table(300_007, seed=41)
        fn, tabs = W.filter_sum_query(t.get_data_type()), [t]
    elif name == "groupby":
        t = W.groupby_table(300_007, seed=42)
        fn, tabs = W.groupby_query(t.get_data_type()), [t]
    else:
        b, p = W.join_tables(20_000, 300_007, seed=43)
        fn, tabs = W.join_query(b.get_data_type(), p.get_data_type()), [b, p]
    plan = compile_text(eng, name, fn)
    got = plan.run(*[eng.upload(t) for t in tabs])
    assert_same(got, loopgen.Query(fn)(*tabs))


def test_table_queries_from_reference_builder(eng):
    st = rq.students_table()
    fn = rq.transform_op(st, 5, 10)
    assert_table_same(plan_run_table(eng, compile_text(eng, "transform_op", fn), st), loopgen.Query(fn)(st))
    rt = rq.runend_table()
    out = plan_run_table(eng, compile_text(eng, "multidim_op", rq.multidim_op(rt)), rt)
    assert list(out["cols"][0]) == [1, 2, 3, 4] and list(out["cols"][1]) == [3, 7, 26, 9]
    fn = rq.nested_op(10, 10)
    assert_table_same(plan_run_table(eng, compile_text(eng, "nested_op", fn)), loopgen.Query(fn)())
    flat = W.hashgroup_table(200_003, 20_000, 1.1, seed=44)
    fn = W.hashgroup_query(flat.get_data_type())
    out = plan_run_table(eng, compile_text(eng, "hashgroup", fn), flat)
    order = np.argsort(out["cols"][0], kind="stable")
    out = {"len": out["len"], "cols": [c[order] for c in out["cols"]]}
    ree = W.ree_sorted(flat)
    assert_table_same(out, loopgen.Query(W.hashgroup_query(ree.get_data_type()))(ree))
    # JoinOpTest: tables from the generator query, then the three-way merge
    gen = compile_text(eng, "gen_table_op", rq.gen_table_op())
    ts = []
    for lo, hi in [(0, 10), (5, 15), (7, 12)]:
        o = plan_run_table(eng, gen, lo, hi)
        ts.append(Table.from_arrays(1, {"t": o["cols"][0], "v": o["cols"][1]}))
    fn = rq.join_op(*ts)
    out = plan_run_table(eng, compile_text(eng, "join_op", fn), *ts)
    np.testing.assert_array_equal(out["cols"][0], np.arange(7, 10))
    np.testing.assert_array_equal(out["cols"][1], 3 * np.arange(7, 10))
