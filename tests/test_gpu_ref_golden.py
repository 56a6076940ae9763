"""The GPU against the recorded answers of Reffine's own compile path
(tests/golden/ref_pipeline.json: Reffine's LoopGen, CanonPass, ReadWritePass, ScalarPass and
CEmitter, the emitted C++ compiled and run on the CPU), for the four benchmark query shapes on the
seeded tables the answers were recorded on.

Each query is compiled twice: from the Python builder's Func and from the text the binding prints
for the same query built with Reffine's own builder (tests/golden/ref_func_text.tsv).  Integers
(counts, keys) bit-exact; FP64 within 1e-12 relative of both recorded builds of Reffine's code (no
contraction, and a*b + c fused as Reffine's JIT gives on a CPU with FMA).  The grouped query runs
on the key-sorted run-end table (segmented reduce) and on the unsorted flat table (hash group-by),
each compared key-sorted with Reffine's answer on the run-end table.
"""
import numpy as np
import pytest

from parity import assert_same, assert_table_same
from reffine_gb300 import workloads as W
from test_gpu_materialize import plan_run_table
from test_gpu_ref_binding import compile_text
from test_ref_golden import CASES, GOLD

pytestmark = pytest.mark.gpu


def _check(got, res):
    for mode in ("scalar_exact", "scalar_fma"):
        if isinstance(got, dict):
            assert_table_same(got, res[mode])
        else:
            assert_same(got, res[mode])


@pytest.mark.parametrize("source", ["python", "reffine_builder"])
@pytest.mark.parametrize("name", ["filter_sum", "groupby", "join_agg"])
def test_gpu_matches_reffines_answers(eng, name, source):
    _, res = GOLD[name]
    _, fn, tables, _ = CASES[name]
    plan = eng.compile(fn) if source == "python" else compile_text(eng, name, fn)
    dts = [eng.upload(t) for t in tables]
    _check(plan.run(*dts), res)
    plan.free()
    for d in dts:
        d.free()


def _key_sorted(out):
    order = np.argsort(out["cols"][0], kind="stable")
    return {"len": out["len"], "cols": [c[:out["len"]][order] for c in out["cols"]]}


@pytest.mark.parametrize("layout", ["runend_sorted", "flat_unsorted"])
def test_gpu_grouped_sum_matches_reffines_answer(eng, layout):
    _, res = GOLD["hashgroup_ree"]
    _, fn, tables, _ = CASES["hashgroup_ree"]
    if layout == "runend_sorted":
        t = tables[0]
        plan = eng.compile(fn)
    else:
        t = W.hashgroup_table(100_003, 10_000, 1.1, seed=14)  # the same rows before sorting
        plan = eng.compile(W.hashgroup_query(t.get_data_type()))
    out = _key_sorted(plan_run_table(eng, plan, t))
    plan.free()
    assert out["cols"][2].sum() == 100_003
    _check(out, res)
