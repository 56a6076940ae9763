"""rf_plan_run_noalloc: the run entry point for callers that cannot allocate device memory while
they run queries (a fixed device-memory budget, or a loop where cudaMalloc/cudaFree would stall
the device).  Its scratch is a fixed 4 MiB array the library holds in device memory.

Checked through the C-ABI against rf_plan_run, twice in a row (the array keeps the previous
call's contents, so the second call also shows that everything that must start from zero is
cleared).  Runs alone in a fresh process or after the other tests.
"""
import ctypes

import pytest

from parity import assert_same
from reffine_gb300 import _capi, engine, workloads as W

pytestmark = pytest.mark.gpu


def _run(eng, plan, fn, args, noalloc):
    out = plan.new_out()
    f = eng.lib.rf_plan_run_noalloc if noalloc else eng.lib.rf_plan_run
    eng.check(f(plan.h, args, len(fn.inputs), ctypes.byref(out), None))
    return engine.from_c(out)


@pytest.mark.parametrize("which", ["filter_sum", "groupby", "join"])
def test_noalloc_matches_rf_plan_run_twice(eng, which):
    if which == "filter_sum":
        t = W.filter_sum_table(1_000_003, seed=31)
        fn, tabs = W.filter_sum_query(t.get_data_type()), [t]
    elif which == "groupby":
        t = W.groupby_table(2_000_001, seed=32)
        fn, tabs = W.groupby_query(t.get_data_type()), [t]
    else:
        b, p = W.join_tables(50_000, 800_001, seed=33)
        fn, tabs = W.join_query(b.get_data_type(), p.get_data_type()), [b, p]
    dts = [eng.upload(t) for t in tabs]
    plan = eng.compile(fn)
    if which == "join":
        dts[0].build_index()  # probes need the index; building it allocates, so it comes first
    args = plan.args(*dts)
    ref = _run(eng, plan, fn, args, noalloc=False)
    first = _run(eng, plan, fn, args, noalloc=True)
    second = _run(eng, plan, fn, args, noalloc=True)
    assert_same(first, ref)
    assert_same(second, ref)


def test_noalloc_rejects_a_run_beyond_the_fixed_scratch(eng, monkeypatch):
    # the grouped plan keeps 6 x 6 partial sums per unit; with the usable scratch lowered to
    # 4 KiB the run does not fit and is refused with a message, not run out of bounds
    t = W.groupby_table(500_001, seed=34)
    fn = W.groupby_query(t.get_data_type())
    plan = eng.compile(fn)
    args = plan.args(eng.upload(t))
    ref = _run(eng, plan, fn, args, noalloc=False)
    monkeypatch.setenv("RF_NOALLOC_LIMIT", "4096")
    out = plan.new_out()
    st = eng.lib.rf_plan_run_noalloc(plan.h, args, 1, ctypes.byref(out), None)
    assert st == _capi.RF_ERR_INVALID
    assert b"scratch" in eng.lib.rf_last_error(eng.h)
    monkeypatch.delenv("RF_NOALLOC_LIMIT")
    assert_same(_run(eng, plan, fn, args, noalloc=True), ref)
