"""rf_plan_run_noalloc: the run entry point for callers that cannot allocate device memory while
they run queries (a fixed device-memory budget, or a loop where cudaMalloc/cudaFree would stall
the device).  Its scratch is a fixed 4 MiB array the library holds in device memory.

Checked through the C-ABI against rf_plan_run, twice in a row (the array keeps the previous
call's contents, so the second call also shows that everything that must start from zero is
cleared); device memory (free memory and the stream-ordered pool's reserved and used bytes) does
not grow across calls; a run that fails on the device leaves the caller's result untouched; and
a fresh process whose first run is a no-allocation run gets the same answer.  Runs alone in a
fresh process or after the other tests.
"""
import ctypes
import gc
import os
import subprocess
import sys

import pytest

from parity import assert_same
from reffine_gb300 import _capi, cudart, engine, workloads as W

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(eng, plan, fn, args, noalloc):
    out = plan.new_out()
    f = eng.lib.rf_plan_run_noalloc if noalloc else eng.lib.rf_plan_run
    eng.check(f(plan.h, args, len(fn.inputs), ctypes.byref(out), None))
    return engine.from_c(out)


def _device_memory(device=0):
    """(free bytes, pool reserved bytes, pool used bytes) of the device's default memory pool."""
    rt = cudart.rt()
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    assert rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    pool = ctypes.c_void_p()
    assert rt.cudaDeviceGetDefaultMemPool(ctypes.byref(pool), ctypes.c_int(device)) == 0
    reserved, used = ctypes.c_uint64(), ctypes.c_uint64()
    assert rt.cudaMemPoolGetAttribute(pool, ctypes.c_int(5), ctypes.byref(reserved)) == 0  # ReservedMemCurrent
    assert rt.cudaMemPoolGetAttribute(pool, ctypes.c_int(7), ctypes.byref(used)) == 0      # UsedMemCurrent
    return free.value, reserved.value, used.value


def _case(which):
    if which == "filter_sum":
        t = W.filter_sum_table(1_000_003, seed=31)
        return W.filter_sum_query(t.get_data_type()), [t]
    if which == "groupby":
        t = W.groupby_table(2_000_001, seed=32)
        return W.groupby_query(t.get_data_type()), [t]
    b, p = W.join_tables(50_000, 800_001, seed=33)
    return W.join_query(b.get_data_type(), p.get_data_type()), [b, p]


@pytest.mark.parametrize("which", ["filter_sum", "groupby", "join"])
def test_noalloc_matches_rf_plan_run_twice(eng, which):
    fn, tabs = _case(which)
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


@pytest.mark.parametrize("which", ["filter_sum", "groupby", "join"])
def test_noalloc_allocates_no_device_memory(eng, which):
    fn, tabs = _case(which)
    dts = [eng.upload(t) for t in tabs]
    plan = eng.compile(fn)
    if which == "join":
        dts[0].build_index()
    args = plan.args(*dts)
    ref = _run(eng, plan, fn, args, noalloc=True)  # warm-up: kernels loaded, driver state settled
    eng.sync()
    gc.collect()  # tables of earlier tests are freed now, not during the measurement
    gc.disable()
    try:
        before = _device_memory()
        outs = [_run(eng, plan, fn, args, noalloc=True) for _ in range(5)]
        eng.sync()
        after = _device_memory()
    finally:
        gc.enable()
    assert after[1] <= before[1], "the memory pool reserved more memory during no-allocation runs"
    assert after[2] <= before[2], "memory pool allocations were held during no-allocation runs"
    assert after[0] >= before[0], "device memory shrank during no-allocation runs"
    for o in outs:
        assert_same(o, ref)


def test_noalloc_leaves_the_result_untouched_on_a_device_error(eng):
    # ReduceOpTest's space starts at Locate(max(lb, col0[0])); a key absent from the iterator
    # column makes the run fail on the device (RF_ERR_DEVICE), with nothing written to host_out
    import refqueries as rq
    st = rq.students_table()
    ids = st.columns[0].data.copy()
    ids[9] = 10_000_000
    st.columns[0].data = ids
    fn = rq.vector_op(st)
    plan = eng.compile(fn)
    dt = eng.upload(st)
    dt.build_index()
    args = plan.args(dt)
    out = plan.new_out()
    sentinel = ctypes.c_int64(-12345)
    ctypes.memmove(ctypes.byref(out), ctypes.byref(sentinel), min(ctypes.sizeof(out), 8))
    st_code = eng.lib.rf_plan_run_noalloc(plan.h, args, len(fn.inputs), ctypes.byref(out), None)
    assert st_code == _capi.RF_ERR_DEVICE
    got = ctypes.c_int64()
    ctypes.memmove(ctypes.byref(got), ctypes.byref(out), min(ctypes.sizeof(out), 8))
    assert got.value == -12345
    # the context and the array stay usable
    st = rq.students_table()
    fn = rq.vector_op(st)
    plan = eng.compile(fn)
    dt = eng.upload(st)
    dt.build_index()
    assert _run(eng, plan, fn, plan.args(dt), noalloc=True) == 696


_FRESH = r"""
import ctypes, json, sys
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/tests")
from reffine_gb300 import engine, workloads as W
from test_zz_no_alloc import _device_memory
eng = engine.Engine(0)
t = W.groupby_table(1_000_001, seed=35)
fn = W.groupby_query(t.get_data_type())
dt = eng.upload(t)
plan = eng.compile(fn)
args = plan.args(dt)
eng.sync()
def run(noalloc):
    out = plan.new_out()
    f = eng.lib.rf_plan_run_noalloc if noalloc else eng.lib.rf_plan_run
    eng.check(f(plan.h, args, 1, ctypes.byref(out), None))
    return engine.from_c(out)
before = _device_memory()
first = run(True)       # the process's first run of any kind
eng.sync()
after = _device_memory()
second = run(True)
ref = run(False)
print(json.dumps({"first": first, "second": second, "ref": ref, "pool_before": before[1:], "pool_after": after[1:]}))
"""


def test_noalloc_first_run_of_a_fresh_process():
    # a process that sets up its context, uploads and compiles, then runs its very first query
    # through the no-allocation entry point: the array was set up by rf_gpu_init, so the run takes
    # nothing from the memory pool and gives rf_plan_run's answer
    import json
    r = subprocess.run([sys.executable, "-c", _FRESH, ROOT], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
    assert d["pool_after"] == d["pool_before"]
    assert_same(d["first"], d["ref"])
    assert_same(d["second"], d["ref"])


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
