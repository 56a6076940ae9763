"""Arrow IPC files loaded straight into device tables (Engine.load_ipc / rf_table_load_ipc): the
queries of the configs give the oracle's results on them, and the columns come back intact."""
import ctypes
import os

import numpy as np
import pytest

from oracle import loopgen
from parity import assert_same, assert_table_same
from reffine_gb300 import engine, workloads as W
from reffine_gb300.table import table_from_ipc

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_filter_sum_on_loaded_table(eng):
    path = os.path.join(GOLDEN, "ipc_filter_sum.arrow")
    host = table_from_ipc(path, 2)
    dt = eng.load_ipc(path, 2)
    fn = W.filter_sum_query(host.get_data_type(), 100, 2000)
    assert_same(eng.compile(fn).run(dt), loopgen.Query(fn)(host))


def test_run_end_table_grouped_sum(eng):
    path = os.path.join(GOLDEN, "ipc_runend.arrow")
    host = table_from_ipc(path, 2)
    dt = eng.load_ipc(path, 2)
    fn = W.hashgroup_query(host.get_data_type())  # over a run-end key column: the segmented reduce
    plan = eng.compile(fn)
    assert plan.kind == 4
    h = ctypes.c_void_p()
    eng.check(eng.lib.rf_plan_run(plan.h, plan.args(dt), 1, ctypes.byref(h), None))
    out = engine.DeviceTable(eng, h, fn.output.type, [])
    try:
        got = out.export()
    finally:
        out.free()
    ref = loopgen.Query(fn)(host)
    assert_table_same(got, ref)
    assert got["len"] == len(np.load(os.path.join(GOLDEN, "ipc_runend.npz"))["run_values"])


def test_columns_round_trip_with_nulls(eng):
    path = os.path.join(GOLDEN, "ipc_types.arrow")
    ref = np.load(os.path.join(GOLDEN, "ipc_types.npz"))
    dt = eng.load_ipc(path, 1)
    got = dt.export()
    names = [n for n in ref.files if not n.startswith("valid_")]
    for i, n in enumerate(names):
        valid = got["valid"][i] if got["valid"][i] is not None else np.ones(len(got["cols"][i]), bool)
        assert np.array_equal(valid, ref["valid_" + n]), n
        assert np.array_equal(got["cols"][i][valid], ref[n][valid]), n


def test_c_entry_point_and_errors(eng):
    h = ctypes.c_void_p()
    path = os.path.join(GOLDEN, "ipc_filter_sum.arrow").encode()
    eng.check(eng.lib.rf_table_load_ipc(eng.h, path, 2, None, ctypes.byref(h)))
    n = ctypes.c_int64()
    eng.check(eng.lib.rf_table_num_rows(h, ctypes.byref(n)))
    assert n.value == 5003
    eng.lib.rf_table_free(h)
    rc = eng.lib.rf_table_load_ipc(eng.h, os.path.join(GOLDEN, "ipc_lz4.arrow").encode(), 1, None, ctypes.byref(h))
    assert rc != 0 and b"compressed" in eng.lib.rf_last_error(eng.h)


@pytest.mark.parametrize("path", ["default", "staged"])
def test_large_file_loads_exactly(eng, tmp_path, monkeypatch, path):
    # 8M rows x 36 B = 288 MB.  default: copied straight out of the populated mapping on a Grace
    # host; staged: several rounds of the 2 x 64 MiB pinned ring, slices of every column buffer
    # split across rounds.  Either way the loaded table gives the uploaded table's exact bits.
    from reffine_gb300.ipc_write import write_ipc
    if path == "staged":
        monkeypatch.setenv("RF_IPC_LOAD", "staged")
    t = W.filter_sum_table(8_000_003, seed=31)
    path = str(tmp_path / "big.arrow")
    write_ipc(path, t)
    dt = eng.load_ipc(path, 2)
    assert dt.nrows == len(t)
    fn = W.filter_sum_query(t.get_data_type())
    plan = eng.compile(fn)
    assert plan.run(dt) == plan.run(eng.upload(t))
    got = dt.export()
    for c, col in enumerate(t.columns):
        assert np.array_equal(got["cols"][c], col.data), col.name
