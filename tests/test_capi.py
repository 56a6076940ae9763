"""The C-ABI library and the lowering pass, without a GPU.

* the library loads and exports every function include/rf_gpu.h declares;
* every benchmark query and the reference's reduce tests lower to a kernel template and the
  generated source compiles for sm_103a (NVRTC, no device needed);
* shapes the GPU backend does not map are rejected with RF_ERR_UNSUPPORTED, never run elsewhere.
"""
import ctypes
import os
import re

import pytest

import refqueries as rq
from reffine_gb300 import _capi, engine, ir, workloads as W
from reffine_gb300.ir import _add, _f64, _func, _get, _i64, _idx, _len, _red, _subvec, _sym

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:int|int64_t|const char\*)\s+(rf_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_function():
    lib = _capi.load()
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(_capi.SIGNATURES) >= names


def test_status_and_error_paths_without_device():
    lib = _capi.load()
    buf = ctypes.create_string_buffer(4096)
    assert lib.rf_plan_check(b"(func broken", 0, buf, len(buf)) == _capi.RF_ERR_INVALID
    assert b"unbalanced" in buf.value or b"end of text" in buf.value
    assert lib.rf_plan_check(None, 0, buf, len(buf)) == _capi.RF_ERR_INVALID
    assert lib.rf_table_free(None) == _capi.RF_OK


def test_filter_sum_lowers_and_compiles():
    t = W.filter_sum_table(64)
    src = engine.check(W.filter_sum_query(t.get_data_type()))
    assert "RF_SCAN_REDUCE_KERNEL(rf_main" in src


def test_groupby_lowers_to_grouped_template():
    t = W.groupby_table(64)
    src = engine.check(W.groupby_query(t.get_data_type()))
    assert "RF_GROUP_REDUCE_KERNEL(rf_main" in src
    assert "#define RF_G 6" in src and "#define RF_M 6" in src


def test_join_lowers_to_grouped_template_with_probe():
    b, p = W.join_tables(64, 256)
    src = engine.check(W.join_query(b.get_data_type(), p.get_data_type()))
    assert "rf_locate(P.t[0].ix" in src
    assert "#define RF_G 5" in src


def test_only_full_row_grouped_scans_prefetch_the_next_tile():
    # the grouped scan that reads every row's columns asks for the next tile in L2 (every column it
    # reads at the loop's row, whole 16-byte blocks); the join's compacting scan and the one-tile
    # filter+sum scan measured slower with a prefetch and have none
    g = W.groupby_table(64)
    src = engine.check(W.groupby_query(g.get_data_type()))
    assert "#define RF_PREFETCH 1" in src
    body = src[src.index("rf_prefetch_rows"):]
    body = body[:body.index("}")]
    cols = {int(c) for c in re.findall(r"rf_pf\(P\.t\[0\]\.col\[(\d+)\]\.data", body)}
    assert cols == {1, 2, 3, 4, 5, 6, 7}
    b, p = W.join_tables(64, 256)
    assert "RF_PREFETCH" not in engine.check(W.join_query(b.get_data_type(), p.get_data_type()))
    t = W.filter_sum_table(64)
    assert "RF_PREFETCH" not in engine.check(W.filter_sum_query(t.get_data_type()))


@pytest.mark.parametrize("vectorize", [False, True])
def test_reference_reduce_queries_compile(vectorize):
    st2 = rq.students_table(2)
    engine.check(rq.sum_col1_op(st2), vectorize)
    st = rq.students_table()
    src = engine.check(rq.vector_op(st), vectorize)
    assert "rf_range" in src  # the Op iteration space starts at Locate(max(10, col0[0]))


def test_constants_are_hoisted_so_instances_share_a_module():
    t = W.filter_sum_table(64)
    a = engine.check(W.filter_sum_query(t.get_data_type(), day_lo=700))
    b = engine.check(W.filter_sum_query(t.get_data_type(), day_lo=800))
    assert a == b


def test_non_associative_accumulator_is_rejected():
    t = W.filter_sum_table(64)
    vec = _sym("v", t.get_data_type())
    # s' = s * v.price: not a per-field associative update the GPU templates map
    red = _red(_subvec(vec, _idx(0), _len(vec, 1)), lambda: _f64(1), lambda s, v: s * _get(v, 1))
    rs = _sym("r", red)
    fn = _func("bad", rs, [vec])
    fn.tbl[rs] = red
    with pytest.raises(_capi.RfError) as e:
        engine.check(fn)
    assert e.value.status == _capi.RF_ERR_UNSUPPORTED


def test_text_form_round_trips_through_the_parser():
    # every node kind the builder makes is printed, parsed by the C++ reader and lowered
    st = rq.students_table()
    txt = rq.vector_op(st).text()
    assert txt.startswith("(func foo")
    engine.check(rq.vector_op(st))
