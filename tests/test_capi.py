"""The C-ABI library and the lowering pass, without a GPU.

* the library loads and exports every function include/rf_gpu.h declares;
* every benchmark query and the reference's reduce tests lower to a kernel template and the
  generated source compiles for sm_103a (NVRTC, no device needed);
* shapes the GPU backend does not map are rejected with RF_ERR_UNSUPPORTED, never run elsewhere.
"""
import ctypes
import os
import re

import numpy as np
import pytest

import refqueries as rq
from reffine_gb300 import _capi, engine, ir, workloads as W
from reffine_gb300.table import Table
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


def _row_sum_query(tbl_type, value_of):
    # SUM over the rows of the group-by table of value_of(row's columns: flag_a, flag_b, qty,
    # price, disc, tax, day)
    vec = W._sym("lineitem", tbl_type)

    def acc(s, v):
        return W._add(s, value_of([W._get(v, i) for i in range(7)]))

    red = W._red(W._subvec(vec, W._idx(0), W._len(vec, 1)), lambda: W._f64(0), acc)
    red_sym = W._sym("red", red)
    fn = W._func("rowsum", red_sym, [vec])
    fn.tbl[red_sym] = red
    return fn


def test_one_minus_and_one_plus_products_lower_to_fused_forms():
    # x*(1-y) and x*(1+y) over FP64 (either operand order) become rf_mul_1m / rf_mul_1p; other
    # constants, the other subtraction order and plain products stay as written
    tt = W.groupby_table(64).get_data_type()
    cases = [(lambda c: W._mul(c[3], W._sub(W._f64(1), c[4])), "rf_mul_1m("),
             (lambda c: W._mul(W._add(W._f64(1), c[5]), c[3]), "rf_mul_1p("),
             (lambda c: W._mul(c[3], W._sub(W._f64(2), c[4])), None),
             (lambda c: W._mul(c[3], W._sub(c[4], W._f64(1))), None),
             (lambda c: W._mul(c[3], c[4]), None)]
    for value_of, fused in cases:
        src = engine.check(_row_sum_query(tt, value_of))
        got = [f for f in ("rf_mul_1m(", "rf_mul_1p(") if f in src]
        assert got == ([fused] if fused else []), (fused, got)
    src = engine.check(W.groupby_query(tt))
    assert "rf_mul_1p(rf_mul_1m(ld4, ld5), ld6)" in src


def test_grouped_scan_loads_four_rows_before_evaluating_any():
    # the group-by's row function is split into its loads (rf_group_ld: every column the row
    # reads) and the rest (rf_group_v: no column load of its own), and the kernel takes four rows
    # a thread per iteration
    src = engine.check(W.groupby_query(W.groupby_table(64).get_data_type()))
    assert "#define RF_GROUP_SPLIT 1" in src and "#define RF_GROUP_ROWS 4" in src
    ld = src[src.index("RF_DEV void rf_group_ld("):]
    ld = ld[:ld.index("\n}\n")]
    cols = {int(c) for c in re.findall(r"rf_ld<\w+>\(P\.t\[0\]\.col\[(\d+)\]\.data, r\)", ld)}
    assert cols == {1, 2, 3, 4, 5, 6, 7}
    v = src[src.index("RF_DEV int rf_group_v("):]
    v = v[:v.index("\n}\n")]
    assert "rf_ld<" not in v


def test_grouped_scan_takes_fewer_rows_per_step_for_wide_rows():
    # four rows a step up to 12 register words of loaded columns, two up to 32, else one
    from widequery import wide_groupby_query, wide_table
    for ncol, rows in [(4, 4), (12, 2), (14, 2)]:
        src = engine.check(wide_groupby_query(wide_table(64, ncol).get_data_type(), ncol))
        assert "#define RF_GROUP_ROWS %d" % rows in src, ncol


def test_split_grouped_row_function_compiles_for_narrow_column_types():
    # the grouped scan's split row function (RfRowLd members, rf_group_ld, rf_group_v) for int8
    # keys and int16 / float32 / uint8 values: lowered and compiled for sm_103a
    rng = np.random.default_rng(0)
    n = 64
    t = Table.from_arrays(2, {"key": np.arange(n, dtype=np.int64), "k": rng.integers(0, 2, n).astype(np.int8),
                              "s16": rng.integers(-5, 5, n).astype(np.int16),
                              "f32": rng.uniform(0, 1, n).astype(np.float32),
                              "u8": rng.integers(0, 9, n).astype(np.uint8)}, name="mixed")
    vec = ir._sym("m", t.get_data_type())

    def acc(s, v):
        k, s16, f32, u8 = (ir._get(v, i) for i in range(4))
        out = []
        for g in range(2):
            c = ir._eq(k, ir._i8(g))
            sg = ir._get(s, g)
            out.append(ir._new([ir._sel(c, ir._add(ir._get(sg, 0), f32), ir._get(sg, 0)),
                                ir._sel(c, ir._add(ir._get(sg, 1), ir._cast(ir._i64_t, s16)), ir._get(sg, 1)),
                                ir._sel(c, ir._add(ir._get(sg, 2), ir._cast(ir._i64_t, u8)), ir._get(sg, 2))]))
        return ir._new(out)

    init = lambda: ir._new([ir._new([ir._f32(0), ir._i64(0), ir._i64(0)]) for _ in range(2)])
    red = ir._red(ir._subvec(vec, ir._idx(0), ir._len(vec, 1)), init, acc)
    red_sym = ir._sym("red", red)
    fn = ir._func("mixed", red_sym, [vec])
    fn.tbl[red_sym] = red
    src = engine.check(fn)
    assert "#define RF_GROUP_SPLIT 1" in src and "#define RF_GROUP_ROWS 4" in src
    ld = src[src.index("struct RfRowLd {"):]
    ld = ld[:ld.index("};")]
    for ty in ("int8_t", "int16_t", "float", "uint8_t"):
        assert "    %s ld" % ty in ld, ty


def test_probe_kernel_reads_probe_key_first_and_value_after_the_probe():
    # the join's row function loads the probe key with the row's other columns, ahead of the
    # probe, and the summed value only once the row has passed it (and is not split for
    # four-row steps: its rows come from the per-warp queue)
    b, p = W.join_tables(64, 256)
    src = engine.check(W.join_query(b.get_data_type(), p.get_data_type()))
    g = src[src.index("RF_DEV int rf_group("):]
    g = g[:g.index("\n}\n")]
    key = g.index("rf_ld<int64_t>(P.t[1].col[1].data, r)")
    assert key < g.index("rf_locate(")
    assert "rf_locate(P.t[0].ix, (long long)(ld1))" in g
    assert g.index("rf_ld<double>(P.t[1].col[2].data, r)") > g.index("if (g < 0) return -1;")
    assert "RF_GROUP_SPLIT" not in src


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
