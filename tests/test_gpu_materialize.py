"""GPU parity of Op materialisation (selection-vector compaction; vectorised validity) and of
the integer-pipe binary64 comparisons, against the oracle."""
import numpy as np
import pytest

import refqueries as rq
from oracle import loopgen
from parity import assert_same, assert_table_same
from reffine_gb300 import ir, workloads as W
from reffine_gb300.ir import (_add, _eq, _func, _get, _gt, _gte, _i64, _idx, _in, _len, _lt, _lte, _new, _not,
                              _op, _red, _sel, _subvec, _sym, _i64_t)
from reffine_gb300.table import Table

pytestmark = pytest.mark.gpu

SPECIAL = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, -np.nan, 5e-324, -5e-324, 2.2250738585072014e-308,
                    1.7976931348623157e308, -1.7976931348623157e308, 0.05, 0.07, 24.0, 1e-300, -1e-300])


def compare_counts_query(t):
    vec = _sym("v", t.get_data_type())

    def acc(s, v):
        a, b = _get(v, 0), _get(v, 1)
        conds = [_lt(a, b), _lte(a, b), _gt(a, b), _gte(a, b), _eq(a, b), _not(_eq(a, b))]
        return _new([_sel(c, _add(_get(s, i), _i64(1)), _get(s, i)) for i, c in enumerate(conds)])

    red = _red(_subvec(vec, _idx(0), _len(vec, 1)), lambda: _new([_i64(0)] * 6), acc)
    rs = _sym("r", red)
    fn = _func("cmp", rs, [vec])
    fn.tbl[rs] = red
    return fn


def test_binary64_comparisons_match_ieee(eng):
    rng = np.random.default_rng(3)
    a = np.concatenate([np.repeat(SPECIAL, len(SPECIAL)), rng.standard_normal(100_000) * 10.0 ** rng.integers(-300, 300, 100_000)])
    b = np.concatenate([np.tile(SPECIAL, len(SPECIAL)), rng.standard_normal(100_000) * 10.0 ** rng.integers(-300, 300, 100_000)])
    b[-50_000:] = a[-50_000:]  # equal pairs
    t = Table.from_arrays(2, {"k": np.arange(len(a), dtype=np.int64), "a": a, "b": b})
    fn = compare_counts_query(t)
    got = eng.compile(fn).run(eng.upload(t))
    with np.errstate(invalid="ignore"):
        ref = (int((a < b).sum()), int((a <= b).sum()), int((a > b).sum()), int((a >= b).sum()), int((a == b).sum()),
               int((a != b).sum()))
    assert got == ref
    assert_same(got, loopgen.Query(fn)(t))


@pytest.mark.parametrize("vectorize", [False, True])
def test_transform_op_parity(eng, vectorize):
    st = rq.students_table()
    fn = rq.transform_op(st, 5, 10)
    plan = eng.compile(fn, vectorize)
    assert plan.kind == 3
    out = plan_run_table(eng, plan, st)
    ref = loopgen.Query(fn, vectorize)(st)
    assert_table_same(out, ref)
    assert out["len"] == len(st) - 5


@pytest.mark.parametrize("vectorize", [False, True])
def test_gen_table_ranges(eng, vectorize):
    fn = rq.gen_table_op()
    plan = eng.compile(fn, vectorize)
    for lo, hi in [(0, 10), (5, 15), (7, 12), (3, 3), (10, 4), (-7, 100_003)]:
        out = plan_run_table(eng, plan, lo, hi)
        ref = loopgen.Query(fn, vectorize)(lo, hi)
        assert_table_same(out, ref)


@pytest.mark.parametrize("vectorize", [False, True])
def test_filtered_op_with_nulls(eng, vectorize):
    # an Op over a vector with a filter symbol and a null iterator value: vectorised output keeps
    # every visited row and marks filtered ones null (finalize_vector, vinstr.h:113-135)
    n = 200_001
    rng = np.random.default_rng(5)
    mask = rng.random(n) > 0.01
    mask[0] = True  # the space starts at Locate(col0[0]) (VecSpace lower bound), which must exist
    t = Table.from_arrays(1, {"k": np.arange(n, dtype=np.int64), "x": rng.integers(0, 100, n),
                              "y": rng.standard_normal(n)}, valid={"k": mask})
    tt = _sym("t", _i64_t)
    vec = _sym("vec", t.get_data_type())
    e = vec[tt]
    f = _lt(_get(e, 0), _i64(37))
    fs = _sym("f", f)
    op = _op([tt], _in(tt, vec) & fs, [_add(_get(e, 0), _i64(1)), _get(e, 1)])
    os_ = _sym("op", op)
    fn = _func("flt", os_, [vec])
    fn.tbl[fs] = f
    fn.tbl[os_] = op
    out = plan_run_table(eng, eng.compile(fn, vectorize), t)
    ref = loopgen.Query(fn, vectorize)(t)
    if not vectorize:
        assert_table_same(out, ref)
    else:
        assert out["len"] == ref["len"]
        v = ref["valid"]
        assert v is not None and out["valid"][0] is not None
        np.testing.assert_array_equal(out["valid"][0], v)
        for g, r in zip(out["cols"], ref["cols"]):
            np.testing.assert_array_equal(g[v], r[v])


def plan_run_table(eng, plan, *inputs):
    import ctypes
    from reffine_gb300 import engine as E
    args = []
    for s, v in zip(plan.fn.inputs, inputs):
        args.append(eng.upload(v) if s.type.is_vector() else v)
    pa = plan.args(*args)
    h = ctypes.c_void_p()
    eng.check(eng.lib.rf_plan_run(plan.h, pa, len(args), ctypes.byref(h), None))
    dt = E.DeviceTable(eng, h, plan.fn.output.type, [])
    try:
        return dt.export()
    finally:
        dt.free()


def test_join_op_merge_coiteration(eng):
    # JoinOpTest (test_join.cpp:39-87): three tables generated by the gen_table query itself
    g = eng.compile(rq.gen_table_op())
    bounds = [(0, 10), (5, 15), (7, 12)]
    ts = []
    for lo, hi in bounds:
        out = plan_run_table(eng, g, lo, hi)
        ts.append(Table.from_arrays(1, {"t": out["cols"][0], "v": out["cols"][1]}))
    fn = rq.join_op(*ts)
    plan = eng.compile(fn)
    assert plan.kind == 6
    out = plan_run_table(eng, plan, *ts)
    lb, ub = max(b[0] for b in bounds), min(b[1] for b in bounds)
    assert out["len"] == ub - lb
    np.testing.assert_array_equal(out["cols"][0], np.arange(lb, ub))
    np.testing.assert_array_equal(out["cols"][1], 3 * np.arange(lb, ub))
    assert_table_same(out, loopgen.Query(fn)(*ts))


def test_merge_join_sorted_with_gaps_and_duplicates(eng):
    rng = np.random.default_rng(12)
    a = np.sort(rng.integers(0, 50_000, 100_000))
    b = np.sort(rng.integers(0, 50_000, 60_000))
    a[0] = b[0] = 0
    ta = Table.from_arrays(1, {"t": a.astype(np.int64), "v": rng.integers(0, 1000, len(a))})
    tb = Table.from_arrays(1, {"t": b.astype(np.int64), "v": rng.integers(0, 1000, len(b))})
    tt = _sym("t", _i64_t)
    av, bv = _sym("av", ta.get_data_type()), _sym("bv", tb.get_data_type())
    x, y = av[tt][0], bv[tt][0]
    op = _op([tt], _in(tt, av) & _in(tt, bv), [_add(x, y)])
    os_ = _sym("op", op)
    fn = _func("mj", os_, [av, bv])
    fn.tbl[os_] = op
    out = plan_run_table(eng, eng.compile(fn), ta, tb)
    assert_table_same(out, loopgen.Query(fn)(ta, tb))
