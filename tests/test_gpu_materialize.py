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


def _nest3(ub_a, ub_b, ub_c):
    """A three-level nest with scalar bounds: Op([a, b, c], 0 <= a < A & 1 <= b <= B & -2 <= c < C,
    [a * 100 + b * 10 + c, b - c])."""
    from reffine_gb300.ir import _mul, _sub
    a, b, c = _sym("a", _i64_t), _sym("b", _i64_t), _sym("c", _i64_t)
    A, B, C = _sym("A", _i64_t), _sym("B", _i64_t), _sym("C", _i64_t)
    pred = (_gte(a, _i64(0)) & _lt(a, A) & _gte(b, _i64(1)) & _lte(b, B) & _gte(c, _i64(-2)) & _lt(c, C))
    op = _op([a, b, c], pred, [_add(_add(_mul(a, _i64(100)), _mul(b, _i64(10))), c), _sub(b, c)])
    op_sym = _sym("op", op)
    fn = _func("nest3", op_sym, [A, B, C])
    fn.tbl[op_sym] = op
    return fn


@pytest.mark.parametrize("vectorize", [False, True])
def test_nested_op_identities(eng, vectorize):
    # NestedOpTest (test_nested.cpp:29-53): every valid row of the 10 x 10 nest in order, with
    # a = idx / 10, b = idx % 10 and a + b; vectorised, each inner loop's end is a null row
    fn = rq.nested_op(10, 10)
    plan = eng.compile(fn, vectorize)
    out = plan_run_table(eng, plan)
    ref = loopgen.Query(fn, vectorize)()
    assert_table_same(out, ref)
    valid = np.ones(out["len"], bool) if out["valid"][0] is None else out["valid"][0]
    idx = 0
    for i in range(out["len"]):
        if valid[i]:
            assert (out["cols"][0][i], out["cols"][1][i], out["cols"][2][i]) == (idx // 10, idx % 10, idx // 10 + idx % 10)
            idx += 1
    assert idx == 100
    assert out["len"] == (110 if vectorize else 100)


@pytest.mark.parametrize("vectorize", [False, True])
@pytest.mark.parametrize("bounds", [(3, 4, 2), (1, 1, -2), (4, 0, 3), (0, 5, 5), (7, 30, 40)])
def test_nested_op_three_levels(eng, vectorize, bounds):
    # scalar bounds, empty levels included: the same rows, nulls and values as the oracle's loop
    fn = _nest3(*bounds)
    plan = eng.compile(fn, vectorize)
    out = plan_run_table(eng, plan, *bounds)
    ref = loopgen.Query(fn, vectorize)(*bounds)
    assert_table_same(out, ref)
    if vectorize and ref["valid"] is not None:
        np.testing.assert_array_equal(out["valid"][0], ref["valid"])


def union_op(ta, tb):
    """An outer merge as the reference's micro benchmark writes it (micro.h:83-102, ojoin_op): Op
    over In(t, left) | In(t, right) with lval - rval, plus each side's value."""
    from reffine_gb300.ir import _sub
    tt = _sym("t", _i64_t)
    left, right = _sym("left", ta.get_data_type()), _sym("right", tb.get_data_type())
    lval, rval = _get(left[tt], 0), _get(right[tt], 0)
    op = _op([tt], _in(tt, left) | _in(tt, right), [_sub(lval, rval), lval, rval])
    os_ = _sym("op", op)
    fn = _func("ojoin", os_, [left, right])
    fn.tbl[os_] = op
    return fn


def _sorted_table(rng, n, hi):
    k = np.sort(rng.integers(0, hi, n)).astype(np.int64)
    return Table.from_arrays(1, {"k": k, "v": rng.integers(-1000, 1000, n).astype(np.int64)})


@pytest.mark.parametrize("vectorize", [False, True])
@pytest.mark.parametrize("sizes", [(1000, 700, 500), (0, 50, 100), (50, 0, 100), (1, 1, 3), (200_003, 150_001, 120_000),
                                   (1_000_000, 1_000_000, 3_000_000)])
def test_union_merge_matches_oracle(eng, vectorize, sizes):
    # duplicates on both sides, keys on one side only, empty sides, sides that end first
    na, nb, hi = sizes
    rng = np.random.default_rng(na + nb)
    ta, tb = _sorted_table(rng, na, hi), _sorted_table(rng, nb, hi)
    fn = union_op(ta, tb)
    plan = eng.compile(fn, vectorize)
    assert plan.kind == 7
    out = plan_run_table(eng, plan, ta, tb)
    ref = loopgen.Query(fn, vectorize)(ta, tb)
    assert_table_same(out, ref)
    # the walk visits every key of either side: max(count in left, count in right) times each
    ka, kb = ta.columns[0].data, tb.columns[0].data
    keys = np.union1d(ka, kb)
    expect = sum(max(int((ka == k).sum()), int((kb == k).sum())) for k in keys) if len(keys) < 5000 else None
    if expect is not None:
        assert out["len"] == expect


def test_union_merge_of_one_table_with_itself(eng):
    # main.cpp:386-400 (shift_op): the same table on both sides pairs every row with itself
    rng = np.random.default_rng(9)
    t = _sorted_table(rng, 10_000, 4_000)
    u = Table.from_arrays(1, {"k": t.columns[0].data.copy(), "v": t.columns[1].data.copy()})
    out = plan_run_table(eng, eng.compile(union_op(t, u)), t, u)
    assert out["len"] == 10_000
    np.testing.assert_array_equal(out["cols"][1], np.zeros(10_000, dtype=np.int64))
