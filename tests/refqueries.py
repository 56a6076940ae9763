"""Reffine's own test queries, restated with the Python builder.

Each builder follows the reference test it names, node for node, so that the oracle and the
GPU backend run the same query the reference's gtest suite runs.
"""
import os

import numpy as np

from reffine_gb300 import ir
from reffine_gb300.ir import (_add, _f64, _func, _get, _gt, _gte, _i64, _in, _lt, _lte, _new, _op,
                              _red, _subvec, _len, _idx, _sym, _i64_t)
from reffine_gb300.table import Table

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STUDENT_COLS = ["id", "hours_studied", "attendance", "sleep_hours", "previous_scores", "exam_score"]


def students_table(dim: int = 1) -> Table:
    """students.arrow loaded with ``dim`` iterator columns (test_utils.cpp:8-24 uses 1)."""
    z = np.load(os.path.join(GOLDEN, "students.npz"))
    return Table.from_arrays(dim, {c: z[c] for c in STUDENT_COLS}, name="students")


def runend_table() -> Table:
    """runend.arrow loaded with dim 2: x run-end encoded, y, d flat."""
    z = np.load(os.path.join(GOLDEN, "runend.npz"))
    return Table.from_arrays(2, {"x": z["x_values"], "y": z["y"], "d": z["d"]},
                             runend={"x": z["x_run_ends"]}, name="runend")


def sum_col1_op(tbl: Table) -> ir.Func:
    """The query of ReduceLoopTest (test_reduce.cpp:9-59: sum of column 1), written as the
    Reduce-over-SubVector it hand-builds as loop IR.  A SubVector reduce needs a table of
    dim >= 2 (Reduce asserts a vector, op.h:95), as TPC-H Q6 loads lineitem (tpch.h:168)."""
    assert tbl.dim >= 2
    vec = _sym("vec", tbl.get_data_type())
    red = _red(_subvec(vec, _idx(0), _len(vec, 1)), lambda: _i64(0), lambda s, v: _add(s, _get(v, 0)))
    red_sym = _sym("red", red)
    fn = _func("foo", red_sym, [vec])
    fn.tbl[red_sym] = red
    return fn


def vector_op(tbl: Table) -> ir.Func:
    """test_reduce.cpp:61-110 (ReduceOpTest, golden 696)."""
    t = _sym("t", _i64_t)
    vec_in = _sym("vec_in", tbl.get_data_type())
    op = _op([t], _in(t, vec_in) & _lte(t, _i64(48)) & _gte(t, _i64(10)),
             [vec_in[t][2],
              _new([vec_in[t][1], vec_in[t][2], vec_in[t][0], vec_in[t][3]]),
              vec_in[t][3]])

    def acc(s, v):
        v0 = _get(_get(v, 2), 0)
        v1 = _get(_get(v, 2), 1)
        v2 = _get(_get(v, 2), 2)
        v3 = _get(_get(v, 2), 3)
        s0 = _get(_get(s, 0), 0)
        s1 = _get(_get(s, 0), 1)
        s2 = _get(_get(s, 1), 0)
        s3 = _get(_get(s, 1), 1)
        return _new([_new([_add(s0, v0), _add(s1, v1)]), _new([_add(s2, v2), _add(s3, v3)])])

    red = _red(op, lambda: _new([_new([_i64(0), _i64(0)]), _new([_i64(0), _i64(0)])]), acc)
    sum_sym = _sym("sum", red)
    res = _get(_get(sum_sym, 1), 0)
    res_sym = _sym("res", res)
    fn = _func("foo", res_sym, [vec_in])
    fn.tbl[sum_sym] = red
    fn.tbl[res_sym] = res
    return fn


def transform_op(tbl: Table, lb: int, n: int) -> ir.Func:
    """test_transform.cpp:9-30 (TransformOpTest)."""
    t = _sym("t", _i64_t)
    vec_in = _sym("vec_in", tbl.get_data_type())
    elem = vec_in[t]
    elem_sym = _sym("elem", elem)
    out = _add(elem_sym[0], _i64(n))
    out_sym = _sym("out", out)
    op = _op([t], _in(t, vec_in) & _gt(t, _i64(lb)), [out_sym])
    op_sym = _sym("op", op)
    fn = _func("foo", op_sym, [vec_in])
    fn.tbl[elem_sym] = elem
    fn.tbl[out_sym] = out
    fn.tbl[op_sym] = op
    return fn


def multidim_op(tbl: Table) -> ir.Func:
    """test_multidim.cpp:9-29 (MultiDimOpTest; golden keys [1,2,3,4], sums [3,7,26,9])."""
    vec = _sym("vec_in", tbl.get_data_type())
    t = _sym("t_sym", _i64_t)
    red = _red(vec[t], lambda: _i64(0), lambda s, v: _add(s, _get(v, 1)))
    red_sym = _sym("sum", red)
    op = _op([t], _in(t, vec), [red_sym])
    op_sym = _sym("op", op)
    fn = _func("red", op_sym, [vec])
    fn.tbl[op_sym] = op
    fn.tbl[red_sym] = red
    return fn


def gen_table_op() -> ir.Func:
    """test_utils.cpp:32-46 (the generator of JoinOpTest's tables): t in [lb, ub)."""
    t = _sym("t", _i64_t)
    lb = _sym("lb", _i64_t)
    ub = _sym("ub", _i64_t)
    op = _op([t], _gte(t, lb) & _lt(t, ub), [t])
    op_sym = _sym("op", op)
    fn = _func("gen_table", op_sym, [lb, ub])
    fn.tbl[op_sym] = op
    return fn


def join_op(a: Table, b: Table, c: Table) -> ir.Func:
    """test_join.cpp:9-37 (JoinOpTest): three-way merge co-iteration."""
    avec = _sym("avec", a.get_data_type())
    bvec = _sym("bvec", b.get_data_type())
    cvec = _sym("cvec", c.get_data_type())
    t = _sym("t", _i64_t)
    aelem, belem, celem = avec[t][0], bvec[t][0], cvec[t][0]
    a_s, b_s, c_s = _sym("a", aelem), _sym("b", belem), _sym("c", celem)
    op = _op([t], _in(t, avec) & _in(t, bvec) & _in(t, cvec), [_add(_add(a_s, b_s), c_s)])
    op_sym = _sym("op", op)
    fn = _func("join", op_sym, [avec, bvec, cvec])
    fn.tbl[a_s] = aelem
    fn.tbl[b_s] = belem
    fn.tbl[c_s] = celem
    fn.tbl[op_sym] = op
    return fn


def nested_op(a_ub: int, b_ub: int) -> ir.Func:
    """test_nested.cpp:9-27 (NestedOpTest)."""
    a = _sym("a", _i64_t)
    b = _sym("b", _i64_t)
    op = _op([a, b], _gte(a, _i64(0)) & _lt(a, _i64(a_ub)) & _gte(b, _i64(0)) & _lt(b, _i64(b_ub)),
             [_add(a, b)])
    op_sym = _sym("op", op)
    fn = _func("foo", op_sym, [])
    fn.tbl[op_sym] = op
    return fn


def table_from_out(res, names, dim=1, name="gen") -> Table:
    """Wraps an Op result (list of columns) as an input table, as the reference feeds the
    generated ArrowTable back into the next query (test_join.cpp:42-52)."""
    return Table.from_arrays(dim, {n: c for n, c in zip(names, res["cols"])}, name=name)
