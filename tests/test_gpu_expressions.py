"""GPU parity of the predicate/projection expression set (the math operators of the functional
IR, expr.h:141-281, as the reference's C emitter prints them, cemitter.cpp:112-160) against the
oracle, row by row.

Each case is an Op over a table of every primitive width (signed and unsigned integers, f32,
f64) whose output columns are expressions of the row; every output row is compared: integer
columns bit-exact, floating-point columns bit-exact where IEEE fixes the result (+ - * /, sqrt,
ceil, floor, abs, min/max, neg, casts) and within the relative tolerance where the library is
free to differ by an ulp (pow: CUDA documents 2 ulp for double pow).  Operands avoid the C++
undefined cases (integer division by zero, signed overflow, out-of-range float-to-int casts).
"""
import numpy as np
import pytest

from oracle import loopgen
from parity import RTOL_F64
from reffine_gb300 import ir
from reffine_gb300.ir import (_abs, _add, _and, _cast, _ceil, _div, _eq, _floor, _func, _get, _gt, _gte, _i64, _in,
                              _lt, _lte, _max, _min, _mod, _mul, _neg, _not, _op, _or, _pow, _sel, _sqrt, _sub, _sym,
                              _i64_t)
from reffine_gb300.table import Table
from test_gpu_materialize import plan_run_table

pytestmark = pytest.mark.gpu

N = 50_001
INT_TYPES = ["i8", "i16", "i32", "i64", "u8", "u16", "u32", "u64"]
FLOAT_TYPES = ["f32", "f64"]
NP = {"i8": np.int8, "i16": np.int16, "i32": np.int32, "i64": np.int64, "u8": np.uint8, "u16": np.uint16,
      "u32": np.uint32, "u64": np.uint64, "f32": np.float32, "f64": np.float64}


def _table(seed=7):
    """Columns a_<ty> and b_<ty> per type.  Integers stay small enough that no product, sum or
    difference of two of them overflows a signed type after C++ promotion; every b is nonzero."""
    rng = np.random.default_rng(seed)
    cols = {"k": np.arange(N, dtype=np.int64)}
    for ty in INT_TYPES:
        info = np.iinfo(NP[ty])
        lo = max(int(info.min), -30_000)
        hi = min(int(info.max), 30_000)
        a = rng.integers(lo, hi + 1, N).astype(NP[ty])
        b = rng.integers(lo, hi + 1, N).astype(NP[ty])
        b[b == 0] = 3
        cols["a_" + ty], cols["b_" + ty] = a, b
    for ty in FLOAT_TYPES:
        a = (rng.standard_normal(N) * 10.0 ** rng.integers(-3, 4, N)).astype(NP[ty])
        b = (rng.standard_normal(N) * 10.0 ** rng.integers(-3, 4, N)).astype(NP[ty])
        a[:8] = np.array([0.0, -0.0, 1.5, -1.5, 2.5, -2.5, 1e-3, 7.0], dtype=NP[ty])
        b[b == 0] = 0.5
        cols["a_" + ty], cols["b_" + ty] = a, b
    return Table.from_arrays(1, cols, name="types")


TABLE = None


def table():
    global TABLE
    if TABLE is None:
        TABLE = _table()
    return TABLE


def _col_index(t, name):
    return [c.name for c in t.columns].index(name)


def _op_of(t, make_outputs):
    """Op([k], In(k, vec), outputs(elem)), elem = the row's columns by name."""
    k = _sym("k", _i64_t)
    vec = _sym("vec", t.get_data_type())
    elem = vec[k]
    names = [c.name for c in t.columns]
    row = {n: _get(elem, i - 1) for i, n in enumerate(names) if i >= 1}
    outs = make_outputs(row)
    op = _op([k], _in(k, vec), outs)
    op_sym = _sym("op", op)
    fn = _func("exprs", op_sym, [vec])
    fn.tbl[op_sym] = op
    return fn


def _run_and_compare(eng, fn, t, exact_cols=None, vectorize=False):
    plan = eng.compile(fn, vectorize)
    got = plan_run_table(eng, plan, t)
    ref = loopgen.Query(fn, vectorize)(t)
    assert got["len"] == ref["len"] == N
    for c, (g, r) in enumerate(zip(got["cols"], ref["cols"])):
        assert g.dtype == r.dtype, (c, g.dtype, r.dtype)
        if np.issubdtype(r.dtype, np.floating) and exact_cols is not None and c not in exact_cols:
            # f64: the FP64 tolerance; f32: one single-precision ulp
            rtol = RTOL_F64 if r.dtype == np.float64 else 2.0 ** -23
            np.testing.assert_allclose(g, r, rtol=rtol, atol=0, err_msg="column %d" % c)
        elif np.issubdtype(r.dtype, np.floating):
            # bit for bit, NaN payloads aside
            same = (g.view(np.uint8).reshape(len(g), -1) == r.view(np.uint8).reshape(len(r), -1)).all(axis=1)
            same |= np.isnan(g) & np.isnan(r)
            assert same.all(), "column %d: %d rows differ, first %r vs %r" % (
                c, int((~same).sum()), g[~same][:3], r[~same][:3])
        else:
            np.testing.assert_array_equal(g, r, err_msg="column %d" % c)
    plan.free()


@pytest.mark.parametrize("ty", INT_TYPES)
def test_integer_arithmetic(eng, ty):
    # + - * / % min max neg abs, with C++'s promotion and narrowing back to the operand type
    def outs(r):
        a, b = r["a_" + ty], r["b_" + ty]
        return [_add(a, b), _sub(a, b), _mul(a, b), _div(a, b), _mod(a, b), _max(a, b), _min(a, b), _neg(a),
                _abs(a), _add(_mul(a, ir.Const(ir.DataType(ty), 3)), b)]
    _run_and_compare(eng, _op_of(table(), outs), table())


@pytest.mark.parametrize("ty", FLOAT_TYPES)
def test_float_arithmetic(eng, ty):
    # IEEE-exact operators: + - * / neg abs sqrt ceil floor min max (kernels build without FMA
    # contraction, as the oracle's C++ does); pow within the tolerance (output column 13; column 0
    # is the iterator)
    def outs(r):
        a, b = r["a_" + ty], r["b_" + ty]
        return [_add(a, b), _sub(a, b), _mul(a, b), _div(a, b), _neg(a), _abs(a), _sqrt(_abs(a)), _ceil(a),
                _floor(a), _max(a, b), _min(a, b), _mul(_add(a, b), _sub(a, b)), _pow(_abs(a), b)]
    _run_and_compare(eng, _op_of(table(), outs), table(), exact_cols=set(range(1, 13)))


@pytest.mark.parametrize("src", INT_TYPES + FLOAT_TYPES)
def test_casts_between_all_widths(eng, src):
    # a cast from `src` to every primitive type: integer narrowing wraps, widening sign- or
    # zero-extends, float to integer truncates (operands in range of every target), integer to
    # float rounds to nearest
    t = table()
    targets = INT_TYPES + FLOAT_TYPES

    def outs(r):
        a = r["a_" + src]
        if src in FLOAT_TYPES:
            # keep float-to-integer casts inside [0, 127], the range every target holds
            a = _min(_abs(a), ir.Const(ir.DataType(src), 127.0))
        return [_cast(ir.DataType(dt), a) for dt in targets]
    _run_and_compare(eng, _op_of(t, outs), t)


def test_comparisons_and_logic_per_type(eng):
    # < <= > >= == and/or/not over every type, as 0/1 columns
    t = table()

    def outs(r):
        res = []
        for ty in INT_TYPES + FLOAT_TYPES:
            a, b = r["a_" + ty], r["b_" + ty]
            c = (_lt(a, b) & _not(_eq(a, b))) | (_gte(a, b) & _lte(a, _add(b, b)))
            res.append(_sel(c, _i64(1), _i64(0)))
            res.append(_sel(_gt(a, b), _i64(1), _i64(0)))
        return res
    _run_and_compare(eng, _op_of(t, outs), t)


def test_expressions_vectorized(eng):
    # the vectorised Op form (every row visited, filtered rows null) over the same expressions
    t = table()

    def outs(r):
        a, b = r["a_f64"], r["b_f64"]
        x, y = r["a_u32"], r["b_u32"]
        return [_div(a, b), _sqrt(_abs(b)), _mod(x, y), _cast(ir.DataType("i16"), x)]
    _run_and_compare(eng, _op_of(t, outs), t, vectorize=True)
