"""Row-chunked runs through the reference-shaped call (compile_op -> rf_plan_thunk): the driving
table is copied in row chunks on a copy stream and each chunk's work units start once their rows
have landed.  The result must have the same bits as the plan run on a device-resident table (same
units, same fold order), and match the oracle."""
import numpy as np
import pytest

from oracle import loopgen
from parity import assert_same
from reffine_gb300 import engine, ir, workloads as W
from reffine_gb300.ir import _add, _f64, _func, _get, _gte, _i64, _idx, _len, _lt, _mul, _new, _red, _sel, _subvec, _sym
from reffine_gb300.table import Column, Table, pack_validity

pytestmark = pytest.mark.gpu


def offset_sum_query(tbl_type, start):
    """SUM(price * discount), COUNT over rows [start, len) with day >= 100."""
    vec = _sym("lineitem", tbl_type)

    def acc(s, v):
        ok = _gte(_get(v, 0), ir._i32(100))
        return _new([_sel(ok, _add(_get(s, 0), _mul(_get(v, 1), _get(v, 2))), _get(s, 0)),
                     _sel(ok, _add(_get(s, 1), _i64(1)), _get(s, 1))])

    red = _red(_subvec(vec, _idx(start), _len(vec, 1)), lambda: _new([_f64(0), _i64(0)]), acc)
    red_sym = _sym("red", red)
    fn = _func("offset_sum", red_sym, [vec])
    fn.tbl[red_sym] = red
    return fn


def case(name):
    if name == "filter_sum":
        t = W.filter_sum_table(6_000_017, seed=41)
        return W.filter_sum_query(t.get_data_type()), [t]
    if name == "groupby":
        t = W.groupby_table(6_000_003, seed=42)
        return W.groupby_query(t.get_data_type()), [t]
    if name == "join":
        b, p = W.join_tables(50_000, 6_000_011, seed=43)
        return W.join_query(b.get_data_type(), p.get_data_type()), [b, p]
    if name == "nulls":
        t = W.filter_sum_table(6_000_001, seed=44)
        t.columns[1].valid = pack_validity(np.random.default_rng(2).random(len(t)) < 0.8)
        return W.filter_sum_query(t.get_data_type()), [t]
    if name == "offset":
        t = W.filter_sum_table(7_000_003, seed=45)
        return offset_sum_query(t.get_data_type(), 777_777), [t]
    raise KeyError(name)


def pinned_copy(eng, t, keep):
    """The same table with its values (and validity) in pinned host memory."""
    cols = []
    for c in t.columns:
        buf = eng.host_alloc(c.data.nbytes)
        v = buf.view(c.data.dtype, len(c.data))
        v[:] = c.data
        keep.append(buf)
        valid = None
        if c.valid is not None:
            vb = eng.host_alloc(c.valid.nbytes)
            valid = vb.view(np.uint8, len(c.valid))
            valid[:] = c.valid
            keep.append(vb)
        cols.append(Column(c.name, c.dtype, v, valid, c.run_ends))
    return Table(t.name, t.dim, cols)


@pytest.fixture(scope="module")
def fresh():
    """A context of its own, with no tuning from earlier tests: the default tiling leaves several
    units per SM, so a call from pinned memory is streamed in chunks.  (A tuned one-wave tiling
    has too few units to chunk; such a call is copied whole, then run.)"""
    e = engine.Engine(0)
    yield e
    e.close()


@pytest.mark.parametrize("name", ["filter_sum", "groupby", "join", "nulls", "offset"])
def test_streamed_call_same_bits(fresh, name):
    eng = fresh
    fn, tables = case(name)
    keep = []
    pinned = [pinned_copy(eng, t, keep) for t in tables]
    q = engine.compile_op(fn, engine=eng)
    l0 = eng.launch_count()
    got = q(*pinned)
    assert eng.launch_count() - l0 >= 2  # launched a chunk of units at a time
    plan = eng.compile(fn)
    resident = plan.run(*[eng.upload(t) for t in tables])
    assert got == resident
    assert_same(got, loopgen.Query(fn)(*tables))
    assert q(*pinned) == got  # staging buffers reused: same bits again
    # pageable host memory takes the whole-copy path: the same bits
    l0 = eng.launch_count()
    assert q(*tables) == got
    for b in keep:
        b.free()


def test_tiny_and_empty_tables(eng):
    for n in (0, 1, 100):
        t = W.filter_sum_table(n, seed=46)
        fn = W.filter_sum_query(t.get_data_type())
        got = engine.compile_op(fn, engine=eng)(t)
        assert got == eng.compile(fn).run(eng.upload(t))
        assert_same(got, loopgen.Query(fn)(t))
