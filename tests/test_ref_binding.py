"""The binding of Reffine's own IR to the C-ABI (reffine_gb300/binding/ref_binding.cpp): queries
built with the reference's builder, printed by func_text, against the same queries built with
this package's Python builder.

tests/golden/ref_func_text.tsv holds the binding's output for the benchmark queries and the
reference's gtest queries (made by tests/golden/make_ref_func_text.py from a Reffine checkout).
With REFFINE_SRC pointing at a checkout, the fixture is rebuilt and must not have changed.

Both texts are brought to a canonical form - symbol-table entries substituted into the output,
symbols renamed in order of first use, constants read as numbers - and must be equal: the
reference's Func and the Python builder's Func are the same expression graph.  Each text must
also lower and compile for sm_103a (rf_plan_check; no GPU needed).
"""
import os

import pytest

import refqueries as rq
from reffine_gb300 import _capi, workloads as W
from reffine_gb300.table import Table

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "ref_func_text.tsv")


def fixture():
    out = {}
    for line in open(FIXTURE):
        name, text = line.rstrip("\n").split("\t", 1)
        out[name] = text
    return out


def python_funcs():
    st = rq.students_table()
    gen = Table.from_arrays(1, {"t": np.arange(4, dtype=np.int64), "v": np.arange(4, dtype=np.int64)})
    b, p = W.join_tables(8, 8)
    return {
        "vector_op": rq.vector_op(st),
        "transform_op": rq.transform_op(st, 5, 10),
        "multidim_op": rq.multidim_op(rq.runend_table()),
        "gen_table_op": rq.gen_table_op(),
        "join_op": rq.join_op(gen, gen, gen),
        "nested_op": rq.nested_op(10, 10),
        "filter_sum": W.filter_sum_query(W.filter_sum_table(8).get_data_type()),
        "groupby": W.groupby_query(W.groupby_table(8).get_data_type()),
        "hashgroup": W.hashgroup_query(W.hashgroup_table(8, 4).get_data_type()),
        "join_agg": W.join_query(b.get_data_type(), p.get_data_type()),
        "hashgroup_ree": W.hashgroup_query(W.ree_sorted(W.hashgroup_table(8, 4)).get_data_type()),
    }


# ---------------------------------------------------------------------------- canonical form
def _parse(text):
    toks = text.replace("(", " ( ").replace(")", " ) ").split()
    pos = 0

    def read():
        nonlocal pos
        t = toks[pos]
        pos += 1
        if t == "(":
            lst = []
            while toks[pos] != ")":
                lst.append(read())
            pos += 1
            return lst
        return t

    tree = read()
    assert pos == len(toks)
    return tree


def canonical(text):
    _, name, output, inputs, tbl = _parse(text)
    defs = {k: v for k, v in tbl[1:]}
    names = {}

    def rename(sym):
        if sym not in names:
            names[sym] = "s%d" % len(names)
        return names[sym]

    declared = {nm for nm, _ in inputs[1:]}

    def walk(x, scope):
        if isinstance(x, str):
            if x in defs and x not in scope:
                return walk(defs[x], scope)
            if x in scope or x in declared:
                return rename(x)
            return x
        head = x[0] if x else None
        if head == "const":
            return ["const", x[1], repr(float(x[2]))]
        if head == "op":
            iters = x[1]
            inner = scope | {nm for nm, _ in iters}
            return ["op", [[rename(nm), ty] for nm, ty in iters], walk(x[2], inner), [walk(o, inner) for o in x[3]]]
        if head == "reduce":
            (st, st_t), (vl, vl_t) = x[3], x[4]
            inner = scope | {st, vl}
            return ["reduce", walk(x[1], scope), walk(x[2], scope), [rename(st), st_t], [rename(vl), vl_t],
                    walk(x[5], inner)]
        if head in ("get", "len", "readdata"):
            return [head] + [walk(a, scope) for a in x[1:-1]] + [x[-1]]
        if head == "cast":
            return ["cast", x[1], walk(x[2], scope)]
        return [walk(a, scope) if i else a for i, a in enumerate(x)]

    ins = [[rename(nm), ty] for nm, ty in inputs[1:]]
    return repr([name, walk(output, frozenset()), ins])


# ---------------------------------------------------------------------------- tests
def test_fixture_is_current():
    src = os.environ.get("REFFINE_SRC")
    if not src or not os.path.isdir(os.path.join(src, "include", "reffine")):
        pytest.skip("REFFINE_SRC (a Reffine checkout) not set")
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_ref_func_text import build_and_run
    assert build_and_run(src) == open(FIXTURE).read()


@pytest.mark.parametrize("name", sorted(python_funcs()))
def test_reference_built_func_is_the_python_built_func(name):
    ref = fixture()[name]
    py = python_funcs()[name].text()
    assert canonical(ref) == canonical(py)


@pytest.mark.parametrize("name", sorted(python_funcs()))
def test_reference_built_func_lowers_for_sm103a(name):
    import ctypes
    lib = _capi.load()
    text = fixture()[name].encode()
    for vectorize in (0, 1):
        buf = ctypes.create_string_buffer(1 << 20)
        st = lib.rf_plan_check(text, vectorize, buf, len(buf))
        if name in ("groupby", "hashgroup") and vectorize and st == _capi.RF_ERR_UNSUPPORTED:
            continue
        assert st == _capi.RF_OK, buf.value.decode(errors="replace")[:500]


def test_canonical_form_tells_queries_apart():
    fx = fixture()
    forms = {canonical(t) for t in fx.values()}
    assert len(forms) == len(fx)
    # a changed constant, a swapped operand or a different column is a different query
    t = fx["filter_sum"]
    assert canonical(t.replace("(const i32 730)", "(const i32 731)", 1)) != canonical(t)
    assert canonical(t.replace("(gte (get val 0)", "(gte (get val 1)", 1)) != canonical(t)
    assert canonical(fx["join_agg"].replace("(readdata build", "(readdata probe", 1)) != canonical(fx["join_agg"])
