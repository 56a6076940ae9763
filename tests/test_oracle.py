"""The oracle against the reference's own known answers (CPU only).

Golden values are the assertions of Reffine's gtest suite: test_reduce.cpp:58 (131977),
test_reduce.cpp:121 (696), test_multidim.cpp:47-54 (keys [1,2,3,4], sums [3,7,26,9]),
test_join.cpp:62-86, test_transform.cpp:43-52, test_nested.cpp:42-53.
"""
import numpy as np
import pytest

import refqueries as rq
from oracle import loopgen


@pytest.mark.parametrize("vectorize", [False, True])
def test_reduce_loop_golden(vectorize):
    st = rq.students_table(2)
    assert loopgen.Query(rq.sum_col1_op(st), vectorize)(st) == 131977


@pytest.mark.parametrize("vectorize", [False, True])
def test_reduce_op_golden(vectorize):
    st = rq.students_table()
    assert loopgen.Query(rq.vector_op(st), vectorize)(st) == 696


@pytest.mark.parametrize("vectorize", [False, True])
def test_transform_identities(vectorize):
    st = rq.students_table()
    r = loopgen.Query(rq.transform_op(st, 5, 10), vectorize)(st)
    n = len(st)
    assert r["len"] == n - 5
    ids = st.columns[0].data
    hs = st.columns[1].data
    np.testing.assert_array_equal(r["cols"][0], ids[5:])
    np.testing.assert_array_equal(r["cols"][1], hs[5:] + 10)


@pytest.mark.parametrize("vectorize", [False, True])
def test_multidim_golden(vectorize):
    t = rq.runend_table()
    r = loopgen.Query(rq.multidim_op(t), vectorize)(t)
    assert r["len"] == 4
    assert list(r["cols"][0]) == [1, 2, 3, 4]
    assert list(r["cols"][1]) == [3, 7, 26, 9]


@pytest.mark.parametrize("vectorize", [False, True])
def test_join_identities(vectorize):
    g = loopgen.Query(rq.gen_table_op(), vectorize)
    bounds = [(0, 10), (5, 15), (7, 12)]
    ts = [rq.table_from_out(g(lo, hi), ["t", "v"]) for lo, hi in bounds]
    r = loopgen.Query(rq.join_op(*ts), vectorize)(*ts)
    lb, ub = max(b[0] for b in bounds), min(b[1] for b in bounds)
    assert r["len"] == ub - lb
    np.testing.assert_array_equal(r["cols"][0], np.arange(lb, ub))
    np.testing.assert_array_equal(r["cols"][1], 3 * np.arange(lb, ub))


@pytest.mark.parametrize("vectorize", [False, True])
def test_nested_identities(vectorize):
    r = loopgen.Query(rq.nested_op(10, 10), vectorize)()
    valid = r["valid"] if r["valid"] is not None else np.ones(r["len"], bool)
    a, b, ab = r["cols"]
    idx = np.arange(100)
    np.testing.assert_array_equal(a[valid], idx // 10)
    np.testing.assert_array_equal(b[valid], idx % 10)
    np.testing.assert_array_equal(ab[valid], idx // 10 + idx % 10)
    assert valid.sum() == 100
