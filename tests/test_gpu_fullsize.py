"""GPU parity at the benchmark sizes: the four query shapes on the same seeded tables the
benchmark times (6M-row filter+sum, 60M-row 6-group group-by, 100M-row Zipf(1.1) hash group-by
over 10M ranks, 10M x 200M filtered join), each compared with the oracle on the full table.

Integers (counts, keys, row counts) bit-exact; FP64 sums within 1e-12 relative of the oracle's
serial sums.  For the hash group-by, whose largest group holds about a tenth of the rows, the
test also measures both sums' distance from the exact sum (math.fsum) of the largest groups: the
GPU's reassociated sum must be no further from it than the tolerance allows.
"""
import math

import numpy as np
import pytest

from oracle import loopgen
from parity import RTOL_F64, assert_same, assert_table_same
from reffine_gb300 import workloads as W
from test_gpu_materialize import plan_run_table

pytestmark = pytest.mark.gpu


def _free(*objs):
    for o in objs:
        o.free()


def test_filter_sum_6M_matches_oracle(eng):
    t = W.filter_sum_table(6_000_000, seed=0)
    fn = W.filter_sum_query(t.get_data_type())
    dt = eng.upload(t)
    plan = eng.compile(fn)
    got = plan.run(dt)
    ref = loopgen.Query(fn)(t)
    assert got[1] == ref[1] and ref[1] > 100_000
    assert_same(got, ref)
    _free(plan, dt)


def test_groupby_60M_matches_oracle(eng):
    t = W.groupby_table(60_000_000, seed=1)
    fn = W.groupby_query(t.get_data_type())
    dt = eng.upload(t)
    plan = eng.compile(fn)
    got = plan.run(dt)
    ref = loopgen.Query(fn)(t)
    assert sum(g[7] for g in ref) > 55_000_000
    assert_same(got, ref)
    _free(plan, dt)


def test_hash_groupby_100M_zipf_matches_oracle(eng):
    flat = W.hashgroup_table(100_000_000, 10_000_000, 1.1, seed=2)
    plan = eng.compile(W.hashgroup_query(flat.get_data_type()))
    assert plan.kind == 5
    out = plan_run_table(eng, plan, flat)
    plan.free()
    order = np.argsort(out["cols"][0], kind="stable")
    out = {"len": out["len"], "cols": [c[order] for c in out["cols"]]}
    ree = W.ree_sorted(flat)
    ref = loopgen.Query(W.hashgroup_query(ree.get_data_type()))(ree)
    assert out["cols"][2].sum() == 100_000_000
    assert_table_same(out, ref)
    # the largest groups: both sums against the exact sum
    keys, vals = flat.columns[0].data, flat.columns[1].data
    for i in np.argsort(ref["cols"][2])[-4:]:
        exact = math.fsum(vals[keys == ref["cols"][0][i]].tolist())
        assert abs(out["cols"][1][i] - exact) <= RTOL_F64 * abs(exact)
        assert abs(ref["cols"][1][i] - exact) <= RTOL_F64 * abs(exact)


def test_join_10M_x_200M_matches_oracle(eng):
    b, p = W.join_tables(10_000_000, 200_000_000, seed=3)
    fn = W.join_query(b.get_data_type(), p.get_data_type())
    db, dp = eng.upload(b), eng.upload(p)
    plan = eng.compile(fn)
    got = plan.run(db, dp)
    _free(plan, db, dp)
    ref = loopgen.Query(fn)(b, p)
    assert sum(g[1] for g in ref) > 1_000_000
    assert_same(got, ref)
