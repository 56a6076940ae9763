"""GPU parity of the run-end segmented reduce (the reference's grouped aggregation over a 2-d
vector with a run-end encoded key column) against the oracle."""
import numpy as np
import pytest

import refqueries as rq
from oracle import loopgen
from parity import assert_table_same
from reffine_gb300 import workloads as W
from test_gpu_materialize import plan_run_table

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("vectorize", [False, True])
def test_multidim_golden_on_gpu(eng, vectorize):
    t = rq.runend_table()
    plan = eng.compile(rq.multidim_op(t), vectorize)
    assert plan.kind == 4
    out = plan_run_table(eng, plan, t)
    assert out["len"] == 4
    assert list(out["cols"][0]) == [1, 2, 3, 4]
    assert list(out["cols"][1]) == [3, 7, 26, 9]


@pytest.mark.parametrize("n,nd", [(1, 1), (1000, 50), (300_007, 20_000), (2_000_003, 200_000)])
def test_zipf_grouped_sum_parity(eng, n, nd):
    t = W.ree_sorted(W.hashgroup_table(n, nd, 1.1, seed=4))
    fn = W.hashgroup_query(t.get_data_type())
    plan = eng.compile(fn)
    assert plan.kind == 4
    out = plan_run_table(eng, plan, t)
    ref = loopgen.Query(fn)(t)
    assert_table_same(out, ref)
    assert out["cols"][2].sum() == n


def canon(out):
    order = np.argsort(out["cols"][0], kind="stable")
    return {"len": out["len"], "cols": [c[order] for c in out["cols"]]}


@pytest.mark.parametrize("n,nd", [(1, 1), (5000, 300), (1_000_003, 100_000), (3_000_001, 1_000_000)])
def test_hash_group_by_matches_sorted_runs(eng, n, nd):
    # the same query over unsorted flat keys (hash group-by) and over the keys sorted and
    # run-end encoded (the reference's form, run by the oracle): equal rows, canonicalised by key
    flat = W.hashgroup_table(n, nd, 1.1, seed=6)
    ree = W.ree_sorted(flat)
    fn_flat = W.hashgroup_query(flat.get_data_type())
    plan = eng.compile(fn_flat)
    assert plan.kind == 5
    out = canon(plan_run_table(eng, plan, flat))
    ref = loopgen.Query(W.hashgroup_query(ree.get_data_type()))(ree)
    assert_table_same(out, ref)
    # and the GPU's own run-end path agrees
    seg = plan_run_table(eng, eng.compile(W.hashgroup_query(ree.get_data_type())), ree)
    assert_table_same(canon(seg), ref)


def test_hash_group_by_null_keys_and_values(eng):
    n = 200_000
    flat = W.hashgroup_table(n, 5000, 1.1, seed=8)
    rng = np.random.default_rng(2)
    kmask, vmask = rng.random(n) > 0.05, rng.random(n) > 0.1
    from reffine_gb300.table import pack_validity
    flat.columns[0].valid = pack_validity(kmask)
    flat.columns[1].valid = pack_validity(vmask)
    out = canon(plan_run_table(eng, eng.compile(W.hashgroup_query(flat.get_data_type())), flat))
    # expected: groups are the valid keys; a row adds to its group only if its value is valid
    keys = flat.columns[0].data[kmask]
    vals = flat.columns[1].data[kmask]
    vm = vmask[kmask]
    uk, inv = np.unique(keys, return_inverse=True)
    np.testing.assert_array_equal(out["cols"][0], uk)
    np.testing.assert_array_equal(out["cols"][2], np.bincount(inv, weights=vm, minlength=len(uk)).astype(np.int64))
    np.testing.assert_allclose(out["cols"][1], np.bincount(inv, weights=np.where(vm, vals, 0.0), minlength=len(uk)),
                               rtol=1e-12, atol=1e-9)
