"""Batched execution: many queries of several shapes in one launch per shape, replayed as a CUDA
graph.  Each result must have the same bits as the query run alone (same units, same fold
order), and match the oracle."""
import numpy as np
import pytest

from oracle import loopgen
from parity import assert_same
from reffine_gb300 import engine, workloads as W

pytestmark = pytest.mark.gpu


def test_batch_results_equal_standalone(eng):
    rng = np.random.default_rng(0)
    t0 = [W.filter_sum_table(int(n), seed=i) for i, n in enumerate([1000, 50_000, 700_001])]
    t1 = [W.groupby_table(int(n), seed=10 + i) for i, n in enumerate([3000, 400_003])]
    b, p = W.join_tables(20_000, 300_007, seed=7)
    d0 = [eng.upload(t) for t in t0]
    d1 = [eng.upload(t) for t in t1]
    db, dp = eng.upload(b).build_index(), eng.upload(p)
    queries = []
    for k in range(40):
        s = k % 3
        if s == 0:
            lo = int(rng.integers(0, 2000))
            fn = W.filter_sum_query(t0[0].get_data_type(), lo, lo + int(rng.integers(1, 600)))
            i = int(rng.integers(0, 3))
            queries.append((fn, [d0[i]], [t0[i]]))
        elif s == 1:
            fn = W.groupby_query(t1[0].get_data_type(), int(rng.integers(100, 2557)))
            i = int(rng.integers(0, 2))
            queries.append((fn, [d1[i]], [t1[i]]))
        else:
            lo = int(rng.integers(0, 2000))
            fn = W.join_query(b.get_data_type(), p.get_data_type(), 5, lo, lo + 365)
            queries.append((fn, [db, dp], [b, p]))
    plans = [eng.compile(fn) for fn, _, _ in queries]
    alone = [pl.run(*dts) for pl, (_, dts, _) in zip(plans, queries)]
    batch = engine.Batch(eng, 64)
    for rep in range(3):  # the second and third launches replay the captured graph
        batch.reset()
        for pl, (_, dts, _) in zip(plans, queries):
            batch.add(pl, *dts)
        batch.launch()
        mixed = batch.wait()
        assert mixed == alone  # bit-identical
    for (fn, _, tabs), got in zip(queries[:6], mixed[:6]):
        assert_same(got, loopgen.Query(fn)(*tabs))


def test_batch_poll_and_capacity(eng):
    t = W.filter_sum_table(10_000, seed=3)
    dt = eng.upload(t)
    plan = eng.compile(W.filter_sum_query(t.get_data_type()))
    batch = engine.Batch(eng, 2)
    batch.add(plan, dt)
    batch.add(plan, dt)
    with pytest.raises(Exception):
        batch.add(plan, dt)  # full
    batch.launch()
    import time
    t_end = time.time() + 30
    while not batch.poll():
        assert time.time() < t_end
    r = [engine.from_c(o) for _, o in batch._keep]
    assert r[0] == r[1] == plan.run(dt)
