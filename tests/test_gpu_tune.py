"""The tiling autotuner: its choice is used by every later run of the query shape and size
bucket (alone and batched alike, so the results keep the same bits), results stay within the
oracle's tolerance, and the choices survive export/import and the JSON file."""
import numpy as np
import pytest

import refqueries as rq
from oracle import loopgen
from parity import assert_same
from reffine_gb300 import engine, workloads as W
from test_gpu_materialize import plan_run_table

pytestmark = pytest.mark.gpu


def test_tune_filter_sum_and_groupby(eng, tmp_path):
    t = W.filter_sum_table(3_000_017, seed=41)
    dt = eng.upload(t)
    plan = eng.compile(W.filter_sum_query(t.get_data_type(), 700, 1300))
    before = plan.run(dt)
    tile, ms = plan.tune(dt, reps=3)
    assert tile % 4 == 0 and 256 <= tile <= 65536 and ms > 0
    # the block size chosen with it: kept for the shape (bucket -1) and used by the plan's kernels
    blocks = [int(l.split()[2]) for l in eng.tune_export().splitlines() if l.split()[1] == "-1"]
    assert blocks and all(b in (128, 256, 512) for b in blocks)
    after = plan.run(dt)
    ref = loopgen.Query(plan.fn)(t)
    assert_same(after, ref)
    assert_same(before, ref)
    # another query of the same shape (other constants) takes the same tiling; batched runs too
    other = eng.compile(W.filter_sum_query(t.get_data_type(), 100, 2000))
    b = engine.Batch(eng, 4)
    o1, o2 = b.add(plan, dt), b.add(other, dt)
    b.launch()
    got = b.wait()
    assert got[0] == after and got[1] == other.run(dt)
    block = [m for m in (128, 256, 512) if "RF_SCAN_REDUCE_KERNEL(rf_main, %d)" % m in plan.source]
    assert len(block) == 1 and "RF_SCAN_REDUCE_KERNEL(rf_main, %d)" % block[0] in other.source
    assert_same(other.run(dt), loopgen.Query(other.fn)(t))
    text = eng.tune_export()
    assert str(tile) in text and len(text.splitlines()) >= 1
    g = W.groupby_table(1_000_003, seed=42)
    dg = eng.upload(g)
    gp = eng.compile(W.groupby_query(g.get_data_type()))
    gt, _ = gp.tune(dg)
    assert_same(gp.run(dg), loopgen.Query(gp.fn)(g))
    path = str(tmp_path / "tune.json")
    eng.tune_save(path)
    eng2 = engine.Engine()
    eng2.tune_load(path)
    assert sorted(eng2.tune_export().splitlines()) == sorted(eng.tune_export().splitlines())
    eng2.close()


def test_tune_hash_group_by_table_sizing(eng):
    # a hash group-by tunes its table's slots per 100 distinct keys; the output keeps its rows
    # and counts, FP64 sums within the oracle's tolerance, and the choice is exported
    t = W.hashgroup_table(400_003, 20_000, seed=43)
    plan = eng.compile(W.hashgroup_query(t.get_data_type()))
    assert plan.kind == 5
    before = plan_run_table(eng, plan, t)
    choice, ms = plan.tune(eng.upload(t), reps=2)
    assert choice in (160, 220, 300) and ms > 0
    after = plan_run_table(eng, plan, t)
    assert before["len"] == after["len"]
    order_b = np.argsort(before["cols"][0])
    order_a = np.argsort(after["cols"][0])
    np.testing.assert_array_equal(before["cols"][0][order_b], after["cols"][0][order_a])
    for c in range(1, len(after["cols"])):
        if np.issubdtype(after["cols"][c].dtype, np.floating):
            np.testing.assert_allclose(after["cols"][c][order_a], before["cols"][c][order_b], rtol=1e-12, atol=0)
        else:
            np.testing.assert_array_equal(after["cols"][c][order_a], before["cols"][c][order_b])
    assert any(l.split()[-1] == str(choice) for l in eng.tune_export().splitlines())


def test_tune_rejects_other_table_outputs(eng):
    st = rq.students_table()
    plan = eng.compile(rq.transform_op(st, 5, 10))
    with pytest.raises(RuntimeError, match="UNSUPPORTED"):
        plan.tune(eng.upload(st))
