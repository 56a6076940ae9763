"""The serving loop on the GPU: a mixed workload over resident tables, replayed with Poisson
arrivals in batched and per-query mode; every result must equal the query run alone (value
results bit for bit, hash group-by tables key-sorted within 1e-12)."""
import ctypes
import math

import numpy as np
import pytest

from oracle import loopgen
from parity import assert_same
from reffine_gb300 import _capi, serve, workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wl(eng):
    return serve.build_workload(eng, n_queries=400, tables_per_shape=3, min_rows=1_000, max_rows=2_000_000, seed=5)


@pytest.fixture(scope="module")
def alone(eng, wl):
    return serve.run_alone(eng, wl.requests)


def test_workload_mix(wl):
    shapes = np.bincount([r.shape for r in wl.requests], minlength=4)
    assert (shapes > 50).all()
    assert len({r.plan.h.value for r in wl.requests}) > 100  # fresh constants per query


def test_alone_matches_oracle(wl, alone):
    # a sample of the stand-alone results against the oracle (filter+sum, group-by, join)
    seen = set()
    for r, a in zip(wl.requests, alone):
        if r.shape in seen or r.shape == 2 or len(seen) == 3:
            continue
        seen.add(r.shape)
        out = r.plan.new_out()
        ctypes.memmove(ctypes.addressof(out), a, len(a))
        assert_same(serve.from_c(out), loopgen.Query(r.plan.fn)(*r.host))
    assert seen == {0, 1, 3}


@pytest.mark.parametrize("mode,rate", [("batched", math.inf), ("batched", 20_000.0), ("per_query", math.inf)])
def test_mixed_results_equal_alone(eng, wl, alone, mode, rate):
    summ = serve.serve_run(eng, wl, mode, rate, alone, check_tables=True, lanes=2, max_batch=64)
    assert summ["failed"] == 0
    assert summ["mismatches"] == 0
    if mode == "batched" and math.isinf(rate):
        assert summ["mean_batch"] > 1.5  # queries were actually packed together


def test_table_lanes_results_equal_alone(eng, wl, alone):
    # three table-result lanes (high stream priority, the default): hash group-bys run beside each other
    # (never two runs of one plan at once) and beside the batches; results unchanged
    summ = serve.serve_run(eng, wl, "batched", math.inf, alone, check_tables=True, lanes=2, max_batch=64,
                           table_lanes=3)
    assert summ["failed"] == 0
    assert summ["mismatches"] == 0


def test_small_budget_and_one_lane(eng, wl, alone):
    # a budget below most requests' scratch: they run one at a time, results unchanged
    summ = serve.serve_run(eng, wl, "batched", math.inf, alone, check_tables=True, lanes=1, max_batch=8,
                           hbm_budget_bytes=4096)
    assert summ["failed"] == 0 and summ["mismatches"] == 0
    assert summ["peak_inflight_bytes"] > 0


def test_pause_cancel_and_queue_full(eng, wl):
    reqs = [r for r in wl.requests if r.shape in (0, 1)][:3]
    srv = serve.Server(eng, "batched", queue_capacity=3)
    srv.pause(True)
    outs = [srv.submit(r.plan, *r.inputs, tag=i) for i, r in enumerate(reqs)]
    with pytest.raises(RuntimeError, match="queue full"):
        srv.submit(reqs[0].plan, *reqs[0].inputs, tag=99)
    srv.cancel(1)
    with pytest.raises(RuntimeError):
        srv.cancel(42)  # unknown
    srv.pause(False)
    got = {}
    for _ in range(200):
        for c in srv.poll(16, 10_000):
            got[c.tag] = c.status
        if len(got) == 3:
            break
    assert got == {0: _capi.RF_OK, 1: _capi.RF_ERR_CANCELLED, 2: _capi.RF_OK}
    st = srv.stats()
    assert st["rejected"] == 1 and st["cancelled"] == 1 and st["completed"] == 2
    assert serve.from_c(outs[0]) == reqs[0].plan.run(*reqs[0].inputs)
    srv.close()


def test_free_cancels_pending(eng, wl):
    r = wl.requests[0]
    srv = serve.Server(eng, "per_query")
    srv.pause(True)
    srv.submit(r.plan, *r.inputs, tag=7)
    srv.close()  # pending work completes as cancelled, nothing runs after free
