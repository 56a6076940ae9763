"""Host-side pieces of the serving loop, without a GPU: arrival process, table sizes, latency
summary and the result comparison rules."""
import math

import numpy as np

from reffine_gb300 import serve


def test_poisson_arrivals_rate():
    a = serve.poisson_arrivals(20_000, 5_000.0, seed=1)
    assert (np.diff(a) >= 0).all()
    assert abs(a[-1] / 1e9 - 20_000 / 5_000.0) < 0.1  # ~4 s of arrivals
    assert (serve.poisson_arrivals(10, math.inf, seed=1) == 0).all()  # closed loop: all at once


def test_log_uniform_sizes_bounds_and_spread():
    s = serve.log_uniform_sizes(np.random.default_rng(4), 2000, 1_000, 50_000_000)
    assert min(s) >= 1_000 and max(s) <= 50_000_000
    logs = np.log10(s)
    # log-uniform: each decade holds about the same share
    h, _ = np.histogram(logs, bins=[3, 4, 5, 6, 7])
    assert h.min() > 0.7 * h.max()


def test_latency_summary():
    dt = np.dtype([("tag", "<u8"), ("status", "<i4"), ("batch_queries", "<i4"), ("t_submit_ns", "<i8"),
                   ("t_launch_ns", "<i8"), ("t_done_ns", "<i8")])
    rec = np.zeros(100, dtype=dt)
    rec["t_submit_ns"] = np.arange(100) * 1000
    rec["t_done_ns"] = rec["t_submit_ns"] + (np.arange(100) + 1) * 1000  # latencies 1..100 us
    rec["batch_queries"] = 4
    rec["status"][5] = 8  # one cancelled
    s = serve.latency_summary(rec)
    assert s["failed"] == 1
    assert 49 <= s["p50_us"] <= 52 and 98 <= s["p99_us"] <= 100
    assert s["mean_batch"] == 4


def test_tables_close_rules():
    a = {"cols": [np.array([1, 2, 3]), np.array([1.0, 2.0, 3.0])], "len": 3}
    b = {"cols": [np.array([1, 2, 3]), np.array([1.0, 2.0 * (1 + 1e-14), 3.0])], "len": 3}
    c = {"cols": [np.array([1, 2, 4]), np.array([1.0, 2.0, 3.0])], "len": 3}
    d = {"cols": [np.array([1, 2, 3]), np.array([1.0, 2.0 * (1 + 1e-10), 3.0])], "len": 3}
    assert serve.tables_close(a, b)          # FP64 within 1e-12
    assert not serve.tables_close(a, c)      # keys bit-exact
    assert not serve.tables_close(a, d)      # FP64 beyond 1e-12
