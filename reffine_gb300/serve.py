"""Batched serving over resident tables: the Python side of rf_server_* and the mixed workload.

The workload is many queries drawn uniformly from four operator shapes - filter+sum
(TPC-H Q6's Reduce, tpch.h:174-208), low-cardinality group-by (Q1's select-per-group
accumulators, tpch.h:412-478), high-cardinality group-by over Zipf keys, and a hash-join probe
with a grouped sum (Q3's Locate, tpch.h:51-56) - with filter constants drawn per query (at
most 6 decimals, the precision the reference's C emitter prints constants with,
cemitter.cpp:99-101) over tables whose sizes are log-uniform, all resident on the device.
Arrivals are Poisson.  The same requests run through the server in batched mode and in
per-query mode (one rf_plan_run per request, in arrival order), and every result of every run
is compared with the query run alone.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _capi, ir
from . import workloads as W
from .engine import DeviceTable, Engine, Plan, from_c
from .table import Table

SHAPES = ("filter_sum", "groupby", "hashgroup", "join")


class Server:
    """A running rf_server (its scheduler threads live in the library)."""

    def __init__(self, eng: Engine, mode: str = "batched", max_batch: int = 256, lanes: int = 2,
                 queue_capacity: int = 1 << 16, hbm_budget_bytes: int = 8 << 30, lane_share_pct: int = 75,
                 table_lanes: int = 0, table_priority: int = 0, table_share_pct: int = 0):
        self.eng = eng
        cfg = _capi.RfServerConfig()
        cfg.mode = {"batched": _capi.RF_SERVE_BATCHED, "per_query": _capi.RF_SERVE_PER_QUERY}[mode]
        cfg.max_batch, cfg.lanes, cfg.queue_capacity, cfg.hbm_budget_bytes = max_batch, lanes, queue_capacity, \
            hbm_budget_bytes
        cfg.lane_share_pct = lane_share_pct
        cfg.table_lanes, cfg.table_priority, cfg.table_share_pct = table_lanes, table_priority, table_share_pct
        h = ctypes.c_void_p()
        eng.check(eng.lib.rf_server_create(eng.h, ctypes.byref(cfg), ctypes.byref(h)))
        self.h = h
        self.mode = mode
        self._keep: Dict[int, object] = {}

    def submit(self, plan: Plan, *inputs, tag: int):
        """Queues one run; returns the object that receives its result (a ctypes struct for a
        value, a c_void_p holding the rf_table* for a table)."""
        args = plan.args(*inputs)
        out = ctypes.c_void_p() if plan.info.output_is_table else plan.new_out()
        self.eng.check(self.eng.lib.rf_server_submit(self.h, plan.h, args, len(inputs), ctypes.byref(out), tag))
        self._keep[tag] = (args, out)
        return out

    def pause(self, paused: bool = True):
        self.eng.check(self.eng.lib.rf_server_pause(self.h, int(paused)))

    def cancel(self, tag: int):
        self.eng.check(self.eng.lib.rf_server_cancel(self.h, tag))

    def poll(self, max_n: int = 256, timeout_us: int = 0) -> List[_capi.RfCompletion]:
        buf = (_capi.RfCompletion * max_n)()
        n = ctypes.c_int32()
        self.eng.check(self.eng.lib.rf_server_poll(self.h, buf, max_n, ctypes.byref(n), timeout_us))
        done = [buf[i] for i in range(n.value)]
        for c in done:
            self._keep.pop(c.tag, None)
        return done

    def stats(self) -> Dict[str, int]:
        st = _capi.RfServerStats()
        self.eng.check(self.eng.lib.rf_server_get_stats(self.h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in st._fields_}

    def replay(self, plans: Sequence[Plan], inputs: Sequence[tuple], outs: Sequence, arrival_ns: np.ndarray):
        """Open-loop replay (rf_server_replay): request i is submitted arrival_ns[i] after the
        start; returns the completion records as a numpy structured array indexed by request."""
        n = len(plans)
        args = [p.args(*x) for p, x in zip(plans, inputs)]
        c_plans = (ctypes.c_void_p * n)(*[p.h.value for p in plans])
        c_args = (ctypes.POINTER(_capi.RfArg) * n)(*[ctypes.cast(a, ctypes.POINTER(_capi.RfArg)) for a in args])
        c_nargs = (ctypes.c_int32 * n)(*[len(x) for x in inputs])
        c_outs = (ctypes.c_void_p * n)(*[ctypes.addressof(o) for o in outs])
        c_arr = (ctypes.c_int64 * n)(*[int(t) for t in arrival_ns])
        rec = (_capi.RfCompletion * n)()
        self.eng.check(self.eng.lib.rf_server_replay(self.h, n, c_plans, c_args, c_nargs, c_outs, c_arr, rec))
        dt = np.dtype([("tag", "<u8"), ("status", "<i4"), ("batch_queries", "<i4"), ("t_submit_ns", "<i8"),
                       ("t_launch_ns", "<i8"), ("t_done_ns", "<i8")])
        return np.frombuffer(bytes(rec), dtype=dt).copy()

    def close(self):
        if self.h:
            self.eng.lib.rf_server_free(self.h)
            self.h = None

    def __del__(self):
        try:
            if self.eng.h:
                self.close()
        except Exception:
            pass


# ----------------------------------------------------------------------------- the workload
@dataclass
class Request:
    shape: int
    plan: Plan
    inputs: tuple
    rows: int             # rows scanned
    nbytes: int           # algorithmic bytes: referenced input columns, read once
    host: tuple = ()      # the host tables behind `inputs`


@dataclass
class Workload:
    requests: List[Request]
    tables: Dict[int, list] = field(default_factory=dict)  # shape -> [(host Table(s), DeviceTable(s))]
    resident_bytes: int = 0
    tuning: Dict[str, int] = field(default_factory=dict)  # "shape/rows" -> tile rows chosen


def log_uniform_sizes(rng, k: int, lo: int, hi: int) -> List[int]:
    return [int(round(math.exp(rng.uniform(math.log(lo), math.log(hi))))) for _ in range(k)]


def _prefix(t: Table, n: int) -> Table:
    return Table.from_arrays(t.dim, {c.name: c.data[:n] for c in t.columns}, name=t.name)


def build_workload(eng: Engine, n_queries: int = 10_000, tables_per_shape: int = 6, min_rows: int = 1_000,
                   max_rows: int = 50_000_000, seed: int = 4, shapes: Sequence[int] = (0, 1, 2, 3),
                   tune: bool = True) -> Workload:
    """Tables per shape with log-uniform row counts in [min_rows, max_rows] (each a prefix of one
    seeded table of the largest drawn size), uploaded once; then n_queries requests, each a
    uniform shape, a uniform table of that shape and fresh filter constants."""
    rng = np.random.default_rng(seed)
    wl = Workload(requests=[])
    sizes = {s: sorted(log_uniform_sizes(rng, tables_per_shape, min_rows, max_rows)) for s in shapes}
    for s in shapes:
        big = sizes[s][-1]
        pool = []
        if s == 0:
            base = W.filter_sum_table(big, seed=seed + 10)
            for n in sizes[s]:
                t = _prefix(base, n)
                pool.append((t, eng.upload(t)))
        elif s == 1:
            base = W.groupby_table(big, seed=seed + 11)
            for n in sizes[s]:
                t = _prefix(base, n)
                pool.append((t, eng.upload(t)))
        elif s == 2:
            # Zipf(1.1) keys over max_rows/10 ids, as 100M rows over 10M keys
            base = W.hashgroup_table(big, ndistinct=max(big // 10, 1), seed=seed + 12)
            for n in sizes[s]:
                t = _prefix(base, n)
                pool.append((t, eng.upload(t)))
        else:
            # build side 1/20 of the probe side, as 10M build rows for 200M probe rows
            bsz = max(big // 20, 1000)
            b, p = W.join_tables(bsz, big, seed=seed + 13)
            db = eng.upload(b).build_index()
            for n in sizes[s]:
                t = _prefix(p, n)
                pool.append(((b, t), (db, eng.upload(t))))
        wl.tables[s] = pool
    for s, pool in wl.tables.items():
        for host, _ in pool:
            for t in (host if isinstance(host, tuple) else (host,)):
                wl.resident_bytes += t.nbytes()
    # each shape's query type is the same for every table of the pool
    types = {s: (wl.tables[s][0][0][0].get_data_type(), wl.tables[s][0][0][1].get_data_type()) if s == 3
             else wl.tables[s][0][0].get_data_type() for s in wl.tables}
    plan_cache: Dict[str, Plan] = {}

    def plan_of(fn: ir.Func) -> Plan:
        key = fn.text()
        if key not in plan_cache:
            plan_cache[key] = eng.compile(fn)
        return plan_cache[key]

    shape_list = list(wl.tables)
    tuned = {}  # (shape, table index) -> first plan of that shape on that table
    for _ in range(n_queries):
        s = shape_list[int(rng.integers(0, len(shape_list)))]
        pool = wl.tables[s]
        host, dev = pool[int(rng.integers(0, len(pool)))]
        if s == 0:
            lo = int(rng.integers(0, 2200))
            hi = lo + int(rng.integers(30, 400))
            dlo = int(rng.integers(0, 9)) / 100.0
            fn = W.filter_sum_query(types[0], lo, hi, dlo, round(dlo + 0.02, 6), float(rng.integers(10, 41)))
            req = Request(0, plan_of(fn), (dev,), len(host), W.algorithmic_bytes(host, [1, 2, 3, 4]), (host,))
        elif s == 1:
            fn = W.groupby_query(types[1], int(rng.integers(1000, 2557)))
            req = Request(1, plan_of(fn), (dev,), len(host), W.algorithmic_bytes(host, [1, 2, 3, 4, 5, 6, 7]),
                          (host,))
        elif s == 2:
            fn = W.hashgroup_query(types[2])
            req = Request(2, plan_of(fn), (dev,), len(host), W.algorithmic_bytes(host, [0, 1]), (host,))
        else:
            lo = int(rng.integers(0, 2000))
            fn = W.join_query(types[3][0], types[3][1], int(rng.integers(1, 26)), lo, lo + int(rng.integers(30, 500)))
            b, p = host
            req = Request(3, plan_of(fn), dev, len(p),
                          W.algorithmic_bytes(b, [0, 1]) + W.algorithmic_bytes(p, [1, 2, 3]), host)
        wl.requests.append(req)
    if tune:
        # the autotuner's tiling for each Reduce shape and table size (one representative query
        # each; the choice applies to every query of the shape and size bucket).  The hash
        # group-bys keep the default table sizing here
        for r in wl.requests:
            if r.plan.info.output_is_table:
                continue
            key = (r.shape, r.rows)
            if key in tuned:
                continue
            tuned[key] = r.plan.tune(*r.inputs)
        wl.tuning = {"%s/%d" % (SHAPES[k[0]], k[1]): v[0] for k, v in sorted(tuned.items())}
    return wl


# ----------------------------------------------------------------------------- running it
def new_outs(reqs: Sequence[Request]) -> list:
    return [ctypes.c_void_p() if r.plan.info.output_is_table else r.plan.new_out() for r in reqs]


def canonical(eng: Engine, plan: Plan, h) -> Dict:
    """A table result exported and sorted by its key columns (a hash group-by emits its groups in
    no fixed order)."""
    dt = DeviceTable(eng, ctypes.c_void_p(h), plan.fn.output.type, [])
    try:
        out = dt.export()
    finally:
        dt.free()
    cols = out["cols"]
    order = np.lexsort(tuple(reversed(cols[:1]))) if cols and len(cols[0]) else np.arange(0)
    return {"cols": [c[order] for c in cols], "len": out["len"]}


def table_rows(eng: Engine, h) -> int:
    n = ctypes.c_int64()
    eng.check(eng.lib.rf_table_num_rows(ctypes.c_void_p(h), ctypes.byref(n)))
    return n.value


def run_alone(eng: Engine, reqs: Sequence[Request], table_sample: Optional[set] = None) -> list:
    """Every request run by itself (rf_plan_run): the reference results of the mixed runs.  A
    value result is kept as its bytes; a table result as its key-sorted export when its index is
    in `table_sample` (None: all), else as its row count."""
    res = []
    for i, r in enumerate(reqs):
        o = new_outs([r])[0]
        args = r.plan.args(*r.inputs)
        eng.check(eng.lib.rf_plan_run(r.plan.h, args, len(r.inputs), ctypes.byref(o), None))
        if not r.plan.info.output_is_table:
            res.append(bytes(o))
        elif table_sample is None or i in table_sample:
            res.append(canonical(eng, r.plan, o.value))
        else:
            res.append(table_rows(eng, o.value))
            DeviceTable(eng, ctypes.c_void_p(o.value), r.plan.fn.output.type, []).free()
    return res


def tables_close(a: Dict, b: Dict, rtol: float = 1e-12) -> bool:
    if a["len"] != b["len"] or len(a["cols"]) != len(b["cols"]):
        return False
    for x, y in zip(a["cols"], b["cols"]):
        if x.dtype.kind == "f":
            if not np.allclose(x, y, rtol=rtol, atol=0.0):
                return False
        elif not np.array_equal(x, y):
            return False
    return True


def compare(eng: Engine, reqs: Sequence[Request], outs: list, alone: list, check_tables: bool = True) -> int:
    """Mismatches of a mixed run against the results alone: value results bit for bit; table
    results key-sorted with FP64 columns within 1e-12 relative (a hash group-by adds each key's
    rows in arrival order at the slot, which varies run to run) where the alone result was kept
    whole, else by row count.  Frees the table results."""
    bad = 0
    for r, o, a in zip(reqs, outs, alone):
        if r.plan.info.output_is_table:
            if not o.value:
                bad += 1
                continue
            if isinstance(a, dict) and check_tables:
                bad += not tables_close(canonical(eng, r.plan, o.value), a)
                continue
            n = table_rows(eng, o.value)
            bad += n != (a["len"] if isinstance(a, dict) else a)
            DeviceTable(eng, ctypes.c_void_p(o.value), r.plan.fn.output.type, []).free()
        else:
            bad += bytes(o) != a
    return bad


def latency_summary(rec: np.ndarray) -> Dict[str, float]:
    ok = rec["status"] == 0
    lat = (rec["t_done_ns"] - rec["t_submit_ns"])[ok] / 1e3
    span = (rec["t_done_ns"].max() - rec["t_submit_ns"].min()) / 1e9 if len(rec) else 0.0
    return {"p50_us": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_us": float(np.percentile(lat, 99)) if len(lat) else None,
            "mean_us": float(lat.mean()) if len(lat) else None,
            "qps": float(ok.sum() / span) if span > 0 else None,
            "failed": int((~ok).sum()),
            "mean_batch": float(rec["batch_queries"][ok].mean()) if ok.any() else None}


def poisson_arrivals(n: int, rate_qps: float, seed: int) -> np.ndarray:
    if not math.isfinite(rate_qps):
        return np.zeros(n, dtype=np.int64)
    gaps = np.random.default_rng(seed).exponential(1e9 / rate_qps, n)
    return np.cumsum(gaps).astype(np.int64)


def serve_run(eng: Engine, wl: Workload, mode: str, rate_qps: float, alone: list, seed: int = 4,
              check_tables: bool = False, **server_kw) -> Dict:
    reqs = wl.requests
    srv = Server(eng, mode=mode, **server_kw)
    try:
        outs = new_outs(reqs)
        rec = srv.replay([r.plan for r in reqs], [r.inputs for r in reqs], outs, poisson_arrivals(len(reqs), rate_qps,
                                                                                                    seed))
        st = srv.stats()
    finally:
        srv.close()
    summ = latency_summary(rec)
    shapes = np.array([r.shape for r in reqs])
    summ["by_shape"] = {SHAPES[k]: latency_summary(rec[shapes == k]) for k in sorted(set(shapes.tolist()))}
    bad = rec["status"] != 0
    summ["failures"] = {"%s:%s" % (SHAPES[k], _capi.STATUS_NAMES.get(int(st), st)): int(c)
                        for (k, st), c in zip(*np.unique(np.stack([shapes[bad], rec["status"][bad]], 1), axis=0,
                                                         return_counts=True))} if bad.any() else {}
    summ["last_error"] = eng.lib.rf_last_error(eng.h).decode(errors="replace")[:200] if bad.any() else ""
    span = (rec["t_done_ns"].max() - rec["t_submit_ns"].min()) / 1e9
    summ["gbps"] = sum(r.nbytes for r in reqs) / span / 1e9 if span > 0 else None
    summ["mismatches"] = compare(eng, reqs, outs, alone, check_tables)
    summ["batches"] = st["batches"]
    summ["max_queue_depth"] = st["max_queue_depth"]
    summ["peak_inflight_bytes"] = st["peak_inflight_bytes"]
    return summ
