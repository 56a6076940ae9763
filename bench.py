#!/usr/bin/env python3
"""Benchmark: compiled Reffine query on one GB300, against Reffine's own code on the host cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--config 1] [--impl ours|reference]

A step is one run of the query over its whole synthetic table.  Default workload: the
low-cardinality group-by (60M rows, 6 groups; --config 1).  Metric: scan
GB/s = algorithmic bytes (each referenced column read once) / time.

  value      kernel throughput with the table resident in HBM (CUDA events on the launch stream)
  e2e        the same metric through the reference-shaped host call (compile_op's function
             pointer: ArrowTable* in, result out), host tables in pinned memory, host->device
             copies of the referenced columns and the device->host result copy inside the timing
  roofline   achieved algorithmic GB/s of the main kernel against the measured HBM copy peak
  cpu_baseline  Reffine's own emitted C++ for the query (oracle/ref/generated, g++ -O3) on the
             same table: one copy per host thread at once (value) and one thread alone; the
             oracle port's one-core figure beside it
  parity     the GPU result against the oracle's on the same full-size tables: integers
             bit-exact, FP64 max relative error (the bar is 1e-12)
  per_config the same measurements (value, roofline, e2e, cpu_baseline, parity) for the other
             three configurations: filter+sum 6M, hash group-by 100M Zipf, join 10M x 200M
  serving    10k requests over resident tables of log-uniform size, Poisson arrivals: the
             continuous-batching server against per-query launches on the same GPU (p50/p99
             latency, queries/s, GB/s), every result checked against the query run alone

--impl reference times Reffine's emitted code alone on every host thread (the reference's CPU
path runs a query serially, so one copy per thread); it counts bytes from the columns each
workload declares and loads nothing of the GPU backend.
Multi-GPU (torchrun): each rank scans its own partition (weak scaling; a join's build side is
the same on every rank), no collective on the data path; rank 0 prints the max-over-ranks time.
After the timed steps each rank's partial state is gathered to rank 0 and folded in rank order
into one answer ("sharded": reffine_gb300.shard).
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import platform
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# a fatal signal in the library's threads prints their native frames (reffine_gb300 crash report)
os.environ.setdefault("RF_CRASH_TRACE", "1")

METRIC = "scan GB/s vs HBM peak per query; batched p99 latency vs per-query launch"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Barrier and max-reduce over ranks (torch.distributed when launched by torchrun)."""

    def __init__(self, world: int):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def gather(self, obj):
        """Every rank's object on rank 0, in rank order (None elsewhere)."""
        if self.world == 1:
            return [obj]
        out = [None] * self.world if self.td.get_rank() == 0 else None
        self.td.gather_object(obj, out, dst=0)
        return out

    def sum(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())


def peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            d = json.load(open(p))
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.out = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        sms, maxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for row in csv.reader(io.StringIO(out)):
            if len(row) < 9:
                continue
            try:
                sms.append(float(row[1]))
                maxs.append(float(row[2]))
            except ValueError:
                continue
            for n, v in zip(names, row[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sms)) if sms else None, "sm_max_mhz": max(maxs) if maxs else None,
                "reasons": sorted(reasons), "samples": len(sms)}


class Workload:
    """One benchmark configuration: seeded tables, the query, and the columns it reads (declared
    here, so the CPU arm counts algorithmic bytes without the GPU library)."""

    def __init__(self, name, tables, fn, rows, cfg, cols):
        self.name, self.tables, self.fn, self.rows, self.cfg, self.cols = name, tables, fn, rows, cfg, cols

    def algorithmic_bytes(self) -> int:
        return sum(t.nbytes(c) for t, c in zip(self.tables, self.cols))


WORKLOAD_NAMES = {0: "filter_sum_6M", 1: "groupby_6groups_60M", 2: "hash_groupby_zipf1.1_100M", 3: "join_10M_x_200M"}


def build_workload(config: int, rank: int, world: int, rows: int = 0) -> Workload:
    """Each rank gets its own partition (a different seed), so per-GPU work is fixed as N grows."""
    from reffine_gb300 import workloads as W
    seed_off = 1000 * rank
    name = WORKLOAD_NAMES.get(config)
    if config == 0:
        n = rows or 6_000_000
        t = W.filter_sum_table(n, seed=0 + seed_off)
        return Workload(name, [t], W.filter_sum_query(t.get_data_type()), n, build_cfg(0, n), [[1, 2, 3, 4]])
    if config == 1:
        n = rows or 60_000_000
        t = W.groupby_table(n, seed=1 + seed_off)
        return Workload(name, [t], W.groupby_query(t.get_data_type()), n, build_cfg(1, n), [[1, 2, 3, 4, 5, 6, 7]])
    if config == 2:
        n, nd = rows or 100_000_000, 10_000_000
        t = W.hashgroup_table(n, min(nd, n), 1.1, seed=2 + seed_off)
        return Workload(name, [t], W.hashgroup_query(t.get_data_type()), n, build_cfg(2, n), [[0, 1]])
    if config == 3:
        nb, npr = 10_000_000, rows or 200_000_000
        # every rank holds the same build side; probe rows are the rank's own partition
        b, p = W.join_tables(nb, npr, seed=3, probe_seed=None if world == 1 else 3 + seed_off)
        return Workload(name, [b, p], W.join_query(b.get_data_type(), p.get_data_type()), npr, build_cfg(3, npr),
                        [[0, 1], [1, 2, 3]])
    raise SystemExit("config %d is not benchmarked by this script" % config)


L2_NOTE = "inputs larger than L2 (129 MB); no flush between steps"


def reference_form(config, fn, tables):
    """The query and tables in the form the reference runs: the high-cardinality group-by needs
    its keys sorted and run-end encoded (a grouped 2-d vector); the sort is not timed."""
    if config != 2:
        return fn, tables
    from reffine_gb300 import workloads as W
    ree = W.ree_sorted(tables[0])
    return W.hashgroup_query(ree.get_data_type()), [ree]


GENERATED = {0: "filter_sum", 1: "groupby", 2: "hashgroup_ree", 3: "join_agg"}


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def reffine_code(config, fn, tables):
    """Reffine's own emitted C++ for this workload's query (oracle/ref/generated, compiled with
    g++ -O3 and the compiler's default contraction), its tables prepared (Locate indexes built)."""
    from oracle import ref_generated
    q = ref_generated.GeneratedQuery(GENERATED[config], fn)
    q.prepare(*tables)
    return q


def reffine_code_sample(config, fn, tables, target_s):
    """Reffine's emitted code prepared on a bounded sample of the workload: the driving (last)
    table cut to a row prefix whose one-thread run takes about target_s seconds, or whole when it
    takes less (a run-end table is always whole).  (query, fraction of rows, one-thread seconds,
    one-thread result.)"""
    d = tables[-1]
    q = None
    if len(d) >= 64 and all(c.run_ends is None for c in d.columns):
        probe = len(d) // 64
        q = reffine_code(config, fn, tables[:-1] + [d.rows(0, probe)])
        t_small, _ = q.run(1)
        est = t_small * len(d) / probe
        if est > target_s:
            n = max(probe, int(len(d) * target_s / est))
            q.prepare(*(tables[:-1] + [d.rows(0, n)]))
            t1, r1 = q.run(1)
            return q, n / len(d), t1, r1[0]
        q.prepare(*tables)
    if q is None:
        q = reffine_code(config, fn, tables)
    t1, r1 = q.run(1)
    return q, 1.0, t1, r1[0]


def reffine_code_run(config, fn, tables, nbytes, note="", target_s=4.0):
    """Reffine's emitted code on the host cores: one query on one thread (Reffine runs a query
    serially), then one copy of the query on every host thread at once, on a bounded sample.
    (cpu_baseline dict, the one-thread result on the whole table or None for a sample.)"""
    q, frac, t1, r1 = reffine_code_sample(config, fn, tables, target_s)
    nthr = host_threads()
    tn, rn = q.run(nthr)
    q.release()
    agree = all(repr(r) == repr(r1) for r in rn) if not isinstance(r1, dict) else \
        all(r["len"] == r1["len"] for r in rn)
    kind = platform.processor() or platform.machine()
    b = nbytes * frac
    what = "the full table" if frac == 1.0 else "the first %.2f%% of the driving table's rows" % (100 * frac)
    base = {"value": nthr * b / tn / 1e9, "unit": "GB/s", "cores": nthr, "kind": "reference",
            "sample": "Reffine's emitted code for the query (LoopGen..CEmitter output, g++ -O3) on %s: %d copies "
                      "at once, one per host thread, %.3f s; %s%s" % (what, nthr, tn, kind, note),
            "single_thread": {"value": b / t1 / 1e9, "seconds": t1},
            "threads_agree": agree}
    return base, (r1 if frac == 1.0 else None)


def oracle_run(fn, tables, nbytes, budget_s=20.0, note=""):
    """The oracle port (Reffine's serial loop restated, g++ -O3, one core) on the same tables:
    (cpu_baseline dict, seconds per run, the result of the first run)."""
    from oracle import loopgen
    q = loopgen.Query(fn)
    table_out = fn.output.type.is_vector()
    times, result = [], None
    t_end = time.perf_counter() + budget_s
    while len(times) < 5 and (not times or time.perf_counter() + times[-1] < t_end):
        out, cargs = q.prepare(*tables)
        t0 = time.perf_counter()
        q.run_prepared(out, cargs)
        times.append(time.perf_counter() - t0)
        r = q.result(out)  # frees a table result's buffers
        if result is None:
            result = r
    sec = float(np.median(times))
    kind = platform.processor() or platform.machine()
    return ({"value": nbytes / sec / 1e9, "unit": "GB/s", "cores": 1, "kind": "port",
             "sample": "the full table, %d run(s), median %.3f s; %s%s" % (len(times), sec, kind, note)},
            sec, result)


def _flatten(v):
    if isinstance(v, (tuple, list)):
        for x in v:
            yield from _flatten(x)
    else:
        yield v


def value_parity(got, ref) -> dict:
    """Integers bit-exact, FP64 relative error against the oracle (1e-12 is the bar)."""
    import math
    g, r = list(_flatten(got)), list(_flatten(ref))
    if len(g) != len(r):
        return {"int_exact": False, "max_rel_err": None, "fields": [len(g), len(r)], "ok": False}
    int_ok, rel = True, 0.0
    for a, b in zip(g, r):
        if isinstance(b, float):
            if math.isnan(b) or math.isinf(b):
                same = (math.isnan(a) and math.isnan(b)) or a == b
                rel = rel if same else math.inf
            else:
                rel = max(rel, abs(a - b) / max(abs(b), 1e-300))
        else:
            int_ok &= a == b
    return {"int_exact": bool(int_ok), "max_rel_err": rel, "fields": len(r), "ok": bool(int_ok and rel <= 1e-12)}


def table_parity(out, ref, values=None, keys=None) -> dict:
    """A table result against the oracle's: rows canonicalised by column 0 (the key); integer
    columns bit-exact, FP64 columns by relative error.  With the input key/value columns given,
    also the distance of both sums from exact sums (math.fsum) for the 8 largest groups."""
    import math
    order = np.argsort(out["cols"][0], kind="stable")
    cols = [c[order] for c in out["cols"]]
    res = {"rows": int(out["len"]), "oracle_rows": int(ref["len"])}
    if out["len"] != ref["len"]:
        res.update(int_exact=False, max_rel_err=None, ok=False)
        return res
    int_ok, rel = True, 0.0
    for g, r in zip(cols, ref["cols"]):
        if np.issubdtype(r.dtype, np.floating):
            den = np.maximum(np.abs(r), 1e-300)
            rel = max(rel, float(np.max(np.abs(g - r) / den)) if len(r) else 0.0)
        else:
            int_ok &= bool(np.array_equal(g, r))
    res.update(int_exact=int_ok, max_rel_err=rel, ok=bool(int_ok and rel <= 1e-12))
    if keys is not None and len(ref["cols"]) >= 3 and len(ref["cols"][2]):
        top = np.argsort(ref["cols"][2])[-8:]
        worst_gpu = worst_cpu = 0.0
        for i in top:
            k = ref["cols"][0][i]
            exact = math.fsum(values[keys == k].tolist())
            if exact:
                worst_gpu = max(worst_gpu, abs(cols[1][i] - exact) / abs(exact))
                worst_cpu = max(worst_cpu, abs(ref["cols"][1][i] - exact) / abs(exact))
        res["largest_groups_vs_exact_sum"] = {"groups": len(top), "rows_in_largest": int(ref["cols"][2][top[-1]]),
                                              "gpu_max_rel_err": worst_gpu, "oracle_max_rel_err": worst_cpu}
    return res


def run_reference(args, rank, world):
    """The reference's CPU path for the same workload: the C++ Reffine's own compile path emits
    for the query (oracle/ref/generated; g++ -O3), on every host thread.  Reffine runs one query
    serially, so a step runs one copy of the whole query per host thread at once and the value is
    the bytes all copies scanned over the step's wall time; the single-thread figure is reported
    beside it.  Counts bytes from the workload's declared columns; loads nothing of the GPU
    backend."""
    if rank != 0:
        return 0
    wl = build_workload(args.config, 0, 1, args.rows)
    nbytes = wl.algorithmic_bytes()
    fn, tables = reference_form(args.config, wl.fn, wl.tables)
    # each step a bounded sample: the driving table's first rows, about 2 s of one thread's work
    q, frac, t1, _ = reffine_code_sample(args.config, fn, tables, 2.0)
    nthr = host_threads()
    for _ in range(args.warmup):
        q.run(nthr)
    times = [q.run(nthr)[0] for _ in range(args.steps)]
    q.release()
    sec = float(np.mean(times))
    nbytes = nbytes * frac
    val = nthr * nbytes / sec / 1e9
    what = "the whole table" if frac == 1.0 else "the first %.2f%% of the driving table's rows" % (100 * frac)
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "GB/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": wl.name, **wl.cfg, "l2": L2_NOTE},
            "cpu_baseline": {"value": val, "unit": "GB/s", "cores": nthr, "kind": "reference",
                             "sample": "per step, one copy of the query over %s per host thread at once (%d), "
                                       "Reffine's emitted code compiled with g++ -O3" % (what, nthr),
                             "single_thread": {"value": nbytes / t1 / 1e9, "seconds": t1}},
            "e2e": {"value": val, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "algorithmic_bytes_per_step": nbytes}
    print(json.dumps(line), flush=True)
    return 0


def _pinned_copy(eng, tables):
    from reffine_gb300.table import Column, Table
    pinned, ptables = [], []
    for t in tables:
        cols = []
        for c in t.columns:
            buf = eng.host_alloc(c.data.nbytes)
            v = buf.view(c.data.dtype, len(c.data))
            v[:] = c.data
            pinned.append(buf)
            cols.append(Column(c.name, c.dtype, v, c.valid, c.run_ends))
        ptables.append(Table(t.name, t.dim, cols))
    return pinned, ptables


def measure_config(eng, wl: Workload, config: int, args, rank: int, world: int, dist, cpu: bool,
                   pageable: bool = True) -> dict:
    """Times one workload: kernel throughput (tables resident, CUDA events on the launch stream),
    the roofline of its main kernel, end to end through the reference-shaped host call, the CPU
    baseline and full-size parity against the oracle."""
    from reffine_gb300 import cudart, engine
    dts = [eng.upload(t) for t in wl.tables]
    plan = eng.compile(wl.fn)
    nbytes = sum(int(plan.info.bytes_per_row[i]) * len(t) for i, t in enumerate(wl.tables))
    declared = wl.algorithmic_bytes()
    pargs = plan.args(*dts)
    n = len(dts)
    stream = eng.stream
    table_out = bool(plan.info.output_is_table)
    out_rows = [0]
    last = [None]
    tuning = {}
    # the autotuner picks the block size and scan tile (or the hash table's sizing) for this
    # shape and size once, before warm-up (rf_plan_tune; every later run of the shape uses it)
    if args.tune_file:
        tuning["from_file"] = args.tune_file
    elif not table_out and plan.kind in (1, 2):
        tuning["tile_rows"], _ = plan.tune(*dts, reps=3)
        tuning["block"] = next((m for m in (128, 256, 512) if "_KERNEL(rf_main, %d)" % m in plan.source), None)
    elif plan.kind == 5:
        tuning["hash_slots_per_100_keys"], _ = plan.tune(*dts, reps=2)
    if args.save_tune:
        eng.tune_save(args.save_tune)

    def step(keep=False):
        if not table_out:
            plan.launch(pargs, n)
            return
        import ctypes
        h = ctypes.c_void_p()
        eng.check(eng.lib.rf_plan_run(plan.h, pargs, n, ctypes.byref(h), None))
        r = ctypes.c_int64()
        eng.lib.rf_table_num_rows(h, ctypes.byref(r))
        out_rows[0] = r.value
        if keep:
            dtab = engine.DeviceTable(eng, h, None, [])
            last[0] = dtab.export()
            dtab.h = None  # freed below
        eng.lib.rf_table_free(h)

    for _ in range(max(args.warmup, 3)):
        step()
    eng.sync()
    out_bytes = 0
    if table_out:  # output bytes join the algorithmic bytes (rows x output row size)
        out_bytes = out_rows[0] * sum(d.size() for d in wl.fn.output.type.dtypes)
        nbytes += out_bytes
        declared += out_bytes

    evs = [cudart.Event() for _ in range(args.steps + 1)]
    clocks = ClockSampler(eng.device)
    clocks.start()
    dist.barrier()
    eng.sync()
    l0 = eng.launch_count()
    evs[0].record(stream)
    for k in range(args.steps):
        step()
        evs[k + 1].record(stream)
    eng.sync()
    dist.barrier()
    l1 = eng.launch_count()
    clk = clocks.stop()
    per = [evs[k].elapsed_ms(evs[k + 1]) for k in range(args.steps)]
    total_ms = dist.max(sum(per))
    ms_step = total_ms / args.steps
    all_bytes = dist.sum(nbytes)
    value = all_bytes / (ms_step / 1e3) / 1e9

    # the result (outside the timing), for parity
    if table_out:
        step(keep=True)
        got = last[0]
    else:
        out = plan.new_out()
        plan.run_args(pargs, n, out)
        got = engine.from_c(out)

    peak, peak_kind = peak_hbm()
    kern_ms = float(np.mean(per))
    achieved = nbytes / (kern_ms / 1e3) / 1e9
    traffic = None
    tf = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tf):
        try:
            traffic = json.load(open(tf)).get(wl.name)
        except Exception:
            traffic = None

    # end to end through the reference-shaped call (compile_op's function pointer): host
    # tables in pinned memory, host->device copies of the referenced columns and the result's
    # copy back inside the timing
    h2d = sum(int(plan.info.bytes_per_row[i]) * len(t) for i, t in enumerate(wl.tables))
    d2h = out_bytes if table_out else int(plan.info.output_size)
    e2e = {"value": None, "unit": "GB/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}
    pinned = []
    try:
        if args.e2e_steps <= 0:
            raise RuntimeError("e2e skipped (--e2e-steps 0)")
        pinned, ptables = _pinned_copy(eng, wl.tables)
        q = engine.compile_op(wl.fn, engine=eng)
        q(*ptables)
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            q(*ptables)
        e2e_s = dist.max(time.perf_counter() - t0) / args.e2e_steps
        e2e.update(value=all_bytes / e2e_s / 1e9, ms_per_step=e2e_s * 1e3,
                   path="compile_op function pointer (rf_plan_thunk), pinned host tables" +
                        ("; the result table exported to host Arrow memory" if table_out else ""))
        if pageable and not table_out:
            # the same call on the tables' own (pageable, numpy) memory, as a caller's ArrowTable2
            # holds it
            q(*wl.tables)
            dist.barrier()
            t0 = time.perf_counter()
            for _ in range(args.e2e_steps):
                q(*wl.tables)
            pg_s = dist.max(time.perf_counter() - t0) / args.e2e_steps
            e2e["pageable"] = {"value": all_bytes / pg_s / 1e9, "ms_per_step": pg_s * 1e3}
        q.plan.free()
        del ptables
    except Exception as ex:  # report, do not hide
        e2e["error"] = str(ex)[:300]
    finally:
        for b in pinned:
            b.free()

    res = {"workload": wl.name, "value": value, "unit": "GB/s", "ms_per_step": ms_step, "steps": args.steps,
           "warmup": max(args.warmup, 3), "rows_per_s": wl.rows * world / (ms_step / 1e3),
           "bytes_per_step": nbytes, "tuning": tuning or None,
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                        "kernel": {1: "rf_main (scan-reduce)", 2: "rf_main (grouped scan-reduce)",
                                   5: "rf_hg_agg + materialisation (hash group-by)"}.get(plan.kind, str(plan.kind)),
                        "algorithmic_bytes_per_launch": nbytes},
           "e2e": e2e, "gpu_launches": int(l1 - l0), "clocks": clk}
    if nbytes != declared:
        res["bytes_mismatch"] = {"plan": nbytes, "declared": declared}

    if cpu and rank == 0:
        rfn, rtabs = reference_form(config, wl.fn, wl.tables)
        note = "" if config != 2 else \
            "; keys pre-sorted and run-end encoded (the reference's grouped form), sort not timed"
        port, _, ref = oracle_run(rfn, rtabs, nbytes, note=note)
        base, rcode = reffine_code_run(config, rfn, rtabs, nbytes, note=note)
        base["oracle_port"] = {"value": port["value"], "cores": 1}
        res["cpu_baseline"] = base
        if table_out:
            kw = dict(values=wl.tables[0].columns[1].data, keys=wl.tables[0].columns[0].data)
            res["parity"] = table_parity(got, ref, **kw)
        else:
            res["parity"] = value_parity(got, ref)
        res["parity"]["against"] = "oracle on the same full-size tables (rows %d)" % wl.rows
        if rcode is not None:
            res["parity_reffine_code"] = table_parity(got, rcode) if table_out else value_parity(got, rcode)
            res["parity_reffine_code"]["against"] = "Reffine's emitted code on the same tables (default contraction)"
    else:
        res["cpu_baseline"] = None
        res["parity"] = None
    res["result_sample"] = ("%d output rows" % out_rows[0]) if table_out else str(got)[:200]
    if world > 1:
        res["sharded"] = shard_fold(eng, wl, dts, got, dist, rank, world)
    for d in dts:
        d.free()
    plan.free()
    return res


def shard_fold(eng, wl: Workload, dts, got, dist, rank: int, world: int) -> dict:
    """One answer over all ranks' partitions (after the timed steps): each rank's partial Reduce
    state (or partial grouped table) from its GPU, gathered to rank 0 and folded in rank order
    (reffine_gb300.shard)."""
    from reffine_gb300 import shard
    t0 = time.perf_counter()
    if isinstance(got, dict):
        part = {"cols": got["cols"], "len": got["len"]}
    else:
        state_fn, _ = shard.split_reduce(wl.fn)
        sp = eng.compile(state_fn)
        part = sp.run(*dts)
        sp.free()
    parts = dist.gather(part)
    if rank != 0:
        return None
    if isinstance(got, dict):
        folded = shard.fold_tables(parts, ["sum"] * (len(part["cols"]) - 1))
        sample = "%d groups" % folded["len"]
    else:
        _, finish = shard.split_reduce(wl.fn)
        folded = finish(shard.fold_states(parts, shard.leaf_ops(wl.fn)))
        sample = str(folded)[:200]
    return {"ranks": world, "rows_total": wl.rows * world, "fold_ms": (time.perf_counter() - t0) * 1e3,
            "partition": "each rank its own seeded row range; partial states folded on rank 0 in rank order",
            "result_sample": sample}


def bench_serving(eng, n_queries: int, max_rows: int, rates=(0.5, 0.8, 1.0, 1.5), table_lanes: int = 0,
                  table_priority: int = 0):
    """Batched serving over resident tables (10k mixed requests): the same Poisson request stream through
    the continuous-batching server and through per-query launches (one rf_plan_run per request,
    in arrival order) on the same GPU.  Rates are fractions of the per-query path's closed-loop
    capacity.  Every result is compared with the query run alone."""
    import math
    from reffine_gb300 import serve
    t0 = time.perf_counter()
    wl = serve.build_workload(eng, n_queries=n_queries, max_rows=max_rows)
    t_build = time.perf_counter() - t0
    tab = [i for i, r in enumerate(wl.requests) if r.plan.info.output_is_table]
    sample = set(tab[:: max(1, len(tab) // 40)])  # ~40 table results compared in full, all by row count
    alone = serve.run_alone(eng, wl.requests, sample)
    keep = ("qps", "gbps", "p50_us", "p99_us", "mean_us", "mean_batch", "failed", "mismatches", "failures")
    r3 = lambda v: round(v, 1) if isinstance(v, float) else v
    slim = lambda d: dict({k: (round(d[k], 3) if isinstance(d[k], float) else d[k]) for k in keep},
                          by_shape={k: [r3(v["p50_us"]), r3(v["p99_us"])] for k, v in d["by_shape"].items()})
    kw = {"batched": {"table_lanes": table_lanes, "table_priority": table_priority}, "per_query": {}}
    out = {"queries": len(wl.requests),
           "shapes": dict(zip(serve.SHAPES, np.bincount([r.shape for r in wl.requests], minlength=4).tolist())),
           "table_rows": "log-uniform in [1e3, %.0e], 6 tables per shape, resident" % max_rows,
           "resident_gb": round(wl.resident_bytes / 1e9, 2),
           "bytes_per_query_mb": round(sum(r.nbytes for r in wl.requests) / len(wl.requests) / 1e6, 2),
           "server": "2 lanes x 256 queries per launch, %d table lane(s) at %s stream priority, 8 GiB scratch "
                     "budget" % (max(table_lanes, 1), "normal" if table_priority < 0 else "high"),
           "by_shape": "[p50_us, p99_us] per query shape",
           "workload_build_s": round(t_build, 1),
           "check": "value results bit for bit; table results by row count, %d of them key-sorted in full "
                    "(FP64 within 1e-12)" % len(sample),
           "tile_rows_tuned": wl.tuning}
    closed = {}
    for mode in ("per_query", "batched"):
        closed[mode] = slim(serve.serve_run(eng, wl, mode, math.inf, alone, check_tables=True, **kw[mode]))
    out["closed_loop"] = closed
    cap = closed["per_query"]["qps"]
    sweep = []
    for f in rates:
        row = {"rate_qps": round(cap * f, 1), "of_per_query_capacity": f}
        for mode in ("per_query", "batched"):
            row[mode] = slim(serve.serve_run(eng, wl, mode, cap * f, alone, seed=40 + int(f * 10), **kw[mode]))
        sweep.append(row)
    out["poisson"] = sweep
    runs = [closed[m] for m in closed] + [r[m] for r in sweep for m in ("per_query", "batched")]
    out["identical_to_alone"] = all(r["mismatches"] == 0 and r["failed"] == 0 for r in runs)
    return out


def serving_in_child(n_queries: int, max_rows: int, device: int, table_lanes: int = 0, table_priority: int = 0,
                     timeout_s: int = 900):
    """bench_serving in a child process on the same GPU: its server threads and CUDA graphs
    live and end there, and this process prints its line whatever becomes of the child."""
    env = dict(os.environ, LOCAL_RANK=str(device), RANK="0", WORLD_SIZE="1")
    cmd = [sys.executable, os.path.abspath(__file__), "--serving-only", "--serving-queries", str(n_queries),
           "--serving-max-rows", str(max_rows), "--serving-table-lanes", str(table_lanes),
           "--serving-table-priority", str(table_priority)]
    try:
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout_s, env=env, cwd=ROOT)
    except subprocess.TimeoutExpired:
        return {"error": "serving run exceeded %d s" % timeout_s}
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    if r.returncode == 0 and lines:
        try:
            return json.loads(lines[-1])
        except ValueError:
            pass
    return {"error": "serving child exited with %d: %s" % (r.returncode, (r.stderr or "")[-600:])}


def bench_ingest(eng, config: int, rows: int = 0, reps: int = 3):
    """Arrow IPC ingest (load_arrow_file, src/utils/utils.cpp:11-34): the config's table written
    as an IPC file (the page cache holds it after the write; disk speed is not measured), then
    host_read: rf_ipc_read, file -> host Arrow C data (what the reference's load does, CPU only);
    load: rf_table_load_ipc, file -> HBM (on a Grace host: DMA straight out of the mapped file);
    load_staged: the same through the pinned staging ring (the path for hosts whose GPU cannot
    read pageable memory);
    read_then_upload: rf_ipc_read, then rf_table_upload from its pageable memory.
    The config's query runs on the loaded table and on an upload of the in-memory table: both
    results must have the same bits."""
    import ctypes
    import shutil
    import tempfile
    from reffine_gb300.ipc_write import write_ipc
    from reffine_gb300.table import read_ipc_c, release_c
    wl = build_workload(config, 0, 1, rows)
    name, tables, fn, nrows = wl.name, wl.tables, wl.fn, wl.rows
    if len(tables) != 1:
        raise ValueError("ingest is measured on single-table configurations (0, 1, 2)")
    t = tables[0]
    d = tempfile.mkdtemp(prefix="rf_ingest_")
    try:
        path = os.path.join(d, name + ".arrow")
        t0 = time.perf_counter()
        size = write_ipc(path, t)
        t_write = time.perf_counter() - t0

        def host_read():
            s, a = read_ipc_c(path)
            release_c(s, a)

        def load():
            eng.load_ipc(path, t.dim).free()
            eng.sync()

        def load_staged():
            os.environ["RF_IPC_LOAD"] = "staged"
            try:
                load()
            finally:
                del os.environ["RF_IPC_LOAD"]

        def read_then_upload():
            s, a = read_ipc_c(path)
            try:
                h = ctypes.c_void_p()
                eng.check(eng.lib.rf_table_upload(eng.h, ctypes.byref(s), ctypes.byref(a), t.dim, None, ctypes.byref(h)))
                eng.sync()
                eng.lib.rf_table_free(h)
            finally:
                release_c(s, a)

        res = {}
        for nm, f in (("host_read", host_read), ("load", load), ("load_staged", load_staged),
                      ("read_then_upload", read_then_upload)):
            f()  # first run: allocations, staging ring, page cache settled
            ts = []
            for _ in range(reps):
                t0 = time.perf_counter()
                f()
                ts.append(time.perf_counter() - t0)
            res[nm] = {"gbps": round(size / min(ts) / 1e9, 2), "ms_best": round(min(ts) * 1e3, 2),
                       "ms_median": round(float(np.median(ts)) * 1e3, 2)}
        loaded = eng.load_ipc(path, t.dim)
        plan = eng.compile(fn)
        same = plan.run(loaded) == plan.run(eng.upload(t))
        loaded.free()
    finally:
        shutil.rmtree(d, ignore_errors=True)
    return {"metric": "arrow_ipc_ingest", "unit": "GB/s (file bytes / wall time, best of %d)" % reps,
            "workload": name, "rows": nrows, "file_bytes": size, "write_s": round(t_write, 2),
            "page_cache": "warm (file just written)", "host_threads": os.cpu_count(),
            **res, "load_vs_host_read": round(res["host_read"]["ms_best"] / res["load"]["ms_best"], 2),
            "query_result_identical": bool(same)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--config", type=int, default=1)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--rows", type=int, default=0, help="override the row count (profiling a smaller case)")
    ap.add_argument("--per-config", default="auto",
                    help="comma-separated further configurations measured after the headline one and reported "
                         "under per_config ('auto': the other three of 0-3 when the headline is config 1 at "
                         "full size on one GPU; 'none')")
    ap.add_argument("--serving-queries", type=int, default=10_000,
                    help="requests of the batched-serving comparison (0: skip it)")
    ap.add_argument("--serving-max-rows", type=int, default=50_000_000)
    ap.add_argument("--serving-table-lanes", type=int, default=0,
                    help="table-result queries the batched server runs at once (0: the server's default)")
    ap.add_argument("--serving-table-priority", type=int, default=0,
                    help="the batched server's table lanes: >= 0 highest stream priority (default), < 0 normal")
    ap.add_argument("--save-tune", default="",
                    help="write the autotuner's choices to this JSON file after tuning")
    ap.add_argument("--tune-file", default="",
                    help="take the autotuner's choices from this JSON file instead of tuning (profiling runs)")
    ap.add_argument("--tune-as-rows", type=int, default=0,
                    help="with --tune-file: apply the file's tilings to tables of this many rows too (a "
                         "smaller profiling case run with the full-size configuration)")
    ap.add_argument("--ingest", action="store_true",
                    help="measure Arrow IPC ingest of the config's table instead (one JSON line)")
    ap.add_argument("--serving-only", action="store_true",
                    help="run the serving comparison alone and print its JSON object (the child process of a "
                         "default run)")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.serving_only:
        from reffine_gb300 import engine
        eng = engine.Engine(local)
        print(json.dumps(bench_serving(eng, args.serving_queries, args.serving_max_rows,
                                       table_lanes=args.serving_table_lanes,
                                       table_priority=args.serving_table_priority)), flush=True)
        eng.close()
        return 0
    if args.ingest:
        from reffine_gb300 import engine
        eng = engine.Engine(local)
        print(json.dumps(bench_ingest(eng, args.config, args.rows)), flush=True)
        eng.close()
        return 0

    from reffine_gb300 import engine
    dist = Dist(world)
    eng = engine.Engine(local)
    if args.tune_file:
        path = args.tune_file
        if args.tune_as_rows > 0:
            # each tiling entry (bucket >= 0: the size class floor(log2(rows))) copied to the
            # bucket of the given row count; the block sizes (bucket -1) hold for every size
            with open(path) as f:
                tune = json.load(f)
            b = max(0, args.tune_as_rows.bit_length() - 1)
            tune["entries"] += [dict(e, bucket=b) for e in tune["entries"] if e["bucket"] >= 0]
            path = path + ".as%d.json" % args.tune_as_rows
            with open(path, "w") as f:
                json.dump(tune, f)
        eng.tune_load(path)  # compiles below take the file's block sizes and tilings
    wl = build_workload(args.config, rank, world, args.rows)
    head = measure_config(eng, wl, args.config, args, rank, world, dist, cpu=not args.no_cpu)
    del wl

    if args.per_config == "auto":
        others = [c for c in (0, 1, 2, 3) if c != args.config] if (args.config == 1 and not args.rows and world == 1) \
            else []
    elif args.per_config in ("", "none"):
        others = []
    else:
        others = [int(c) for c in args.per_config.split(",") if c.strip() and int(c) != args.config]
    per_config = {}
    for c in others:
        try:
            w = build_workload(c, rank, world, 0)
            per_config[WORKLOAD_NAMES[c]] = measure_config(eng, w, c, args, rank, world, dist, cpu=not args.no_cpu,
                                                           pageable=False)
            del w
        except Exception as ex:  # one configuration's failure is reported, not fatal to the line
            per_config[WORKLOAD_NAMES.get(c, str(c))] = {"error": "%s: %s" % (type(ex).__name__, str(ex)[:400])}

    serving = None
    if rank == 0 and args.serving_queries > 0 and world == 1:
        serving = serving_in_child(args.serving_queries, args.serving_max_rows, local, args.serving_table_lanes,
                                   args.serving_table_priority)

    if rank == 0:
        line = {"metric": METRIC, "value": head["value"], "unit": "GB/s", "n_gpus": world, "steps": args.steps,
                "warmup": max(args.warmup, 3), "ms_per_step": head["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": head["workload"], **build_cfg(args.config, args.rows), "l2": L2_NOTE},
                "tuning": dict(head["tuning"] or {}, source="autotuner (rf_plan_tune) before warm-up"),
                "bytes_per_step": head["bytes_per_step"], "rows_per_s": head["rows_per_s"],
                "roofline": head["roofline"], "cpu_baseline": head["cpu_baseline"], "e2e": head["e2e"],
                "parity": head["parity"], "parity_reffine_code": head.get("parity_reffine_code"),
                "gpu_launches": head["gpu_launches"], "clocks": head["clocks"],
                "per_config": per_config or None, "serving": serving, "result_sample": head["result_sample"]}
        if "bytes_mismatch" in head:
            line["bytes_mismatch"] = head["bytes_mismatch"]
        print(json.dumps(line), flush=True)
    eng.close()
    return 0


def build_cfg(config: int, rows: int) -> dict:
    """The config dict of a workload without building its tables (both arms print the same)."""
    cfgs = {0: lambda n: {"rows": n, "query": "SUM(price*discount), COUNT over day in [730,1095), discount in "
                                               "[0.05,0.07], quantity < 24"},
            1: lambda n: {"rows": n, "groups": 6, "query": "per (flag_a, flag_b): SUM qty/price/disc_price/charge, "
                                                           "AVG qty/price/disc, COUNT over day <= 2450"},
            2: lambda n: {"rows": n, "distinct_ranks": min(10_000_000, n), "zipf_s": 1.1,
                          "query": "per key: SUM(value) f64, COUNT i64 (unsorted int64 keys; hash table at load 0.5)"},
            3: lambda n: {"rows": n, "build_rows": 10_000_000,
                          "query": "SUM(amount), COUNT per build attr < 5, probe day in [0,365)"}}
    default = {0: 6_000_000, 1: 60_000_000, 2: 100_000_000, 3: 200_000_000}
    return cfgs[config](rows or default[config])


if __name__ == "__main__":
    sys.exit(main())
