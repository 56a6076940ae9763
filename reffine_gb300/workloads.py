"""Benchmark workloads: seeded synthetic tables and the Reffine queries run over them.

Shapes follow the five benchmark configurations of this backend (filter+sum, low-cardinality
group-by, high-cardinality group-by, filtered join+aggregate, batched serving).  The queries are
written with the Reffine builder the way the reference's TPC-H queries are
(benchmark/include/tpch.h: Q6 at :160-216 is the filter+sum pattern, Q1 at :398-486 the
select-per-group aggregation, Q3 at :8-81 the Locate probe).  Data is synthetic: seeded numpy
generators with the value distributions of each configuration; no benchmark-suite data is used.
"""
from __future__ import annotations

from typing import Dict, Tuple

import numpy as np

from . import ir
from .ir import (_add, _and, _cast, _div, _eq, _f64, _func, _get, _gte, _i32, _i64, _i8, _idx, _len, _locate,
                 _lt, _lte, _mul, _new, _readdata, _red, _sel, _sub, _subvec, _sym)
from .table import Table

# ----------------------------------------------------------------------------- filter + sum
Q0_DAY_LO, Q0_DAY_HI, Q0_DISC_LO, Q0_DISC_HI, Q0_QTY = 730, 1095, 0.05, 0.07, 24.0


def filter_sum_table(n: int = 6_000_000, seed: int = 0) -> Table:
    """6M rows: key i64 (iterator column, not read), day i32 in [0,2557), price f64 in
    [900,105000), discount f64 = k/100 for k in [0,11) (so 0.05/0.07 equal the literals), quantity
    f64 integers 1..50.  dim 2, as the reference loads lineitem for Q6 (tpch.h:168)."""
    rng = np.random.default_rng(seed)
    day = rng.integers(0, 2557, n, dtype=np.int32)
    price = rng.uniform(900.0, 105000.0, n)
    disc = rng.integers(0, 11, n).astype(np.float64) / 100.0
    qty = rng.integers(1, 51, n).astype(np.float64)
    return Table.from_arrays(2, {"key": np.arange(n, dtype=np.int64), "day": day, "price": price,
                                 "discount": disc, "quantity": qty}, name="filter_sum")


def filter_sum_query(tbl_type: ir.DataType, day_lo=Q0_DAY_LO, day_hi=Q0_DAY_HI, disc_lo=Q0_DISC_LO,
                     disc_hi=Q0_DISC_HI, qty=Q0_QTY) -> ir.Func:
    """SUM(price*discount), COUNT(*) over rows with day in [lo, hi), discount in [dlo, dhi],
    quantity < qty: the Reduce-over-SubVector of TPC-H Q6 (tpch.h:174-208) plus a count."""
    vec = _sym("lineitem", tbl_type)

    def acc(s, v):
        day, price, disc, q = _get(v, 0), _get(v, 1), _get(v, 2), _get(v, 3)
        pred = (_gte(day, _i32(day_lo)) & _lt(day, _i32(day_hi)) & _gte(disc, _f64(disc_lo)) &
                _lte(disc, _f64(disc_hi)) & _lt(q, _f64(qty)))
        return _new([_sel(pred, _add(_get(s, 0), _mul(price, disc)), _get(s, 0)),
                     _sel(pred, _add(_get(s, 1), _i64(1)), _get(s, 1))])

    red = _red(_subvec(vec, _idx(0), _len(vec, 1)), lambda: _new([_f64(0), _i64(0)]), acc)
    red_sym = _sym("red", red)
    fn = _func("filter_sum", red_sym, [vec])
    fn.tbl[red_sym] = red
    return fn


# ----------------------------------------------------------------------------- low-card group-by
Q1_DAY = 2450
FLAG_A, FLAG_B = (0, 1, 2), (0, 1)


def groupby_table(n: int = 60_000_000, seed: int = 1) -> Table:
    """60M rows: key i64, flag_a i8 in {0,1,2}, flag_b i8 in {0,1}, qty f64 integers 1..50,
    price f64 in [900,105000), disc f64 in [0,0.1), tax f64 in [0,0.08), day i32 in [0,2557)."""
    rng = np.random.default_rng(seed)
    cols = {"key": np.arange(n, dtype=np.int64),
            "flag_a": rng.integers(0, 3, n, dtype=np.int8),
            "flag_b": rng.integers(0, 2, n, dtype=np.int8),
            "qty": rng.integers(1, 51, n).astype(np.float64),
            "price": rng.uniform(900.0, 105000.0, n),
            "disc": rng.uniform(0.0, 0.1, n),
            "tax": rng.uniform(0.0, 0.08, n),
            "day": rng.integers(0, 2557, n, dtype=np.int32)}
    return Table.from_arrays(2, cols, name="groupby")


GROUPS = [(a, b) for a in FLAG_A for b in FLAG_B]
GROUP_FIELDS = ["sum_qty", "sum_price", "sum_disc_price", "sum_charge", "sum_disc", "count"]
OUT_FIELDS = ["sum_qty", "sum_price", "sum_disc_price", "sum_charge", "avg_qty", "avg_price", "avg_disc", "count"]


def groupby_query(tbl_type: ir.DataType, day_max=Q1_DAY) -> ir.Func:
    """Per (flag_a, flag_b) group over rows with day <= day_max: SUM qty, price,
    price*(1-disc), price*(1-disc)*(1+tax), disc and COUNT, as TPC-H Q1's select-per-group
    accumulators (tpch.h:412-478); the output adds AVG qty/price/disc = SUM/COUNT."""
    vec = _sym("lineitem", tbl_type)

    def acc(s, v):
        fa, fb, qty, price, disc, tax, day = (_get(v, i) for i in range(7))
        disc_price = _mul(price, _sub(_f64(1), disc))
        charge = _mul(disc_price, _add(_f64(1), tax))
        vals = [qty, price, disc_price, charge, disc]
        out = []
        for g, (a, b) in enumerate(GROUPS):
            c = _eq(fa, _i8(a)) & _eq(fb, _i8(b)) & _lte(day, _i32(day_max))
            sg = _get(s, g)
            fields = [_sel(c, _add(_get(sg, k), vals[k]), _get(sg, k)) for k in range(5)]
            fields.append(_sel(c, _add(_get(sg, 5), _i64(1)), _get(sg, 5)))
            out.append(_new(fields))
        return _new(out)

    init = lambda: _new([_new([_f64(0)] * 5 + [_i64(0)]) for _ in GROUPS])
    red = _red(_subvec(vec, _idx(0), _len(vec, 1)), init, acc)
    red_sym = _sym("red", red)
    outs = []
    for g in range(len(GROUPS)):
        sg = _get(red_sym, g)
        cnt = _cast(ir._f64_t, _get(sg, 5))
        outs.append(_new([_get(sg, 0), _get(sg, 1), _get(sg, 2), _get(sg, 3),
                          _div(_get(sg, 0), cnt), _div(_get(sg, 1), cnt), _div(_get(sg, 4), cnt), _get(sg, 5)]))
    res = _new(outs)
    res_sym = _sym("res", res)
    fn = _func("groupby", res_sym, [vec])
    fn.tbl[red_sym] = red
    fn.tbl[res_sym] = res
    return fn


# ----------------------------------------------------------------------------- high-card group-by
def zipf_keys(n: int, ndistinct: int, s: float, rng) -> np.ndarray:
    """n int64 keys: rank ~ Zipf(s) truncated to `ndistinct` ranks (inverse-CDF sampling), mapped
    through a seeded permutation to distinct ids (an odd multiplier permutes the 2^40 space)."""
    w = np.arange(1, ndistinct + 1, dtype=np.float64) ** (-s)
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    ranks = np.searchsorted(cdf, rng.random(n), side="right")
    np.minimum(ranks, ndistinct - 1, out=ranks)
    mult = (int(rng.integers(1, 1 << 39)) << 1) | 1
    ids = ((ranks.astype(np.uint64) * np.uint64(mult)) & np.uint64((1 << 40) - 1)).astype(np.int64)
    return ids


def hashgroup_table(n: int = 100_000_000, ndistinct: int = 10_000_000, s: float = 1.1, seed: int = 2) -> Table:
    """n rows: key int64 (Zipf(s) over `ndistinct` ids, unsorted, flat), value f64 in [0,1000).
    dim 2: the key is the first of two iterator columns, as a grouped vector."""
    rng = np.random.default_rng(seed)
    keys = zipf_keys(n, ndistinct, s, rng)
    vals = rng.uniform(0.0, 1000.0, n)
    return Table.from_arrays(2, {"key": keys, "value": vals}, name="zipf")


def ree_sorted(t: Table) -> Table:
    """The same rows stably sorted by key, key run-end encoded: the layout the reference's
    grouped aggregation needs (a 2-d vector with a "+r" column 0, test_multidim.cpp)."""
    from .table import ree_encode
    order = np.argsort(t.columns[0].data, kind="stable")
    keys = t.columns[0].data[order]
    vals, ends = ree_encode(keys)
    cols = {"key": vals}
    for c in t.columns[1:]:
        cols[c.name] = c.data[order]
    return Table.from_arrays(2, cols, runend={"key": ends}, name=t.name + "_ree")


def hashgroup_query(tbl_type: ir.DataType) -> ir.Func:
    """Per key: SUM(value) f64 and COUNT i64 - an Op over the 2-d vector whose output reduces
    each key's rows (the grouped form of test_multidim.cpp:9-29 and TPC-H Q18, tpch.h:687-715).
    Over a run-end encoded key column it is the reference's segmented reduce; over a flat,
    unsorted key column the GPU backend runs it as a hash group-by."""
    vec = _sym("vec", tbl_type)
    t = _sym("key", ir._i64_t)
    red = _red(vec[t], lambda: _new([_f64(0), _i64(0)]),
               lambda s, v: _new([_add(_get(s, 0), _get(v, 0)), _add(_get(s, 1), _i64(1))]))
    red_sym = _sym("agg", red)
    op = ir._op([t], ir._in(t, vec), [_get(red_sym, 0), _get(red_sym, 1)])
    op_sym = _sym("op", op)
    fn = _func("group_sum", op_sym, [vec])
    fn.tbl[red_sym] = red
    fn.tbl[op_sym] = op
    return fn


# ----------------------------------------------------------------------------- join + aggregate
Q3_ATTR, Q3_DAY_LO, Q3_DAY_HI = 5, 0, 365


def join_tables(n_build: int = 10_000_000, n_probe: int = 200_000_000, seed: int = 3,
                probe_seed=None) -> Tuple[Table, Table]:
    """Build: unique int64 keys (a seeded sample of a 2^40 space) + attr i32 in [0,25).
    Probe: fk = a uniform build key with p=0.9, else a key from a disjoint range (a miss);
    amount f64 in [1,10000); day i32 in [0,2557).  With `probe_seed`, the probe rows come from
    their own generator (the build side stays that of `seed`): one rank's share of a probe
    table partitioned over ranks that all hold the same build side."""
    rng = np.random.default_rng(seed)
    # distinct keys: a random odd multiplier permutes the 2^40 space; take n consecutive images
    mult = (int(rng.integers(1, 1 << 39)) << 1) | 1
    base = np.arange(n_build, dtype=np.uint64)
    keys = ((base * np.uint64(mult)) & np.uint64((1 << 40) - 1)).astype(np.int64)
    attr = rng.integers(0, 25, n_build, dtype=np.int32)
    build = Table.from_arrays(1, {"key": keys, "attr": attr}, name="build")
    if probe_seed is not None:
        rng = np.random.default_rng(probe_seed)
    hit = rng.random(n_probe) < 0.9
    fk = keys[rng.integers(0, n_build, n_probe)]
    miss = (np.int64(1) << 41) + rng.integers(0, 1 << 40, n_probe, dtype=np.int64)
    fk = np.where(hit, fk, miss)
    amount = rng.uniform(1.0, 10000.0, n_probe)
    day = rng.integers(0, 2557, n_probe, dtype=np.int32)
    probe = Table.from_arrays(2, {"row": np.arange(n_probe, dtype=np.int64), "fk": fk, "amount": amount,
                                  "day": day}, name="probe")
    return build, probe


def join_query(build_type: ir.DataType, probe_type: ir.DataType, attr_max=Q3_ATTR, day_lo=Q3_DAY_LO,
               day_hi=Q3_DAY_HI) -> ir.Func:
    """SUM(amount) and COUNT per build attribute over probe rows whose fk is found in the build
    side (Locate, the reference's hash-join probe: loopgen.cpp:17-22, vinstr.h:137-146), with
    attr < attr_max and day in [day_lo, day_hi); the guarded form of TPC-H Q3 (tpch.h:51-56)."""
    build = _sym("build", build_type)
    probe = _sym("probe", probe_type)

    def acc(s, v):
        fk, amount, day = _get(v, 0), _get(v, 1), _get(v, 2)
        idx = _locate(build, fk)
        attr = _readdata(build, idx, 1)
        base = _gte(idx, _idx(0)) & _lt(attr, _i32(attr_max)) & _gte(day, _i32(day_lo)) & _lt(day, _i32(day_hi))
        out = []
        for g in range(attr_max):
            c = base & _eq(attr, _i32(g))
            sg = _get(s, g)
            out.append(_new([_sel(c, _add(_get(sg, 0), amount), _get(sg, 0)),
                             _sel(c, _add(_get(sg, 1), _i64(1)), _get(sg, 1))]))
        return _new(out)

    red = _red(_subvec(probe, _idx(0), _len(probe, 1)), lambda: _new([_new([_f64(0), _i64(0)]) for _ in range(attr_max)]),
               acc)
    red_sym = _sym("red", red)
    fn = _func("join_agg", red_sym, [build, probe])
    fn.tbl[red_sym] = red
    return fn


def algorithmic_bytes(table: Table, cols) -> int:
    """Bytes of the referenced columns, each read once (validity bitmaps only if present)."""
    return table.nbytes(cols)
