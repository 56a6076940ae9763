"""Queries over a table partitioned by rows across processes (one GPU each), with one answer.

Rows are independent, so each rank runs the query's Reduce over its own contiguous row range
and the partial states are folded on rank 0 in rank order (a fixed order: the FP64 folds give
the same bits on every run); the Func's output expression is then evaluated on the folded state.
A grouped Op's partial tables (key, aggregates...) are concatenated in rank order, sorted by key
(stable) and each key's rows folded in that order.  No collective touches the data path: the
exchange is the partial states (a few hundred bytes for a Reduce) gathered once per query.

    state_fn, finish = split_reduce(fn)        # the Reduce's state, and how to finish it
    part = plan_of(state_fn).run(my_rows)      # on each rank, over row_range(n, rank, world)
    answer = finish(fold_states(gathered, leaf_ops(fn)))   # on rank 0

Partition plans of the benchmark workloads:
  filter + sum, group-by      contiguous row ranges, fold of the Reduce states
  join + aggregate            every rank holds the whole build side, probe rows by range
  hash group-by               row ranges, then the key-sorted fold of the partial tables
"""
from __future__ import annotations

from typing import Callable, Dict, List, Sequence, Tuple

import numpy as np

from . import ir


def row_range(n: int, rank: int, world: int) -> Tuple[int, int]:
    """Rank `rank`'s contiguous share [lo, hi) of n rows (the first n % world ranks take one more)."""
    q, r = divmod(n, world)
    lo = rank * q + min(rank, r)
    return lo, lo + q + (1 if rank < r else 0)


def _resolve(fn: ir.Func, e: ir.Expr) -> ir.Expr:
    while isinstance(e, ir.Sym) and e in fn.tbl:
        e = fn.tbl[e]
    return e


def split_reduce(fn: ir.Func) -> Tuple[ir.Func, Callable]:
    """(state Func, finish): the state Func outputs the Func's Reduce state; finish(state) gives
    the Func's own output (its expression over the state, evaluated on the host)."""
    reds = [s for s, e in fn.tbl.items() if isinstance(e, ir.Reduce)]
    if len(reds) != 1:
        raise ValueError("a sharded query has exactly one Reduce")
    red_sym = reds[0]
    out = fn.output
    if out is red_sym or _resolve(fn, out) is fn.tbl[red_sym]:
        return fn, lambda s: s
    state_fn = ir.Func(fn.name + "_state", red_sym, fn.inputs, {red_sym: fn.tbl[red_sym]})

    def finish(state):
        return _eval(fn, out, {id(red_sym): state})

    return state_fn, finish


def leaf_ops(fn: ir.Func) -> object:
    """How each leaf of the Reduce state folds: nested lists of "sum" / "max" / "min", read off the
    accumulator (state_leaf + x, or select(c, state_leaf + x, state_leaf), and max/min alike)."""
    red = next(e for e in fn.tbl.values() if isinstance(e, ir.Reduce))

    def leaf(path, acc):
        if isinstance(acc, ir.New):
            return [leaf(path + [i], a) for i, a in enumerate(acc.vals)]
        e = acc
        if isinstance(e, ir.Select):
            e = e.t if not _is_state_leaf(e.t, red, path) else e.f
        if isinstance(e, ir.Nary) and e.op in ("add", "max", "min") and any(_is_state_leaf(a, red, path) for a in e.args):
            return {"add": "sum", "max": "max", "min": "min"}[e.op]
        raise ValueError("state leaf %r does not fold by sum, max or min" % (path,))

    return leaf([], red.acc)


def _is_state_leaf(e, red, path) -> bool:
    for p in reversed(path):
        if not (isinstance(e, ir.Get) and e.col == p):
            return False
        e = e.val
    return e is red.state


def _fold(a, b, op):
    if isinstance(op, list):
        return tuple(_fold(x, y, o) for x, y, o in zip(a, b, op))
    if op == "sum":
        return a + b
    return max(a, b) if op == "max" else min(a, b)


def fold_states(states: Sequence, ops) -> object:
    """Folds the ranks' partial states in rank order."""
    acc = states[0]
    for s in states[1:]:
        acc = _fold(acc, s, ops)
    return acc


def fold_tables(tables: Sequence[Dict], ops: Sequence[str]) -> Dict:
    """Partial grouped tables {"cols": [keys, agg...], "len"} of the ranks, in rank order, folded
    into one: stable sort by key, then each key's rows folded in that (rank) order."""
    cols = [np.concatenate([t["cols"][c] for t in tables]) for c in range(len(tables[0]["cols"]))]
    order = np.argsort(cols[0], kind="stable")
    cols = [c[order] for c in cols]
    keys = cols[0]
    if len(keys) == 0:
        return {"cols": cols, "len": 0}
    starts = np.flatnonzero(np.r_[True, keys[1:] != keys[:-1]])
    out = [keys[starts]]
    for c, op in zip(cols[1:], ops):
        if op == "sum":
            if np.issubdtype(c.dtype, np.floating):
                # a key's partial sums added one by one in rank order (reduceat may reassociate)
                res = np.empty(len(starts), dtype=c.dtype)
                ends = np.r_[starts[1:], len(c)]
                for i, (a, b) in enumerate(zip(starts, ends)):
                    s = c[a]
                    for j in range(a + 1, b):
                        s = s + c[j]
                    res[i] = s
                out.append(res)
            else:
                out.append(np.add.reduceat(c, starts))
        elif op == "max":
            out.append(np.maximum.reduceat(c, starts))
        else:
            out.append(np.minimum.reduceat(c, starts))
    return {"cols": out, "len": len(starts)}


# ---------------------------------------------------------------------------- host evaluation
def _eval(fn: ir.Func, e: ir.Expr, env: Dict[int, object]):
    """The output expression over a finished state: Get/New/Select/Cast and arithmetic, with C
    semantics for the types it meets (IEEE doubles; integer division truncates)."""
    if id(e) in env:
        return env[id(e)]
    if isinstance(e, ir.Sym):
        if e in fn.tbl:
            v = _eval(fn, fn.tbl[e], env)
            env[id(e)] = v
            return v
        raise ValueError("unbound symbol %s in the output expression" % e.name)
    if isinstance(e, ir.Const):
        return float(e.val) if e.type.is_float() else int(e.val)
    if isinstance(e, ir.Get):
        return _eval(fn, e.val, env)[e.col]
    if isinstance(e, ir.New):
        return tuple(_eval(fn, a, env) for a in e.vals)
    if isinstance(e, ir.Select):
        return _eval(fn, e.t, env) if _eval(fn, e.cond, env) else _eval(fn, e.f, env)
    if isinstance(e, ir.Cast):
        v = _eval(fn, e.arg, env)
        return float(v) if e.type.is_float() else int(v)
    if isinstance(e, ir.Nary):
        a = [_eval(fn, x, env) for x in e.args]
        f = e.type.is_float()
        ops = {"add": lambda: a[0] + a[1], "sub": lambda: a[0] - a[1], "mul": lambda: a[0] * a[1],
               "div": lambda: (a[0] / a[1]) if f else int(a[0] / a[1]), "max": lambda: max(a),
               "min": lambda: min(a), "neg": lambda: -a[0], "lt": lambda: a[0] < a[1], "lte": lambda: a[0] <= a[1],
               "gt": lambda: a[0] > a[1], "gte": lambda: a[0] >= a[1], "eq": lambda: a[0] == a[1],
               "and": lambda: a[0] and a[1], "or": lambda: a[0] or a[1], "not": lambda: not a[0]}
        if e.op not in ops:
            raise ValueError("operator %s in the output expression is not evaluated on the host" % e.op)
        if f and e.op == "div" and a[1] == 0:
            return float("nan") if a[0] == 0 or a[0] != a[0] else (float("inf") if a[0] > 0 else float("-inf"))
        return ops[e.op]()
    raise ValueError("%s in the output expression is not evaluated on the host" % type(e).__name__)
