"""A grouped sum over a wide row: two int8 key columns (4 groups) and `ncol` FP64 value columns,
every value column summed per group (the grouped scan then takes fewer rows per step)."""
import numpy as np

from reffine_gb300 import workloads as W
from reffine_gb300.table import Table

GROUPS = [(a, b) for a in (0, 1) for b in (0, 1)]


def wide_table(n: int, ncol: int, seed: int = 0) -> Table:
    rng = np.random.default_rng(seed)
    cols = {"key": np.arange(n, dtype=np.int64), "ka": rng.integers(0, 2, n, dtype=np.int8),
            "kb": rng.integers(0, 2, n, dtype=np.int8)}
    for i in range(ncol):
        cols["v%d" % i] = rng.uniform(0.0, 1000.0, n) * 2.0 ** (i - ncol // 2)
    return Table.from_arrays(2, cols, name="wide")


def wide_groupby_query(tbl_type, ncol: int):
    vec = W._sym("wide", tbl_type)

    def acc(s, v):
        ka, kb = W._get(v, 0), W._get(v, 1)
        vals = [W._get(v, 2 + i) for i in range(ncol)]
        out = []
        for g, (a, b) in enumerate(GROUPS):
            c = W._eq(ka, W._i8(a)) & W._eq(kb, W._i8(b))
            sg = W._get(s, g)
            out.append(W._new([W._sel(c, W._add(W._get(sg, k), vals[k]), W._get(sg, k)) for k in range(ncol)]))
        return W._new(out)

    init = lambda: W._new([W._new([W._f64(0)] * ncol) for _ in GROUPS])
    red = W._red(W._subvec(vec, W._idx(0), W._len(vec, 1)), init, acc)
    red_sym = W._sym("red", red)
    fn = W._func("wide", red_sym, [vec])
    fn.tbl[red_sym] = red
    return fn
