"""GPU parity of the scan-reduce templates against the oracle (same seeded inputs).

Integers (counts, integer sums) must be bit-exact; FP64 sums within RTOL_F64 (parity.py).
Sizes are chosen so the oracle finishes in seconds and tails are ragged (not multiples of a
tile or a warp).
"""
import numpy as np
import pytest

import refqueries as rq
from oracle import loopgen
from parity import assert_same
from reffine_gb300 import _capi, engine, workloads as W
from reffine_gb300.table import Table, pack_validity

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [0, 1, 1000, 257_123, 1_000_003])
def test_filter_sum_parity(eng, n):
    t = W.filter_sum_table(n, seed=5)
    fn = W.filter_sum_query(t.get_data_type())
    ref = loopgen.Query(fn)(t)
    got = eng.compile(fn).run(eng.upload(t))
    assert_same(got, ref)
    if n > 1000:
        assert ref[1] > 0


def test_filter_sum_random_constants_share_module(eng):
    t = W.filter_sum_table(300_001, seed=9)
    dt = eng.upload(t)
    rng = np.random.default_rng(0)
    for _ in range(4):
        lo = int(rng.integers(0, 2000))
        hi = lo + int(rng.integers(1, 600))
        dlo = round(float(rng.integers(0, 8)) / 100, 6)
        fn = W.filter_sum_query(t.get_data_type(), lo, hi, dlo, dlo + 0.02, float(rng.integers(2, 50)))
        assert_same(eng.compile(fn).run(dt), loopgen.Query(fn)(t))


@pytest.mark.parametrize("vectorize", [False, True])
def test_groupby_parity(eng, vectorize):
    t = W.groupby_table(1_234_567, seed=7)
    fn = W.groupby_query(t.get_data_type())
    plan = eng.compile(fn, vectorize)
    assert plan.kind == 2  # grouped template
    got = plan.run(eng.upload(t))
    ref = loopgen.Query(fn, vectorize)(t)
    assert_same(got, ref)


def test_join_parity(eng):
    b, p = W.join_tables(100_003, 1_500_007, seed=11)
    fn = W.join_query(b.get_data_type(), p.get_data_type())
    got = eng.compile(fn).run(eng.upload(b), eng.upload(p))
    ref = loopgen.Query(fn)(b, p)
    assert_same(got, ref)
    assert sum(g[1] for g in ref) > 0


@pytest.mark.parametrize("groups", [1, 11, 12, 25])
def test_join_group_counts(eng, groups):
    # 12 groups x 2 aggregates x 256 threads x 8 B is exactly 48 KiB of privatised slots: the
    # kernel must opt in to more than the default dynamic shared memory (48 KiB minus static)
    b, p = W.join_tables(20_000, 400_003, seed=12)
    fn = W.join_query(b.get_data_type(), p.get_data_type(), groups, 100, 900)
    got = eng.compile(fn).run(eng.upload(b).build_index(), eng.upload(p))
    assert_same(got, loopgen.Query(fn)(b, p))


@pytest.mark.parametrize("dups", [False, True])
def test_join_filtered_index_matches_full_probe(eng, dups):
    # the build-side filter (attr < 5) is applied while the probed index is built; with
    # repeated build keys the filtered index must keep exactly the row the full index returns
    # (the first), whatever the other rows of the key hold
    rng = np.random.default_rng(21)
    nb, npr = 50_000, 600_011
    keys = rng.integers(0, 20_000, nb).astype(np.int64) if dups else rng.permutation(1 << 20)[:nb].astype(np.int64)
    build = Table.from_arrays(1, {"key": keys, "attr": rng.integers(0, 25, nb, dtype=np.int32)}, name="build")
    fk = keys[rng.integers(0, nb, npr)]
    probe = Table.from_arrays(2, {"row": np.arange(npr, dtype=np.int64), "fk": fk,
                                  "amount": rng.uniform(1.0, 10000.0, npr), "day": rng.integers(0, 2557, npr, dtype=np.int32)})
    fn = W.join_query(build.get_data_type(), probe.get_data_type(), 5, 0, 900)
    plan = eng.compile(fn)
    db, dp = eng.upload(build).build_index(), eng.upload(probe)
    got = plan.run(db, dp)
    assert_same(got, loopgen.Query(fn)(build, probe))
    assert got == plan.run(db, dp)  # the second run reuses the kept-entry count


def test_validity_of_column_one_gates_rows(eng):
    # loopgen.cpp:238: a SubVector reduce skips rows whose column-1 value is null
    t = W.filter_sum_table(100_000, seed=3)
    mask = np.random.default_rng(1).random(len(t)) < 0.7
    t.columns[1].valid = pack_validity(mask)
    fn = W.filter_sum_query(t.get_data_type())
    assert_same(eng.compile(fn).run(eng.upload(t)), loopgen.Query(fn)(t))


@pytest.mark.parametrize("vectorize", [False, True])
def test_reference_reduce_goldens_on_gpu(eng, vectorize):
    st2 = rq.students_table(2)
    assert eng.compile(rq.sum_col1_op(st2), vectorize).run(eng.upload(st2)) == 131977
    st = rq.students_table()
    assert eng.compile(rq.vector_op(st), vectorize).run(eng.upload(st)) == 696


def test_thunk_has_reference_call_shape(eng):
    # compile_op returns a function called as fn(&out, ArrowTable*): host tables in, result out
    t = W.filter_sum_table(200_003, seed=13)
    fn = W.filter_sum_query(t.get_data_type())
    q = engine.compile_op(fn, engine=eng)
    assert_same(q(t), loopgen.Query(fn)(t))
    st = rq.students_table()
    assert engine.compile_op(rq.vector_op(st), engine=eng)(st) == 696


def test_missing_lower_bound_reports_error(eng):
    # ReduceOpTest's space starts at Locate(max(lb, col0[0])); a key absent from the iterator
    # column makes the reference read row -1.  Here the run fails with RF_ERR_DEVICE.
    st = rq.students_table()
    ids = st.columns[0].data.copy()
    ids[9] = 10_000_000  # no id 10 any more
    st.columns[0].data = ids
    with pytest.raises(_capi.RfError) as e:
        eng.compile(rq.vector_op(st)).run(eng.upload(st))
    assert e.value.status == _capi.RF_ERR_DEVICE
    # the context stays usable
    st = rq.students_table()
    assert eng.compile(rq.vector_op(st)).run(eng.upload(st)) == 696


def test_groupby_fused_products_nonfinite(eng):
    # rows with an infinite or NaN factor must give the reference's inf / NaN sums, and a
    # product that is exactly 0 (or NaN from 0 * inf) must stay so
    t = W.groupby_table(400_003, seed=17)
    price, disc, tax = (t.columns[i].data for i in (4, 5, 6))
    rng = np.random.default_rng(4)
    idx = rng.choice(len(t), 12, replace=False)
    price[idx[0]] = np.inf
    price[idx[1]] = -np.inf
    price[idx[2]] = np.nan
    disc[idx[3]] = np.inf
    tax[idx[4]] = -np.inf
    disc[idx[5]] = 1.0      # x*(1-y) = 0 exactly
    price[idx[6]] = 0.0
    disc[idx[6]] = np.inf   # 0*(1-inf): NaN
    fn = W.groupby_query(t.get_data_type())
    got = eng.compile(fn).run(eng.upload(t))
    assert_same(got, loopgen.Query(fn)(t))


def test_groupby_fused_products_band_edges(eng):
    # x*(1-y) and x*(1+y) are one fused multiply-add only for |x| in [2^-500, 2^500) and
    # |y| < 2^500; rows at and beyond those edges, near overflow, subnormal, and with 1 -/+ y
    # cancelling, must agree with the twice-rounded products
    t = W.groupby_table(300_007, seed=29)
    price, disc, tax = (t.columns[i].data for i in (4, 5, 6))
    rng = np.random.default_rng(29)
    idx = rng.choice(len(t), 16, replace=False)
    price[idx[0]] = 2.0 ** 500               # first value above the band
    price[idx[1]] = np.nextafter(2.0 ** 500, 0)
    price[idx[2]] = 2.0 ** -500              # lowest value in the band
    price[idx[3]] = np.nextafter(2.0 ** -500, 0)
    price[idx[4]] = 1.0e308
    disc[idx[4]] = -0.9                      # 1.9e308: overflows in both forms
    price[idx[5]] = 5e-324                   # subnormal
    disc[idx[6]] = 2.0 ** 500
    tax[idx[7]] = 2.0 ** 600
    disc[idx[8]] = 1.0 - 2.0 ** -52          # 1 - y exact and tiny
    disc[idx[9]] = 1.0 + 2.0 ** -52          # a negative product
    tax[idx[10]] = -1.0 + 2.0 ** -52         # 1 + y exact and tiny
    tax[idx[11]] = -1.0                      # 1 + y = 0
    price[idx[12]] = -3.5                    # a negative product, -0 from 1 - y = 0
    disc[idx[12]] = 1.0
    fn = W.groupby_query(t.get_data_type())
    got = eng.compile(fn).run(eng.upload(t))
    assert_same(got, loopgen.Query(fn)(t))


@pytest.mark.parametrize("ncol", [4, 14])
def test_wide_row_groupby_parity(eng, ncol):
    # a grouped sum over 4 and 14 FP64 columns: four rows a thread per step for the narrow row,
    # two for the wide one (its 30 register words of loaded columns)
    from widequery import wide_groupby_query, wide_table
    t = wide_table(700_001, ncol, seed=41)
    fn = wide_groupby_query(t.get_data_type(), ncol)
    plan = eng.compile(fn)
    assert "#define RF_GROUP_ROWS %d" % (4 if ncol == 4 else 2) in plan.source
    assert_same(plan.run(eng.upload(t)), loopgen.Query(fn)(t))


def test_groupby_mixed_signs_wide_exponents(eng):
    # grouped FP64 sums over addends of both signs spread over ~60 binades, with tiny, huge,
    # subnormal and signed-zero values at random rows
    t = W.groupby_table(600_011, seed=23)
    rng = np.random.default_rng(23)
    qty, price = t.columns[3].data, t.columns[4].data
    n = len(t)
    qty[:] = rng.uniform(-1.0, 3.0, n) * 2.0 ** rng.integers(-27, 30, n)
    price[:] = rng.uniform(-2.0, 5.0, n) * 2.0 ** rng.integers(-20, 20, n)
    idx = rng.choice(n, 40, replace=False)
    qty[idx[:8]] = 1e-20
    qty[idx[8:16]] = 2.0 ** 40
    price[idx[16:24]] = 5e-324
    price[idx[24:32]] = -0.0
    qty[idx[32:40]] = 0.0
    fn = W.groupby_query(t.get_data_type())
    plan = eng.compile(fn)
    assert plan.kind == 2
    dt = eng.upload(t)
    got = plan.run(dt)
    assert_same(got, loopgen.Query(fn)(t))
    assert plan.run(dt) == got  # same bits on a second run


def test_join_filtered_index_kept_between_runs(eng):
    # a plan keeps its filtered index for the next run on the same table (same bits), and a new
    # upload of the build side (a new table generation) is never answered from the kept index
    b, p = W.join_tables(50_000, 400_001, seed=61)
    fn = W.join_query(b.get_data_type(), p.get_data_type())
    plan = eng.compile(fn)
    db, dp = eng.upload(b), eng.upload(p)
    first = plan.run(db, dp)
    assert plan.run(db, dp) == first
    assert_same(first, loopgen.Query(fn)(b, p))
    rng = np.random.default_rng(62)
    b.columns[1].data = rng.permutation(b.columns[1].data)  # other rows pass the build filter now
    db2 = eng.upload(b)
    again = plan.run(db2, dp)
    assert_same(again, loopgen.Query(fn)(b, p))
    assert again != first
    # back on the first table: its own answer, not the one the kept index would give
    assert plan.run(db, dp) == first


def test_groupby_sums_of_one_sign_over_wide_magnitudes(eng):
    # FP64 sums of positive addends spread over ~120 binades (each thread's sums kept as
    # double-floats on the FP32 pipe while its addends stay non-negative and in range, FP64 after
    # the first that is not): within 1e-12 of the serial FP64 sums; sums of integers (the
    # quantities) stay exact
    t = W.groupby_table(700_001, seed=29)
    rng = np.random.default_rng(29)
    n = len(t)
    price = t.columns[4].data
    price[:] = rng.uniform(1.0, 2.0, n) * 2.0 ** rng.integers(-60, 60, n)
    idx = rng.choice(n, 30, replace=False)
    price[idx[:5]] = 2.0 ** 90        # kept as a double-float
    price[idx[5:10]] = 2.0 ** 99      # beyond the double-float range: that thread continues in FP64
    price[idx[10:20]] = 2.0 ** -103   # the smallest kept
    price[idx[20:]] = 0.0
    fn = W.groupby_query(t.get_data_type())
    dt = eng.upload(t)
    got = eng.compile(fn).run(dt)
    ref = loopgen.Query(fn)(t)
    assert_same(got, ref)
    for g, r in zip(got, ref):
        assert g[0] == r[0] and g[7] == r[7]  # SUM(quantity) of integers and COUNT: exact
