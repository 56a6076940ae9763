// The benchmark and golden queries, built with Reffine's own IR builder
// (include/reffine/builder/reffiner.h).  Each query is written node for node as tests/refqueries.py
// and reffine_gb300/workloads.py write it with the Python builder.  Used by the binding's test
// program (tests/ref_binding/ref_queries.cpp) and by the reference-pipeline oracle
// (oracle/ref/ref_pipeline.cpp); compiles only where Reffine's headers are available.
#pragma once
#include <functional>
#include <string>
#include <utility>
#include <vector>

#include "reffine/builder/reffiner.h"

namespace refq {

using namespace reffine;
using namespace reffine::reffiner;

inline DataType vec_t(size_t dim, std::vector<DataType> cols, std::vector<EncodeType> enc = {})
{
    if (enc.empty()) enc.assign(cols.size(), FLAT);
    return DataType(VECTOR, cols, dim, enc);
}

inline const DataType kStudents = vec_t(1, {_i64_t, _i64_t, _i64_t, _i64_t, _i64_t, _i64_t});
inline const DataType kRunend = vec_t(2, {_i64_t, _i64_t, _i64_t}, {RUNEND, FLAT, FLAT});
inline const DataType kFilterSum = vec_t(2, {_i64_t, _i32_t, _f64_t, _f64_t, _f64_t});
inline const DataType kGroupBy = vec_t(2, {_i64_t, _i8_t, _i8_t, _f64_t, _f64_t, _f64_t, _f64_t, _i32_t});
inline const DataType kHashGroup = vec_t(2, {_i64_t, _f64_t});
// the same table with its keys sorted and run-end encoded: the form Reffine's grouped Op reads
inline const DataType kHashGroupRee = vec_t(2, {_i64_t, _f64_t}, {RUNEND, FLAT});
inline const DataType kJoinBuild = vec_t(1, {_i64_t, _i32_t});
inline const DataType kJoinProbe = vec_t(2, {_i64_t, _i64_t, _f64_t, _i32_t});
inline const DataType kGen = vec_t(1, {_i64_t, _i64_t});

// test_reduce.cpp:61-110 (ReduceOpTest)
inline shared_ptr<Func> vector_op()
{
    auto t = _sym("t", _i64_t);
    auto vec_in = _sym("vec_in", kStudents);
    auto op = _op(vector<Sym>{t}, _in(t, vec_in) & _lte(t, _i64(48)) & _gte(t, _i64(10)),
                  vector<Expr>{vec_in[{t}][2],
                               _new(vector<Expr>{vec_in[{t}][1], vec_in[{t}][2], vec_in[{t}][0], vec_in[{t}][3]}),
                               vec_in[{t}][3]});
    auto red = _red(
        op,
        []() {
            return _new(vector<Expr>{_new(vector<Expr>{_i64(0), _i64(0)}), _new(vector<Expr>{_i64(0), _i64(0)})});
        },
        [](Expr s, Expr v) {
            auto v0 = _get(_get(v, 2), 0);
            auto v1 = _get(_get(v, 2), 1);
            auto v2 = _get(_get(v, 2), 2);
            auto v3 = _get(_get(v, 2), 3);
            auto s0 = _get(_get(s, 0), 0);
            auto s1 = _get(_get(s, 0), 1);
            auto s2 = _get(_get(s, 1), 0);
            auto s3 = _get(_get(s, 1), 1);
            return _new(vector<Expr>{_new(vector<Expr>{_add(s0, v0), _add(s1, v1)}),
                                     _new(vector<Expr>{_add(s2, v2), _add(s3, v3)})});
        });
    auto sum = _sym("sum", red);
    auto res = _get(_get(sum, 1), 0);
    auto res_sym = _sym("res", res);
    auto fn = _func("foo", res_sym, vector<Sym>{vec_in});
    fn->tbl[sum] = red;
    fn->tbl[res_sym] = res;
    return fn;
}

// test_transform.cpp:9-30 (TransformOpTest), lb 5, n 10
inline shared_ptr<Func> transform_op()
{
    auto t = _sym("t", _i64_t);
    auto vec_in = _sym("vec_in", kStudents);
    auto elem = vec_in[{t}];
    auto elem_sym = _sym("elem", elem);
    auto out = _add(elem_sym[0], _i64(10));
    auto out_sym = _sym("out", out);
    auto op = _op(vector<Sym>{t}, _in(t, vec_in) & _gt(t, _i64(5)), vector<Expr>{out_sym});
    auto op_sym = _sym("op", op);
    auto fn = _func("foo", op_sym, vector<Sym>{vec_in});
    fn->tbl[elem_sym] = elem;
    fn->tbl[out_sym] = out;
    fn->tbl[op_sym] = op;
    return fn;
}

// test_multidim.cpp:9-29 (MultiDimOpTest)
inline shared_ptr<Func> multidim_op()
{
    auto vec = _sym("vec_in", kRunend);
    auto t = _sym("t_sym", _i64_t);
    auto red = _red(vec[{t}], []() { return _i64(0); }, [](Expr s, Expr v) { return _add(s, _get(v, 1)); });
    auto red_sym = _sym("sum", red);
    auto op = _op(vector<Sym>{t}, _in(t, vec), vector<Expr>{red_sym});
    auto op_sym = _sym("op", op);
    auto fn = _func("red", op_sym, vector<Sym>{vec});
    fn->tbl[op_sym] = op;
    fn->tbl[red_sym] = red;
    return fn;
}

// test_utils.cpp:32-46 (the generator of JoinOpTest's tables)
inline shared_ptr<Func> gen_table_op()
{
    auto t = _sym("t", _i64_t);
    auto lb = _sym("lb", _i64_t);
    auto ub = _sym("ub", _i64_t);
    auto op = _op(vector<Sym>{t}, _gte(t, lb) & _lt(t, ub), vector<Expr>{t});
    auto op_sym = _sym("op", op);
    auto fn = _func("gen_table", op_sym, vector<Sym>{lb, ub});
    fn->tbl[op_sym] = op;
    return fn;
}

// test_join.cpp:9-37 (JoinOpTest)
inline shared_ptr<Func> join_op()
{
    auto avec = _sym("avec", kGen);
    auto bvec = _sym("bvec", kGen);
    auto cvec = _sym("cvec", kGen);
    auto t = _sym("t", _i64_t);
    auto aelem = avec[{t}][0];
    auto belem = bvec[{t}][0];
    auto celem = cvec[{t}][0];
    auto a_s = _sym("a", aelem);
    auto b_s = _sym("b", belem);
    auto c_s = _sym("c", celem);
    auto op = _op(vector<Sym>{t}, _in(t, avec) & _in(t, bvec) & _in(t, cvec), vector<Expr>{_add(_add(a_s, b_s), c_s)});
    auto op_sym = _sym("op", op);
    auto fn = _func("join", op_sym, vector<Sym>{avec, bvec, cvec});
    fn->tbl[a_s] = aelem;
    fn->tbl[b_s] = belem;
    fn->tbl[c_s] = celem;
    fn->tbl[op_sym] = op;
    return fn;
}

// test_nested.cpp:9-27 (NestedOpTest), 10 x 10
inline shared_ptr<Func> nested_op()
{
    auto a = _sym("a", _i64_t);
    auto b = _sym("b", _i64_t);
    auto op = _op(vector<Sym>{a, b}, _gte(a, _i64(0)) & _lt(a, _i64(10)) & _gte(b, _i64(0)) & _lt(b, _i64(10)),
                  vector<Expr>{_add(a, b)});
    auto op_sym = _sym("op", op);
    auto fn = _func("foo", op_sym, vector<Sym>{});
    fn->tbl[op_sym] = op;
    return fn;
}

// filter + sum over 6M rows: TPC-H Q6's Reduce over a SubVector (tpch.h:174-208) plus a count
inline shared_ptr<Func> filter_sum_query()
{
    auto vec = _sym("lineitem", kFilterSum);
    auto red = _red(
        _subvec(vec, _idx(0), _len(vec, 1)), []() { return _new(vector<Expr>{_f64(0), _i64(0)}); },
        [](Expr s, Expr v) {
            auto day = _get(v, 0), price = _get(v, 1), disc = _get(v, 2), q = _get(v, 3);
            auto pred = _gte(day, _i32(730)) & _lt(day, _i32(1095)) & _gte(disc, _f64(0.05)) & _lte(disc, _f64(0.07)) &
                        _lt(q, _f64(24.0));
            return _new(vector<Expr>{_sel(pred, _add(_get(s, 0), _mul(price, disc)), _get(s, 0)),
                                     _sel(pred, _add(_get(s, 1), _i64(1)), _get(s, 1))});
        });
    auto red_sym = _sym("red", red);
    auto fn = _func("filter_sum", red_sym, vector<Sym>{vec});
    fn->tbl[red_sym] = red;
    return fn;
}

// the 6-group aggregation of TPC-H Q1's select-per-group form (tpch.h:412-478)
inline shared_ptr<Func> groupby_query()
{
    auto vec = _sym("lineitem", kGroupBy);
    const std::vector<std::pair<int, int>> groups = {{0, 0}, {0, 1}, {1, 0}, {1, 1}, {2, 0}, {2, 1}};
    auto red = _red(
        _subvec(vec, _idx(0), _len(vec, 1)),
        [groups]() {
            std::vector<Expr> gs;
            for (size_t g = 0; g < groups.size(); g++)
                gs.push_back(_new(vector<Expr>{_f64(0), _f64(0), _f64(0), _f64(0), _f64(0), _i64(0)}));
            return _new(gs);
        },
        [groups](Expr s, Expr v) {
            auto fa = _get(v, 0), fb = _get(v, 1), qty = _get(v, 2), price = _get(v, 3), disc = _get(v, 4),
                 tax = _get(v, 5), day = _get(v, 6);
            Expr disc_price = _mul(price, _sub(_f64(1), disc));
            Expr charge = _mul(disc_price, _add(_f64(1), tax));
            std::vector<Expr> vals = {qty, price, disc_price, charge, disc};
            std::vector<Expr> out;
            for (size_t g = 0; g < groups.size(); g++) {
                Expr c = _eq(fa, _i8(groups[g].first)) & _eq(fb, _i8(groups[g].second)) & _lte(day, _i32(2450));
                Expr sg = _get(s, g);
                std::vector<Expr> fields;
                for (size_t k = 0; k < 5; k++) fields.push_back(_sel(c, _add(_get(sg, k), vals[k]), _get(sg, k)));
                fields.push_back(_sel(c, _add(_get(sg, 5), _i64(1)), _get(sg, 5)));
                out.push_back(_new(fields));
            }
            return _new(out);
        });
    auto red_sym = _sym("red", red);
    std::vector<Expr> outs;
    for (size_t g = 0; g < groups.size(); g++) {
        Expr sg = _get(red_sym, g);
        Expr cnt = _cast(_f64_t, _get(sg, 5));
        outs.push_back(_new(vector<Expr>{_get(sg, 0), _get(sg, 1), _get(sg, 2), _get(sg, 3), _div(_get(sg, 0), cnt),
                                         _div(_get(sg, 1), cnt), _div(_get(sg, 4), cnt), _get(sg, 5)}));
    }
    Expr res = _new(outs);
    auto res_sym = _sym("res", res);
    auto fn = _func("groupby", res_sym, vector<Sym>{vec});
    fn->tbl[red_sym] = red;
    fn->tbl[res_sym] = res;
    return fn;
}

// per key SUM and COUNT: the grouped Op over a 2-d vector (test_multidim.cpp, tpch.h:687-715)
inline shared_ptr<Func> hashgroup_query(const DataType& type = kHashGroup)
{
    auto vec = _sym("vec", type);
    auto t = _sym("key", _i64_t);
    auto red = _red(vec[{t}], []() { return _new(vector<Expr>{_f64(0), _i64(0)}); },
                    [](Expr s, Expr v) {
                        return _new(vector<Expr>{_add(_get(s, 0), _get(v, 0)), _add(_get(s, 1), _i64(1))});
                    });
    auto red_sym = _sym("agg", red);
    auto op = _op(vector<Sym>{t}, _in(t, vec), vector<Expr>{_get(red_sym, 0), _get(red_sym, 1)});
    auto op_sym = _sym("op", op);
    auto fn = _func("group_sum", op_sym, vector<Sym>{vec});
    fn->tbl[red_sym] = red;
    fn->tbl[op_sym] = op;
    return fn;
}

// filtered hash join + aggregate: Locate probes (loopgen.cpp:17-22; tpch.h:51-56)
inline shared_ptr<Func> join_query()
{
    auto build = _sym("build", kJoinBuild);
    auto probe = _sym("probe", kJoinProbe);
    auto red = _red(
        _subvec(probe, _idx(0), _len(probe, 1)),
        []() {
            std::vector<Expr> gs;
            for (int g = 0; g < 5; g++) gs.push_back(_new(vector<Expr>{_f64(0), _i64(0)}));
            return _new(gs);
        },
        [build](Expr s, Expr v) {
            auto fk = _get(v, 0), amount = _get(v, 1), day = _get(v, 2);
            Expr idx = _locate(build, fk);
            Expr attr = _readdata(build, idx, 1);
            Expr base = _gte(idx, _idx(0)) & _lt(attr, _i32(5)) & _gte(day, _i32(0)) & _lt(day, _i32(365));
            std::vector<Expr> out;
            for (int g = 0; g < 5; g++) {
                Expr c = _and(base, _eq(attr, _i32(g)));
                Expr sg = _get(s, g);
                out.push_back(_new(vector<Expr>{_sel(c, _add(_get(sg, 0), amount), _get(sg, 0)),
                                                _sel(c, _add(_get(sg, 1), _i64(1)), _get(sg, 1))}));
            }
            return _new(out);
        });
    auto red_sym = _sym("red", red);
    auto fn = _func("join_agg", red_sym, vector<Sym>{build, probe});
    fn->tbl[red_sym] = red;
    return fn;
}


using QueryList = std::vector<std::pair<const char*, std::function<shared_ptr<Func>()>>>;

inline const QueryList& queries()
{
    static const QueryList qs = {
        {"vector_op", vector_op},       {"transform_op", transform_op},   {"multidim_op", multidim_op},
        {"gen_table_op", gen_table_op}, {"join_op", join_op},             {"nested_op", nested_op},
        {"filter_sum", filter_sum_query}, {"groupby", groupby_query},     {"hashgroup", [] { return hashgroup_query(); }},
        {"join_agg", join_query},
        {"hashgroup_ree", [] { return hashgroup_query(kHashGroupRee); }}};
    return qs;
}

}  // namespace refq
