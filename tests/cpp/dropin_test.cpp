// A Reffine program, written the way the reference's tests are (test/src/test_reduce.cpp:61-122,
// test/src/test_transform.cpp:9-53), compiled against this backend's headers: the query is built
// with the same builder calls, compiled with compile_op<FnTy> and called through the returned
// function pointer with ArrowTable* inputs.
//
// usage: dropin_test <students.bin>   (int64 row count, then 6 int64 columns)
#include <cstdio>
#include <fstream>
#include <vector>

#include "reffine_gb300/utils.h"

using namespace reffine;
using namespace reffine::reffiner;

static std::shared_ptr<Func> vector_op(ArrowTable2* tbl)
{
    auto t_sym = _sym("t", _i64_t);
    auto vec_in_sym = _sym("vec_in", tbl->get_data_type());
    auto op = _op(vector<Sym>{t_sym}, _in(t_sym, vec_in_sym) & _lte(t_sym, _i64(48)) & _gte(t_sym, _i64(10)),
                  vector<Expr>{
                      vec_in_sym[{t_sym}][2],
                      _new(vector<Expr>{
                          vec_in_sym[{t_sym}][1],
                          vec_in_sym[{t_sym}][2],
                          vec_in_sym[{t_sym}][0],
                          vec_in_sym[{t_sym}][3],
                      }),
                      vec_in_sym[{t_sym}][3],
                  });
    auto sum = _red(
        op,
        []() {
            return _new(vector<Expr>{
                _new(vector<Expr>{_i64(0), _i64(0)}),
                _new(vector<Expr>{_i64(0), _i64(0)}),
            });
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
            return _new(vector<Expr>{
                _new(vector<Expr>{_add(s0, v0), _add(s1, v1)}),
                _new(vector<Expr>{_add(s2, v2), _add(s3, v3)}),
            });
        });
    auto sum_sym = _sym("sum", sum);
    auto res = _get(_get(sum_sym, 1), 0);
    auto res_sym = _sym("res", res);

    auto foo_fn = _func("foo", res_sym, vector<Sym>{vec_in_sym});
    foo_fn->tbl[sum_sym] = sum;
    foo_fn->tbl[res_sym] = res;
    return foo_fn;
}

static std::shared_ptr<Func> transform_op(ArrowTable2* tbl, long lb, long n)
{
    auto t_sym = _sym("t", _i64_t);
    auto vec_in_sym = _sym("vec_in", tbl->get_data_type());
    auto elem = vec_in_sym[{t_sym}];
    auto elem_sym = _sym("elem", elem);
    auto out = _add(elem_sym[0], _i64(n));
    auto out_sym = _sym("out", out);
    auto op = _op(vector<Sym>{t_sym}, _in(t_sym, vec_in_sym) & _gt(t_sym, _i64(lb)), vector<Expr>{out_sym});
    auto op_sym = _sym("op", op);

    auto foo_fn = _func("foo", op_sym, vector<Sym>{vec_in_sym});
    foo_fn->tbl[elem_sym] = elem;
    foo_fn->tbl[out_sym] = out;
    foo_fn->tbl[op_sym] = op;
    return foo_fn;
}

int main(int argc, char** argv)
{
    if (argc < 2) return 2;
    std::ifstream f(argv[1], std::ios::binary);
    int64_t n = 0;
    f.read((char*)&n, 8);
    std::vector<std::string> names{"id", "hours_studied", "attendance", "sleep_hours", "previous_scores", "exam_score"};
    std::vector<DataType> types(6, types::INT64_T);
    ArrowTable2 tbl("students", 1, (size_t)n, names, types);
    for (int c = 0; c < 6; c++) f.read((char*)tbl.data<int64_t>(c), n * 8);

    // ReduceOpTest: golden 696 (test_reduce.cpp:121)
    long output = 0;
    auto query_fn = compile_op<void (*)(long*, void*)>(vector_op(&tbl));
    query_fn(&output, &tbl);
    printf("reduce_op %ld\n", output);

    // TransformOpTest (test_transform.cpp:31-53)
    ArrowTable* out_tbl = nullptr;
    auto tfn = compile_op<void (*)(ArrowTable**, ArrowTable*)>(transform_op(&tbl, 5, 10));
    tfn(&out_tbl, &tbl);
    int64_t len = out_tbl->array->length;
    auto* in0 = tbl.data<int64_t>(0);
    auto* in1 = tbl.data<int64_t>(1);
    auto* o0 = (const int64_t*)out_tbl->array->children[0]->buffers[1];
    auto* o1 = (const int64_t*)out_tbl->array->children[1]->buffers[1];
    long bad = 0;
    for (int64_t i = 5; i < n; i++)
        if (in0[i] != o0[i - 5] || in1[i] + 10 != o1[i - 5]) bad++;
    printf("transform len %ld expect %ld mismatches %ld\n", (long)len, (long)(n - 5), bad);
    return (output == 696 && len == n - 5 && bad == 0) ? 0 : 1;
}
