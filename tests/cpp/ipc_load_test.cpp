// load_arrow_file as a Reffine program calls it (include/reffine/utils/utils.h:56): an Arrow IPC
// file read into an ArrowTable2, its vector type derived from the column formats, and (mode
// "run", needs a GPU) the filter+sum query of TPC-H Q6's shape run on it through compile_op.
//
// usage: ipc_load_test read <file.arrow> <dim>     prints the type, rows and per-column sums
//        ipc_load_test run <file.arrow>            prints the filter+sum result (dim 2)
#include <cstdio>
#include <cstring>
#include <string>

#include "reffine_gb300/utils.h"

using namespace reffine;
using namespace reffine::reffiner;

static double column_sum(const ArrowSchema* s, const ArrowArray* a)
{
    if (std::strcmp(s->format, "+r") == 0) return column_sum(s->children[1], a->children[1]);
    double t = 0;
    const void* buf = a->buffers[1];
    const uint8_t* valid = (const uint8_t*)a->buffers[0];
    for (int64_t i = 0; i < a->length; i++) {
        int64_t j = i + a->offset;
        if (valid && !((valid[j >> 3] >> (j & 7)) & 1)) continue;
        switch (s->format[0]) {
            case 'c': t += ((const int8_t*)buf)[j]; break;
            case 'C': t += ((const uint8_t*)buf)[j]; break;
            case 's': t += ((const int16_t*)buf)[j]; break;
            case 'S': t += ((const uint16_t*)buf)[j]; break;
            case 'i': t += ((const int32_t*)buf)[j]; break;
            case 'I': t += ((const uint32_t*)buf)[j]; break;
            case 'l': t += (double)((const int64_t*)buf)[j]; break;
            case 'L': t += (double)((const uint64_t*)buf)[j]; break;
            case 'f': t += ((const float*)buf)[j]; break;
            case 'g': t += ((const double*)buf)[j]; break;
        }
    }
    return t;
}

static std::shared_ptr<Func> filter_sum(ArrowTable2* tbl)
{
    auto vec = _sym("lineitem", tbl->get_data_type());
    auto red = _red(
        _subvec(vec, _idx(0), _len(vec, 1)), []() { return _new(vector<Expr>{_f64(0), _i64(0)}); },
        [](Expr s, Expr v) {
            auto day = _get(v, 0), price = _get(v, 1), disc = _get(v, 2), q = _get(v, 3);
            auto pred = _gte(day, _i32(100)) & _lt(day, _i32(2000)) & _gte(disc, _f64(0.05)) &
                        _lte(disc, _f64(0.07)) & _lt(q, _f64(24.0));
            return _new(vector<Expr>{_sel(pred, _add(_get(s, 0), _mul(price, disc)), _get(s, 0)),
                                     _sel(pred, _add(_get(s, 1), _i64(1)), _get(s, 1))});
        });
    auto red_sym = _sym("red", red);
    auto fn = _func("filter_sum", red_sym, vector<Sym>{vec});
    fn->tbl[red_sym] = red;
    return fn;
}

int main(int argc, char** argv)
{
    if (argc < 3) return 2;
    std::string mode = argv[1];
    try {
        if (mode == "read") {
            auto tbl = load_arrow_file(argv[2], argc > 3 ? atoll(argv[3]) : 1);
            std::printf("type %s\nrows %lld\n", tbl->get_data_type().str().c_str(), (long long)tbl->array->length);
            for (int64_t c = 0; c < tbl->schema->n_children; c++)
                std::printf("col %s %.17g\n", tbl->schema->children[c]->name,
                            column_sum(tbl->schema->children[c], tbl->array->children[c]));
            return 0;
        }
        if (mode == "run") {
            auto tbl = load_arrow_file(argv[2], 2);
            struct {
                double sum;
                int64_t count;
            } out{};
            auto q = compile_op<void (*)(void*, ArrowTable*)>(filter_sum(tbl.get()));
            q(&out, tbl.get());
            std::printf("filter_sum %.17g %lld\n", out.sum, (long long)out.count);
            return 0;
        }
    } catch (const std::exception& e) {
        std::printf("error %s\n", e.what());
        return 1;
    }
    return 2;
}
