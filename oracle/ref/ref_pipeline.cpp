// Reffine's own CPU compile path, as a C-ABI library for the oracle's tests.
//
// TEST INFRASTRUCTURE ONLY: built by oracle/ref/build_ref.py from a Reffine checkout into
// oracle/_ref/ (never committed), together with Reffine's own sources for the path: the builder,
// the IR, the iteration spaces and the passes LoopGen, CanonPass, ReadWritePass, ScalarPass and
// CEmitter, plus the runtime helpers the generated code calls (make_vector, build_vector_index).
// The product never loads it.
//
// refp_emit runs compile_op's pipeline (include/reffine/utils/utils.h:20-54) on one of the queries
// of ref_queries.h and returns the C++ text CEmitter prints; Reffine hands that text to clang++
// and its JIT (src/pass/llvmgen.cpp:653-696), oracle/ref_pipeline.py to g++ and dlopen.  The
// table functions build Reffine's own ArrowTable2 (include/reffine/arrow/table.h) from Arrow C
// Data Interface structs by copying, and read back the tables the generated code returns.
#include <cstdint>
#include <cstring>
#include <exception>
#include <string>

#include "ref_queries.h"
#include "reffine/arrow/table.h"
#include "reffine/pass/canonpass.h"
#include "reffine/pass/cemitter.h"
#include "reffine/pass/loopgen.h"
#include "reffine/pass/readwritepass.h"
#include "reffine/pass/scalarpass.h"

using namespace reffine;

namespace {

std::string g_err;
std::string g_code;
std::string g_name;

int64_t elem_size(const std::string& fmt)
{
    if (fmt == "c" || fmt == "C") return 1;
    if (fmt == "s" || fmt == "S") return 2;
    if (fmt == "i" || fmt == "I" || fmt == "f") return 4;
    if (fmt == "l" || fmt == "L" || fmt == "g") return 8;
    throw std::runtime_error("unsupported Arrow format " + fmt);
}

char* copy_bytes(const void* src, int64_t n)
{
    if (!src) return nullptr;
    char* d = new char[n > 0 ? n : 1];
    if (n > 0) std::memcpy(d, src, (size_t)n);
    return d;
}

// one primitive child: validity (copied when present, else absent = all valid) and values
ArrowArray2* copy_prim(const ArrowArray* a, const std::string& fmt)
{
    auto* out = new ArrowArray2((size_t)a->length);
    out->length = a->length;
    out->null_count = a->null_count;
    int64_t n = a->length;
    out->add_buffer(copy_bytes(a->n_buffers > 0 ? a->buffers[0] : nullptr, ((n + 15) / 16) * 2));
    out->add_buffer(copy_bytes(a->buffers[1], n * elem_size(fmt)));
    return out;
}

}  // namespace

extern "C" {

const char* refp_error() { return g_err.c_str(); }

// the C++ text of query `name` lowered as compile_op does; nullptr (and refp_error) on failure
const char* refp_emit(const char* name, int vectorize)
{
    try {
        shared_ptr<Func> op;
        for (auto& [n, make] : refq::queries())
            if (std::string(n) == name) op = make();
        if (!op) throw std::runtime_error(std::string("no query named ") + name);
        LoopGen loopgen(nullptr, vectorize != 0);
        loopgen.eval(op);
        auto loop = loopgen.ctx().out_func;
        auto loop1 = CanonPass().eval(loop);
        auto loop2 = ReadWritePass().eval(loop1);
        auto loop3 = ScalarPass().eval(loop2);
        g_code = CEmitter::Build(loop3);
        g_name = loop->name;
        return g_code.c_str();
    } catch (std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

// the generated function's symbol (the Func's name) of the last refp_emit
const char* refp_func_name() { return g_name.c_str(); }

// an ArrowTable2 holding a copy of a struct array ("+s") of primitive or run-end ("+r") columns
void* refp_table_import(int64_t dim, const ArrowSchema* s, const ArrowArray* a)
{
    try {
        auto* t = new ArrowTable2(std::string(s->name ? s->name : "vec"), dim, (size_t)a->length, {}, {});
        t->array->length = a->length;
        auto* sch = static_cast<ArrowSchema2*>(t->schema);
        auto* arr = static_cast<ArrowArray2*>(t->array);
        for (int64_t c = 0; c < s->n_children; c++) {
            const ArrowSchema* cs = s->children[c];
            const ArrowArray* ca = a->children[c];
            std::string fmt = cs->format;
            std::string nm = cs->name ? cs->name : "c" + std::to_string(c);
            if (fmt == "+r") {
                auto* rs = new ArrowSchema2(nm, "+r");
                rs->add_child(new ArrowSchema2("run_ends", "i"));
                rs->add_child(new ArrowSchema2("values", cs->children[1]->format));
                sch->add_child(rs);
                auto* ra = new ArrowArray2((size_t)ca->length);
                ra->length = ca->length;
                ra->add_buffer(nullptr);  // a run-end array has no validity of its own
                ra->add_child(copy_prim(ca->children[0], "i"));
                ra->add_child(copy_prim(ca->children[1], cs->children[1]->format));
                arr->add_child(ra);
            } else {
                sch->add_child(new ArrowSchema2(nm, fmt));
                arr->add_child(copy_prim(ca, fmt));
            }
        }
        return t;
    } catch (std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

// ArrowTable2::build_index (table.h:107-138): the hash index Locate probes
int refp_table_build_index(void* t)
{
    try {
        static_cast<ArrowTable2*>(static_cast<ArrowTable*>(t))->build_index();
        return 0;
    } catch (std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

void refp_table_free(void* t) { delete static_cast<ArrowTable*>(t); }

// readers of a table the generated code made (make_vector, src/vinstr/external.cpp)
int64_t refp_table_len(void* t) { return static_cast<ArrowTable*>(t)->array->length; }
int64_t refp_table_ncols(void* t) { return static_cast<ArrowTable*>(t)->array->n_children; }
const void* refp_col_data(void* t, int64_t c)
{
    return static_cast<ArrowTable*>(t)->array->children[c]->buffers[1];
}
const void* refp_col_validity(void* t, int64_t c)
{
    return static_cast<ArrowTable*>(t)->array->children[c]->buffers[0];
}
int64_t refp_col_null_count(void* t, int64_t c)
{
    return static_cast<ArrowTable*>(t)->array->children[c]->null_count;
}

}  // extern "C"
