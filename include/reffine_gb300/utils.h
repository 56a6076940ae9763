// compile_op for the GB300 backend: the call Reffine programs make, unchanged.
//
// Reference: template <typename T> T compile_op(shared_ptr<Func> op, bool vectorize = false)
// (include/reffine/utils/utils.h:47-54) lowers the Func, JIT-compiles it and returns the raw
// function pointer of `extern "C" void name(OutT* output_addr, inputs...)`.  Here the Func is
// lowered onto the GPU kernel templates and compiled for sm_103a (rf_plan_compile); the returned
// pointer has the same type and calling shape (rf_plan_thunk): tables are `ArrowTable*` in host
// memory, the result is written through `output_addr`.  Plans live as long as the process, as
// the reference's JIT modules do.
//
// ArrowTable2 mirrors the reference's owning table (include/reffine/arrow/table.h:15-151):
// (name, dim, len, column names, types) allocates flat columns; (dim) is an empty table that
// adopts Arrow C data (load_arrow_file fills it); get_data_type() derives the vector type from
// the column formats (a "+r" child is run-end encoded).
//
// load_arrow_file(filename, dim) (include/reffine/utils/utils.h:56, src/utils/utils.cpp:11-34)
// reads record batch 0 of an Arrow IPC file with the library's own parser (rf_ipc_read: integer,
// float and run-end encoded columns; compressed bodies and dictionaries are refused) and throws
// std::runtime_error with the parser's message on failure, where the reference aborts through
// ValueOrDie.
#pragma once

#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "reffine_gb300/arrow_table.h"
#include "reffine_gb300/ir.h"
#include "rf_gpu.h"

namespace reffine {

// One device context for the process (the role of ExecEngine::Get, src/engine/engine.cpp:24-39).
class GpuEngine {
public:
    static GpuEngine* Get()
    {
        static GpuEngine e;
        return &e;
    }
    rf_ctx* ctx() const { return ctx_; }
    rf_plan* compile(const Func& fn, bool vectorize)
    {
        rf_plan* plan = nullptr;
        std::string text = to_text(fn);
        if (rf_plan_compile(ctx_, text.c_str(), vectorize ? 1 : 0, &plan) != RF_OK)
            throw std::runtime_error(std::string("compile_op: ") + rf_last_error(ctx_));
        std::lock_guard<std::mutex> g(mu_);
        plans_.push_back(plan);
        return plan;
    }
    ~GpuEngine()
    {
        for (auto* p : plans_) rf_plan_free(p);
        if (ctx_) rf_gpu_shutdown(ctx_);
    }

private:
    GpuEngine()
    {
        const char* d = getenv("RF_DEVICE");
        if (rf_gpu_init(d ? atoi(d) : 0, &ctx_) != RF_OK)
            throw std::runtime_error("reffine_gb300: no usable GPU (rf_gpu_init failed)");
    }
    rf_ctx* ctx_ = nullptr;
    std::mutex mu_;
    std::vector<rf_plan*> plans_;
};

template <typename T>
T compile_op(std::shared_ptr<Func> op, bool vectorize = false)
{
    rf_plan* plan = GpuEngine::Get()->compile(*op, vectorize);
    void* fn = nullptr;
    if (rf_plan_thunk(plan, &fn) != RF_OK) throw std::runtime_error("compile_op: no free query-function slot");
    return reinterpret_cast<T>(fn);
}

// ---- an owning host table in Reffine's layout -------------------------------------------------
struct ArrowTable2 : public ArrowTable {
    // an empty table whose schema/array are filled by a producer of Arrow C data
    // (table.h:16-22); the producer's release callbacks run when the table is destroyed
    explicit ArrowTable2(int64_t dim) : ArrowTable(dim)
    {
        std::memset(&top_s_, 0, sizeof top_s_);
        std::memset(&top_a_, 0, sizeof top_a_);
        schema = &top_s_;
        array = &top_a_;
    }

    ArrowTable2(std::string name, int64_t dim, size_t len, std::vector<std::string> cols, std::vector<DataType> dtypes)
        : ArrowTable(dim), name_(std::move(name))
    {
        if (cols.size() != dtypes.size()) throw std::runtime_error("ArrowTable2: names and types differ in count");
        size_t n = cols.size();
        names_ = cols;
        types_ = dtypes;
        child_s_.resize(n);
        child_a_.resize(n);
        bufs_.resize(n);
        valid_.resize(n);
        fmts_.resize(n);
        for (size_t i = 0; i < n; i++) {
            fmts_[i] = format_of(dtypes[i]);
            bufs_[i].assign(len * dtypes[i].size() + 16, 0);
            valid_[i].assign((len / 16 + 1) * 2, 0xff);
            ArrowSchema& s = child_s_[i];
            std::memset(&s, 0, sizeof s);
            s.format = fmts_[i].c_str();
            s.name = names_[i].c_str();
            s.flags = ARROW_FLAG_NULLABLE;
            ArrowArray& a = child_a_[i];
            std::memset(&a, 0, sizeof a);
            a.length = (int64_t)len;
            a.n_buffers = 2;
            child_bufs_.push_back({nullptr, bufs_[i].data()});
        }
        for (size_t i = 0; i < n; i++) {
            child_a_[i].buffers = child_bufs_[i].data();
            sp_.push_back(&child_s_[i]);
            ap_.push_back(&child_a_[i]);
        }
        std::memset(&top_s_, 0, sizeof top_s_);
        top_s_.format = "+s";
        top_s_.name = name_.c_str();
        top_s_.n_children = (int64_t)n;
        top_s_.children = sp_.data();
        std::memset(&top_a_, 0, sizeof top_a_);
        top_a_.length = (int64_t)len;
        top_a_.n_buffers = 1;
        top_a_.buffers = top_bufs_;
        top_a_.n_children = (int64_t)n;
        top_a_.children = ap_.data();
        schema = &top_s_;
        array = &top_a_;
    }

    // the values buffer of column c
    template <typename V>
    V* data(size_t c)
    {
        return reinterpret_cast<V*>(bufs_.at(c).data());
    }

    ~ArrowTable2() override
    {
        if (top_a_.release) top_a_.release(&top_a_);
        if (top_s_.release) top_s_.release(&top_s_);
    }
    ArrowTable2(const ArrowTable2&) = delete;
    ArrowTable2& operator=(const ArrowTable2&) = delete;

    // ArrowTable2::get_data_type (table.h:64-80): one element type per child, "+r" = run-end
    DataType get_data_type() const
    {
        std::vector<DataType> dts;
        std::vector<EncodeType> enc;
        for (int64_t i = 0; i < schema->n_children; i++) {
            const ArrowSchema* c = schema->children[i];
            bool ree = std::strcmp(c->format, "+r") == 0;
            dts.push_back(dtype_of(ree ? c->children[1]->format : c->format));
            enc.push_back(ree ? RUNEND : FLAT);
        }
        return DataType(VECTOR, dts, (size_t)dim, enc);
    }

    // the GPU backend builds its own device index when a query probes this table
    void build_index() {}

private:
    // arrow_to_dtype (table.h:82-104), with the unsigned widths the IPC reader also produces
    static DataType dtype_of(const char* f)
    {
        static const char* fmts = "csilCSILfg";
        static const BaseType bts[] = {INT8, INT16, INT32, INT64, UINT8, UINT16, UINT32, UINT64, FLOAT32, FLOAT64};
        if (f && f[0] && !f[1])
            for (int k = 0; fmts[k]; k++)
                if (fmts[k] == f[0]) return DataType(bts[k]);
        throw std::runtime_error(std::string("schema type not supported ") + (f ? f : "(null)"));
    }
    static std::string format_of(const DataType& t)
    {
        switch (t.btype) {
            case BOOL: case INT8: return "c";
            case INT16: return "s";
            case INT32: return "i";
            case INT64: case IDX: return "l";
            case FLOAT32: return "f";
            case FLOAT64: return "g";
            default: throw std::runtime_error("data type not supported " + t.str());
        }
    }
    std::string name_;
    std::vector<std::string> names_, fmts_;
    std::vector<DataType> types_;
    std::vector<ArrowSchema> child_s_;
    std::vector<ArrowArray> child_a_;
    std::vector<std::vector<unsigned char>> bufs_, valid_;
    std::vector<std::vector<const void*>> child_bufs_;
    std::vector<ArrowSchema*> sp_;
    std::vector<ArrowArray*> ap_;
    ArrowSchema top_s_;
    ArrowArray top_a_;
    const void* top_bufs_[1] = {nullptr};
};

inline std::shared_ptr<ArrowTable2> load_arrow_file(std::string filename, int64_t dim)
{
    auto tbl = std::make_shared<ArrowTable2>(dim);
    char err[512];
    if (rf_ipc_read(filename.c_str(), tbl->schema, tbl->array, err, sizeof err) != RF_OK)
        throw std::runtime_error("load_arrow_file: " + std::string(err));
    return tbl;
}

}  // namespace reffine
