// Host side for running the C++ that Reffine's compile path emits (oracle/ref/generated/*.cpp):
// tables over Arrow C Data Interface structs, Locate's hash index, the output tables the emitted
// code asks for, and a timed run of one query on several threads at once.  Benchmark and test
// infrastructure only (the CPU reference arm, the oracle's tests); oracle/ref_generated.py
// compiles it together with one emitted query.
#include <pthread.h>
#include <time.h>

#include <atomic>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "reffine/vinstr/vinstr.h"

namespace {

// an output table made by make_vector: owns its struct array, columns and buffers
struct OutTable {
    ArrowTable t;
    ArrowArray top;
    std::vector<ArrowArray> cols;
    std::vector<ArrowArray*> col_ptrs;
    std::vector<const void*> top_bufs;
    std::vector<std::vector<const void*>> col_bufs;
};

std::mutex g_mu;
std::vector<std::vector<int>> g_out_esize;  // per mem_id: the output columns' element sizes
std::unordered_map<ArrowTable*, OutTable*> g_outputs;  // tables make_vector made, by handle

void add_index(ArrowTable* tbl, const ArrowArray* keys)
{
    // ArrowTable2::build_index (include/reffine/arrow/table.h:107-138): the int64 values of
    // column 0 (the run values of a run-end column), valid rows only, first row of a key kept
    auto* idx = new std::unordered_map<int64_t, int64_t>((size_t)keys->length);
    const uint16_t* bm = keys->n_buffers > 0 ? (const uint16_t*)keys->buffers[0] : nullptr;
    const int64_t* v = (const int64_t*)keys->buffers[1];
    for (int64_t i = 0; i < keys->length; i++)
        if (get_null_bit((uint16_t*)bm, i)) idx->emplace(v[i], i);
    tbl->index = idx;
}

struct Job {
    void* fn;
    int nin;
    void** tables;
    char* out;
};

void* run_job(void* p)
{
    Job* j = (Job*)p;
    // every argument of an emitted query is a pointer: the output slot, then the tables
    if (j->nin == 1)
        ((void (*)(void*, void*))j->fn)(j->out, j->tables[0]);
    else if (j->nin == 2)
        ((void (*)(void*, void*, void*))j->fn)(j->out, j->tables[0], j->tables[1]);
    else if (j->nin == 3)
        ((void (*)(void*, void*, void*, void*))j->fn)(j->out, j->tables[0], j->tables[1], j->tables[2]);
    return nullptr;
}

double now()
{
    timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + ts.tv_nsec * 1e-9;
}

}  // namespace

extern "C" {

void finalize_vector(ArrowTable* tbl, bool* bytemap, int64_t len, int64_t null_count)
{
    ArrowArray* arr = tbl->array;
    for (int64_t c = 0; c < arr->n_children; c++) {
        ArrowArray* col = arr->children[c];
        if (null_count > 0) {
            uint16_t* bm = (uint16_t*)col->buffers[0];
            for (int64_t i = 0; i < len; i++) {
                uint16_t m = (uint16_t)(1u << (i & 15));
                bm[i >> 4] = bytemap[i] ? (uint16_t)(bm[i >> 4] | m) : (uint16_t)(bm[i >> 4] & ~m);
            }
        } else {
            col->buffers[0] = nullptr;
        }
        col->null_count = null_count;
        col->length = len;
    }
    arr->length = len;
}

ArrowTable* make_vector(int64_t len, uint32_t mem_id)
{
    std::vector<int> esize;
    {
        std::lock_guard<std::mutex> g(g_mu);
        if (mem_id < g_out_esize.size()) esize = g_out_esize[mem_id];
    }
    auto* o = new OutTable();
    size_t n = esize.size();
    o->cols.resize(n);
    o->col_ptrs.resize(n);
    o->col_bufs.resize(n);
    for (size_t c = 0; c < n; c++) {
        ArrowArray& a = o->cols[c];
        std::memset(&a, 0, sizeof(a));
        // validity words zeroed, values left as allocated (the emitted code writes every row)
        o->col_bufs[c] = {std::calloc((size_t)(len / 16 + 1), 2), std::malloc((size_t)len * esize[c])};
        a.n_buffers = 2;
        a.buffers = o->col_bufs[c].data();
        o->col_ptrs[c] = &a;
    }
    std::memset(&o->top, 0, sizeof(o->top));
    o->top_bufs = {nullptr};
    o->top.n_buffers = 1;
    o->top.buffers = o->top_bufs.data();
    o->top.n_children = (int64_t)n;
    o->top.children = o->col_ptrs.data();
    o->t.dim = 1;
    o->t.schema = nullptr;
    o->t.array = &o->top;
    o->t.index = nullptr;
    std::lock_guard<std::mutex> g(g_mu);
    g_outputs[&o->t] = o;
    return &o->t;
}

ArrowTable* build_vector_index(ArrowTable* tbl)
{
    ArrowArray* c0 = tbl->array->children[0];
    add_index(tbl, c0->n_children == 2 ? c0->children[1] : c0);
    return tbl;
}

// the column element sizes of the tables make_vector(.., mem_id) returns
int rr_set_output(uint32_t mem_id, int ncols, const int* esize)
{
    std::lock_guard<std::mutex> g(g_mu);
    if (g_out_esize.size() <= mem_id) g_out_esize.resize(mem_id + 1);
    g_out_esize[mem_id].assign(esize, esize + ncols);
    return 0;
}

// a table over the caller's Arrow C structs (borrowed, not copied), with Locate's index when asked
void* rr_table(int64_t dim, ArrowSchema* s, ArrowArray* a, int index)
{
    auto* t = new (std::nothrow) ArrowTable{dim, s, a, nullptr};
    if (t && index) build_vector_index(t);
    return t;
}

void rr_table_free(void* p)
{
    auto* t = (ArrowTable*)p;
    delete t->index;
    delete t;
}

void rr_output_free(ArrowTable* t)
{
    OutTable* o;
    {
        std::lock_guard<std::mutex> g(g_mu);
        auto it = g_outputs.find(t);
        if (it == g_outputs.end()) return;
        o = it->second;
        g_outputs.erase(it);
    }
    for (auto& b : o->col_bufs)
        for (const void* p : b) std::free((void*)p);
    delete o;
}

// runs query `fn` once on each of `nthreads` threads at the same time (threads with 1 GiB stacks:
// the emitted code keeps a 100 MB bytemap on the stack); thread i writes its result to
// out + i * out_bytes.  Returns the wall time from the first start to the last finish, or -1.
double rr_run(void* fn, int nthreads, int nin, void** tables, char* out, int64_t out_bytes)
{
    std::vector<pthread_t> th((size_t)nthreads);
    std::vector<Job> jobs((size_t)nthreads);
    pthread_attr_t attr;
    pthread_attr_init(&attr);
    pthread_attr_setstacksize(&attr, (size_t)1 << 30);
    double t0 = now();
    int started = 0;
    for (int i = 0; i < nthreads; i++) {
        jobs[i] = Job{fn, nin, tables, out + (int64_t)i * out_bytes};
        if (pthread_create(&th[i], &attr, run_job, &jobs[i]) != 0) break;
        started++;
    }
    for (int i = 0; i < started; i++) pthread_join(th[i], nullptr);
    double dt = now() - t0;
    pthread_attr_destroy(&attr);
    return started == nthreads ? dt : -1.0;
}

}  // extern "C"
