// Objects behind the C-ABI handles (rf_ctx, rf_table, rf_plan), shared by the runtime's
// translation units.
#pragma once

#include <cuda.h>
#include <cuda_runtime_api.h>

#include <algorithm>
#include <atomic>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "device/rf_params.h"
#include "lower.h"
#include "rf_gpu.h"

namespace rfrt {

// ------------------------------------------------------------------------------------------
// driver API entry points (resolved through the runtime, so the library does not link libcuda)
// ------------------------------------------------------------------------------------------
struct Driver {
    CUresult (*ModuleLoadData)(CUmodule*, const void*) = nullptr;
    CUresult (*ModuleUnload)(CUmodule) = nullptr;
    CUresult (*ModuleGetFunction)(CUfunction*, CUmodule, const char*) = nullptr;
    CUresult (*LaunchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                             CUstream, void**, void**) = nullptr;
    CUresult (*FuncSetAttribute)(CUfunction, CUfunction_attribute, int) = nullptr;
    CUresult (*FuncGetAttribute)(int*, CUfunction_attribute, CUfunction) = nullptr;
    CUresult (*GraphAddKernelNode)(CUgraphNode*, CUgraph, const CUgraphNode*, size_t,
                                   const CUDA_KERNEL_NODE_PARAMS*) = nullptr;
    CUresult (*OccupancyMaxActiveBlocksPerMultiprocessor)(int*, CUfunction, int, size_t) = nullptr;
    CUresult (*GetErrorString)(CUresult, const char**) = nullptr;
    bool ok = false;
    std::string err;
};

inline Driver& drv()
{
    static Driver d;
    static std::once_flag once;
    std::call_once(once, [] {
        auto get = [&](const char* name, void** fn) -> bool {
            cudaDriverEntryPointQueryResult q;
            cudaError_t e = cudaGetDriverEntryPointByVersion(name, fn, 12000, cudaEnableDefault, &q);
            if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !*fn) {
                d.err = std::string("driver entry point unavailable: ") + name;
                return false;
            }
            return true;
        };
        d.ok = get("cuModuleLoadData", (void**)&d.ModuleLoadData) && get("cuModuleUnload", (void**)&d.ModuleUnload) &&
               get("cuModuleGetFunction", (void**)&d.ModuleGetFunction) &&
               get("cuLaunchKernel", (void**)&d.LaunchKernel) && get("cuFuncSetAttribute", (void**)&d.FuncSetAttribute) &&
               get("cuFuncGetAttribute", (void**)&d.FuncGetAttribute) &&
               get("cuGraphAddKernelNode", (void**)&d.GraphAddKernelNode) &&
               get("cuOccupancyMaxActiveBlocksPerMultiprocessor", (void**)&d.OccupancyMaxActiveBlocksPerMultiprocessor) &&
               get("cuGetErrorString", (void**)&d.GetErrorString);
    });
    return d;
}


}  // namespace rfrt

using rfrt::drv;

// ------------------------------------------------------------------------------------------
// objects
// ------------------------------------------------------------------------------------------
struct JitModule {
    CUmodule mod = nullptr;
    std::map<std::string, CUfunction> fns;
    std::string log;
    ~JitModule()
    {
        if (mod && drv().ok) drv().ModuleUnload(mod);
    }
};

struct rf_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::mutex mu;
    std::mutex err_mu;                // guards err (written by any thread that fails)
    std::string err;
    std::map<std::string, std::shared_ptr<JitModule>> modules;
    std::atomic<long long> launches{0};
    int sm_count = 0;
    int pageable_direct = 0;  // cudaDevAttrPageableMemoryAccessUsesHostPageTables
    int* dev_err = nullptr;  // device error word shared by this context's launches
    // autotuner choices: tile rows per (query shape key, log2 row-count bucket)
    std::mutex tune_mu;
    std::map<std::string, std::map<int, long long>> tune;
    // row-chunked runs (run_streamed): a copy stream beside `stream`, one event per chunk
    std::mutex pipe_mu;
    cudaStream_t copy_stream = nullptr;
    std::vector<cudaEvent_t> pipe_ev;
    // pinned staging ring for host copies from files and pageable memory (staged_h2d)
    std::mutex stage_mu;
    unsigned char* stage = nullptr;
    cudaEvent_t stage_ev[2] = {nullptr, nullptr};
    // filtered join indexes kept by plans between runs (filtered_index): held under ixf_mu from
    // the lookup until the run's kernels are enqueued and its event recorded; at most
    // ixf_budget bytes in all, the plan used longest ago giving its index up first
    std::mutex ixf_mu;
    std::list<rf_plan*> ixf_lru;      // plans holding an index, least recently used first
    size_t ixf_bytes = 0;
    size_t ixf_budget = 0;
};

struct DevCol {
    reffine::DataType type;
    bool runend = false;
    void* data = nullptr;             // values (run values)
    long long nvals = 0;
    unsigned short* valid = nullptr;  // validity of the values (NULL: all valid)
    int* run_ends = nullptr;
    long long logical = 0;            // rows
    std::string name;
    // allocations behind the pointers above (reused by repeated uploads into the same table)
    void* data_buf = nullptr;
    void* valid_buf = nullptr;
    void* re_buf = nullptr;
    size_t data_cap = 0, valid_cap = 0, re_cap = 0;
};

inline unsigned long long next_table_gen()
{
    static std::atomic<unsigned long long> g{0};
    return ++g;
}

struct rf_table {
    rf_ctx* ctx = nullptr;
    unsigned long long gen = next_table_gen();  // unique per table object, for caches keyed on tables
    long long dim = 1;
    std::vector<DevCol> cols;
    std::vector<char> present;        // column uploaded
    long long* ix_slots = nullptr;
    unsigned long long ix_cap = 0;
    long long* ix_special = nullptr;  // [empty-key row][repeated-key flag (int)]
    int ix_unique = -1;               // 1: no key repeats (read once from the flag), -1: unknown
    bool has_index = false;
    long long null_count = 0;
    std::string name;
    std::vector<long long> ndv;       // cached distinct-count estimates per column (-1: unknown)
    // hash group-by: the hottest keys of column 0, from a sample, most frequent first
    bool hot_ready = false;
    std::vector<long long> hot;
    std::mutex stats_mu;              // guards ndv and hot (runs on several streams may share a table)
};

struct rf_plan {
    rf_ctx* ctx = nullptr;
    std::string text;                 // the Func's text (the autotuner recompiles variants from it)
    std::string shape;                // shape key at the default block size (tuning entries)
    std::vector<rf_table*> staging;   // device copies of the host tables of thunk calls
    rfg::Plan plan;
    std::shared_ptr<JitModule> mod;
    std::vector<CUfunction> fns;
    void* buf = nullptr;              // the allocation holding partials .. d_res below
    void* partials = nullptr;
    size_t partials_bytes = 0;
    unsigned* counter = nullptr;
    long long* range = nullptr;
    unsigned char* dout = nullptr;
    int max_units = 0;                // resident blocks of the main kernel (one wave)
    int reduce_units = 0;             // work units a reduce may be cut into (units_for)
    int thunk_slot = -1;
    long long tile_override = 0;      // set while the autotuner times a candidate
    unsigned char* h_res = nullptr;   // pinned: [error word, 16 B][value result]
    // batched execution (value-output plans without device-computed loop bounds)
    CUfunction batch_fn = nullptr;
    int batch_grid = 0;
    size_t batch_smem = 0;
    int batch_threads = 0;
    // table outputs
    void** d_ptrs = nullptr;          // device array: output column pointers, then bitmap pointers
    long long* d_tiles = nullptr;     // per-tile counts / offsets
    size_t tiles_cap = 0;             // bytes
    long long* d_res = nullptr;       // [rows written, null count]
    // hash group-by
    void* hg_keys = nullptr;
    void* hg_acc = nullptr;
    size_t hg_keys_cap = 0, hg_acc_cap = 0;
    long long hg_retry_cap = 0;
    int hg_factor_override = 0;       // set while the autotuner times a hash-table sizing
    void* hg_img = nullptr;           // hot-key image of the last input table (device)
    size_t hg_img_cap = 0;
    unsigned long long hg_img_for = 0;  // generation of the table the image was built for
    bool hg_img_some = false;         // the image holds at least one key
    // filtered index of a probed table (plans with a pushed-down filter): its entry count
    unsigned long long ixf_for = 0;   // generation of the table whose kept-entry count is ixf_count
    long long ixf_count = 0;
    // ... and the index itself, kept for the next run on the same table (0: none kept)
    void* ixf_buf = nullptr;
    size_t ixf_buf_bytes = 0;
    unsigned long long ixf_buf_for = 0;
    RfIndex ixf_ix{};
    cudaEvent_t ixf_ev = nullptr;     // recorded after the last run that read ixf_buf
    // segmented reduce
    long long* seg_woff = nullptr;
    long long* seg_tmp = nullptr;
    void* seg_part = nullptr;
    size_t seg_runs_cap = 0, seg_part_cap = 0, seg_tmp_cap = 0;
};

// Work units of a value reduce over `ntiles` tiles: up to kUnitWaves waves of resident blocks.
// Every path of a plan (alone, batched, served, row-chunked, no-alloc) takes its units from
// here, so a query folds the same partials in the same order whichever path runs it.  Several
// waves let a row-chunked run launch a full wave per chunk of rows.
constexpr int kUnitWaves = 8;
inline int units_for(const rf_plan* p, long long ntiles)
{
    return (int)std::min<long long>(std::max<long long>(ntiles, 1), p->reduce_units);
}

// cudaMallocAsync from the device's stream-ordered pool.  The pool keeps freed blocks (its release
// threshold is unlimited, so per-run buffers are reused without going back to the driver); when it
// cannot grow any more, its unused memory is handed back to the device and the allocation is tried
// again - first once `s`'s work is done, then once the whole device's is.
inline cudaError_t pool_alloc(void** p, size_t bytes, cudaStream_t s)
{
    cudaError_t e = cudaMallocAsync(p, bytes, s);
    if (e != cudaErrorMemoryAllocation) return e;
    cudaGetLastError();
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess) return e;
    cudaStreamSynchronize(s);
    cudaMemPoolTrimTo(pool, 0);
    e = cudaMallocAsync(p, bytes, s);
    if (e != cudaErrorMemoryAllocation) return e;
    cudaGetLastError();
    cudaDeviceSynchronize();
    cudaMemPoolTrimTo(pool, 0);
    return cudaMallocAsync(p, bytes, s);
}

namespace {
// Grows a device buffer to at least `bytes` (contents not kept), stream-ordered on `s`: the old
// buffer is released after the work already queued on `s`, and nothing synchronises the device
// (a cudaFree would stall every stream, including other threads' batches).  The buffer must be
// used on `s` only, or after the caller has synchronised with `s`.
bool grow(void** buf, size_t* cap, size_t bytes, cudaStream_t s)
{
    if (*buf && *cap >= bytes) return true;
    if (*buf) cudaFreeAsync(*buf, s);
    *buf = nullptr;
    *cap = 0;
    if (pool_alloc(buf, bytes, s) != cudaSuccess) return false;
    *cap = bytes;
    return true;
}
}  // namespace


namespace rfrt {
int launch(rf_ctx* ctx, CUfunction f, int grid, int block, size_t smem, cudaStream_t s, RfParams* P);
int fail(rf_ctx* ctx, int code, const char* fmt, ...);
int check_device_error(rf_ctx* ctx);
int device_error(rf_ctx* ctx, int e);  // RF_OK for 0, else clears the context's error word and fails
long long tile_rows_for(rf_plan* p, long long rows);  // the tiling a run of `rows` rows uses
int hg_factor_for(rf_plan* p, long long rows);        // hash group-by slots per 100 distinct keys
void batch_set_share(rf_batch* b, int pct);
// runs from this thread size a hash aggregation's grid at pct % of its resident blocks (a serving
// table lane leaves room for the batch lanes; grid-stride kernel, results do not depend on it)
void set_thread_grid_share(int pct);
int cu_fail(rf_ctx* ctx, CUresult r, const char* what);
}  // namespace rfrt

#define CUDA_TRY(ctx, call)                                                                      \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess)                                                                   \
            return rfrt::fail(ctx, RF_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)
