// C-ABI runtime of the GB300 backend (include/rf_gpu.h).
//
// Replaces, for the compiled-query path, Reffine's ExecEngine/CudaEngine (src/engine/*.cpp):
// a query is lowered (lower.cpp), its CUDA source compiled by NVRTC for sm_103a and loaded
// through the driver API; tables live in device memory; runs are stream-ordered.
#include <cuda.h>
#include <cuda_runtime_api.h>
#include <nvrtc.h>

#include <algorithm>
#include <chrono>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <condition_variable>
#include <vector>

#include <dlfcn.h>
#include <execinfo.h>
#include <signal.h>
#include <unistd.h>

#include "arrow_c.h"
#include "device/rf_params.h"
#include "kernels.h"
#include "lower.h"
#include "rf_gpu.h"
#include "objects.h"
#include "runtime.h"

namespace {

const char* k_device_src =
#include "rf_device.cuh.inc"
    ;
const char* k_templates_src =
#include "rf_templates.cuh.inc"
    ;
const char* k_params_src =
#include "rf_params.h.inc"
    ;

}  // namespace


// ------------------------------------------------------------------------------------------
// helpers
// ------------------------------------------------------------------------------------------
namespace rfrt {

int fail(rf_ctx* ctx, int code, const char* fmt, ...)
{
    char buf[4096];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (ctx) {
        std::lock_guard<std::mutex> g(ctx->err_mu);
        ctx->err = buf;
    }
    return code;
}

int cu_fail(rf_ctx* ctx, CUresult r, const char* what)
{
    const char* s = "?";
    if (drv().GetErrorString) drv().GetErrorString(r, &s);
    return fail(ctx, RF_ERR_CUDA, "%s failed: %s", what, s);
}

}  // namespace rfrt

using rfrt::cu_fail;
using rfrt::fail;

namespace {

bool parse_format(const char* f, reffine::DataType& t)
{
    using namespace reffine;
    std::string s(f ? f : "");
    if (s == "c") t = DataType(INT8);
    else if (s == "C") t = DataType(UINT8);
    else if (s == "s") t = DataType(INT16);
    else if (s == "S") t = DataType(UINT16);
    else if (s == "i") t = DataType(INT32);
    else if (s == "I") t = DataType(UINT32);
    else if (s == "l") t = DataType(INT64);
    else if (s == "L") t = DataType(UINT64);
    else if (s == "f") t = DataType(FLOAT32);
    else if (s == "g") t = DataType(FLOAT64);
    else return false;
    return true;
}

const char* format_of(const reffine::DataType& t)
{
    using namespace reffine;
    switch (t.btype) {
        case BOOL: case INT8: return "c";
        case UINT8: return "C";
        case INT16: return "s";
        case UINT16: return "S";
        case INT32: return "i";
        case UINT32: return "I";
        case INT64: case IDX: return "l";
        case UINT64: return "L";
        case FLOAT32: return "f";
        case FLOAT64: return "g";
        default: return "?";
    }
}

long long eval_host(const rfg::HostExpr& h, const rf_arg* args, int n_args, bool& ok)
{
    switch (h.kind) {
        case rfg::HostExpr::CONST: return h.value;
        case rfg::HostExpr::LEN: {
            if (h.input >= n_args || args[h.input].kind != RF_ARG_TABLE || !args[h.input].table) {
                ok = false;
                return 0;
            }
            auto* t = args[h.input].table;
            if (h.col >= (int)t->cols.size()) {
                ok = false;
                return 0;
            }
            return t->cols[h.col].nvals;
        }
        case rfg::HostExpr::SCALAR:
            if (h.input >= n_args) {
                ok = false;
                return 0;
            }
            return args[h.input].kind == RF_ARG_F64 ? (long long)args[h.input].f64 : args[h.input].i64;
        case rfg::HostExpr::ADD: return eval_host(h.args[0], args, n_args, ok) + eval_host(h.args[1], args, n_args, ok);
        case rfg::HostExpr::SUB: return eval_host(h.args[0], args, n_args, ok) - eval_host(h.args[1], args, n_args, ok);
        case rfg::HostExpr::MUL: return eval_host(h.args[0], args, n_args, ok) * eval_host(h.args[1], args, n_args, ok);
        case rfg::HostExpr::MAX: {
            long long a = eval_host(h.args[0], args, n_args, ok), b = eval_host(h.args[1], args, n_args, ok);
            return a > b ? a : b;
        }
        case rfg::HostExpr::MIN: {
            long long a = eval_host(h.args[0], args, n_args, ok), b = eval_host(h.args[1], args, n_args, ok);
            return a < b ? a : b;
        }
        default: ok = false; return 0;
    }
}

std::string nvrtc_arch()
{
    const char* a = getenv("RF_GPU_ARCH");
    return std::string("--gpu-architecture=") + (a && *a ? a : "sm_103a");
}

}  // namespace

// ------------------------------------------------------------------------------------------
// JIT
// ------------------------------------------------------------------------------------------
namespace rfrt {

// compiles a generated query source for sm_103a; on failure `log` holds the message
bool nvrtc_compile(const std::string& src, std::string& cubin, std::string& log)
{
    nvrtcProgram prog;
    const char* hdrs[] = {k_device_src, k_templates_src, k_params_src};
    const char* names[] = {"rf_device.cuh", "rf_templates.cuh", "rf_params.h"};
    if (nvrtcCreateProgram(&prog, src.c_str(), "query.cu", 3, hdrs, names) != NVRTC_SUCCESS) {
        log = "nvrtcCreateProgram failed";
        return false;
    }
    std::string arch = nvrtc_arch();
    // --fmad=false: products are rounded before sums, as the reference's C++ does with
    // -ffp-contract=off; results then match the serial CPU loop per row
    const char* opts[] = {arch.c_str(), "-std=c++17", "--fmad=false", "-lineinfo"};
    nvrtcResult r = nvrtcCompileProgram(prog, 4, opts);
    size_t lsz = 0;
    nvrtcGetProgramLogSize(prog, &lsz);
    std::string l(lsz, '\0');
    if (lsz) nvrtcGetProgramLog(prog, &l[0]);
    if (r != NVRTC_SUCCESS) {
        nvrtcDestroyProgram(&prog);
        log = std::string("NVRTC compile failed: ") + nvrtcGetErrorString(r) + "\n" + l + "\n--- source ---\n" + src;
        return false;
    }
    size_t csz = 0;
    nvrtcGetCUBINSize(prog, &csz);
    cubin.assign(csz, '\0');
    nvrtcGetCUBIN(prog, &cubin[0]);
    nvrtcDestroyProgram(&prog);
    log = l;
    return true;
}

int jit_compile(rf_ctx* ctx, const std::string& key, const std::string& src, std::shared_ptr<JitModule>& out,
                std::string* cubin_out)
{
    {
        std::lock_guard<std::mutex> g(ctx->mu);
        auto it = ctx->modules.find(key);
        if (it != ctx->modules.end()) {
            out = it->second;
            return RF_OK;
        }
    }
    std::string cubin, log;
    if (!nvrtc_compile(src, cubin, log)) return fail(ctx, RF_ERR_JIT, "%s", log.c_str());
    if (cubin_out) *cubin_out = cubin;
    auto m = std::make_shared<JitModule>();
    m->log = log;
    if (!drv().ok) return fail(ctx, RF_ERR_CUDA, "%s", drv().err.c_str());
    CUresult cr = drv().ModuleLoadData(&m->mod, cubin.data());
    if (cr != CUDA_SUCCESS) return cu_fail(ctx, cr, "cuModuleLoadData");
    std::lock_guard<std::mutex> g(ctx->mu);
    ctx->modules[key] = m;
    out = m;
    return RF_OK;
}

int get_function(rf_ctx* ctx, JitModule& m, const std::string& name, CUfunction& f)
{
    auto it = m.fns.find(name);
    if (it != m.fns.end()) {
        f = it->second;
        return RF_OK;
    }
    CUresult cr = drv().ModuleGetFunction(&f, m.mod, name.c_str());
    if (cr != CUDA_SUCCESS) return cu_fail(ctx, cr, "cuModuleGetFunction");
    m.fns[name] = f;
    return RF_OK;
}

int launch(rf_ctx* ctx, CUfunction f, int grid, int block, size_t smem, cudaStream_t s, RfParams* P)
{
    void* args[] = {P};
    CUresult cr = drv().LaunchKernel(f, grid, 1, 1, block, 1, 1, (unsigned)smem, (CUstream)s, args, nullptr);
    if (cr != CUDA_SUCCESS) return cu_fail(ctx, cr, "cuLaunchKernel");
    ctx->launches++;
    return RF_OK;
}

}  // namespace rfrt

using namespace rfrt;

namespace {
thread_local int t_grid_share = 100;  // set_thread_grid_share
}
void rfrt::set_thread_grid_share(int pct) { t_grid_share = std::min(100, std::max(1, pct)); }

// ------------------------------------------------------------------------------------------
// crash report (opt-in diagnostics: RF_CRASH_TRACE=1 in the environment)
// ------------------------------------------------------------------------------------------
// On SIGSEGV / SIGBUS / SIGABRT in any thread, writes the faulting thread's native frames to
// stderr (each with its object file and the offset inside it, for addr2line), then hands the
// signal to the handler installed before (Python's faulthandler prints the Python frames).
namespace {
struct sigaction g_prev_segv, g_prev_bus, g_prev_abrt;

void put_str(const char* s) { (void)!write(2, s, strlen(s)); }
void put_hex(uintptr_t v)
{
    char b[19];
    b[0] = '0';
    b[1] = 'x';
    for (int i = 0; i < 16; i++) b[2 + i] = "0123456789abcdef"[(v >> (60 - 4 * i)) & 15];
    b[18] = 0;
    put_str(b);
}

void crash_report(int sig, siginfo_t* si, void* uc)
{
    put_str("reffine_gb300: fatal signal ");
    put_hex((uintptr_t)sig);
    put_str(" at address ");
    put_hex((uintptr_t)(si ? si->si_addr : nullptr));
    put_str(", native frames of the faulting thread:\n");
    void* fr[64];
    const int n = backtrace(fr, 64);
    for (int i = 0; i < n; i++) {
        Dl_info di;
        put_str("  #");
        put_hex((uintptr_t)i);
        put_str(" ");
        put_hex((uintptr_t)fr[i]);
        if (dladdr(fr[i], &di) && di.dli_fname) {
            put_str(" ");
            put_str(di.dli_fname);
            put_str(" +");
            put_hex((uintptr_t)fr[i] - (uintptr_t)di.dli_fbase);
            if (di.dli_sname) {
                put_str(" ");
                put_str(di.dli_sname);
            }
        }
        put_str("\n");
    }
    struct sigaction* prev = sig == SIGSEGV ? &g_prev_segv : sig == SIGBUS ? &g_prev_bus : &g_prev_abrt;
    if (prev->sa_flags & SA_SIGINFO) {
        if (prev->sa_sigaction) {
            prev->sa_sigaction(sig, si, uc);
            return;
        }
    } else if (prev->sa_handler != SIG_DFL && prev->sa_handler != SIG_IGN) {
        prev->sa_handler(sig);
        return;
    }
    signal(sig, SIG_DFL);
    raise(sig);
}

void install_crash_report()
{
    static std::once_flag once;
    std::call_once(once, [] {
        const char* v = getenv("RF_CRASH_TRACE");
        if (!v || !*v || *v == '0') return;
        void* warm[2];
        backtrace(warm, 2);  // loads the unwinder now, not inside the handler
        struct sigaction sa {};
        sa.sa_sigaction = crash_report;
        sa.sa_flags = SA_SIGINFO | SA_ONSTACK;
        sigemptyset(&sa.sa_mask);
        sigaction(SIGSEGV, &sa, &g_prev_segv);
        sigaction(SIGBUS, &sa, &g_prev_bus);
        sigaction(SIGABRT, &sa, &g_prev_abrt);
    });
}
}  // namespace

// ------------------------------------------------------------------------------------------
// context
// ------------------------------------------------------------------------------------------
extern "C" int rf_gpu_init(int device, rf_ctx** out)
{
    if (!out) return RF_ERR_INVALID;
    *out = nullptr;
    install_crash_report();
    auto ctx = std::make_unique<rf_ctx>();
    ctx->device = device;
    CUDA_TRY(nullptr, cudaSetDevice(device));
    CUDA_TRY(nullptr, cudaFree(nullptr));
    if (!drv().ok) return RF_ERR_CUDA;
    CUDA_TRY(nullptr, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    // table buffers come from the device's stream-ordered pool; keep freed memory in the pool so
    // per-run output tables do not go back to the driver
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        unsigned long long thr = ~0ULL;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    CUDA_TRY(nullptr, cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device));
    // Grace hosts: the GPU walks the host page tables, so copies from pageable memory run at
    // link speed without a pinned bounce buffer
    cudaDeviceGetAttribute(&ctx->pageable_direct, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device);
    // filtered join indexes kept between runs: 2 GiB in all unless RF_IXF_CACHE_MB says otherwise
    // (0 rebuilds every run)
    {
        const char* mb = getenv("RF_IXF_CACHE_MB");
        ctx->ixf_budget = (size_t)(mb ? atoll(mb) : 2048) << 20;
    }
    CUDA_TRY(nullptr, cudaMalloc((void**)&ctx->dev_err, sizeof(int)));
    CUDA_TRY(nullptr, cudaMemset(ctx->dev_err, 0, sizeof(int)));
    // rf_plan_run_noalloc's fixed array: with lazy module loading the array's device memory is
    // set up when its module first loads, so the address is looked up here (loading the module
    // while the caller may still allocate), never inside a run that promises no allocation
    {
        void* scratch = nullptr;
        size_t scratch_bytes = 0;
        int e = rf_k_noalloc_scratch(device, &scratch, &scratch_bytes);
        if (e) {
            cudaFree(ctx->dev_err);
            cudaStreamDestroy(ctx->stream);
            return RF_ERR_CUDA;
        }
    }
    *out = ctx.release();
    return RF_OK;
}

extern "C" int rf_gpu_shutdown(rf_ctx* ctx)
{
    if (!ctx) return RF_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    ctx->modules.clear();
    cudaFree(ctx->dev_err);
    if (ctx->stage) cudaFreeHost(ctx->stage);
    for (auto& e : ctx->pipe_ev) cudaEventDestroy(e);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    for (auto& e : ctx->stage_ev)
        if (e) cudaEventDestroy(e);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return RF_OK;
}

extern "C" const char* rf_last_error(rf_ctx* ctx)
{
    // a copy per calling thread: the server's threads may fail while a client reads the message
    static thread_local std::string msg;
    if (!ctx) return "no context";
    std::lock_guard<std::mutex> g(ctx->err_mu);
    msg = ctx->err;
    return msg.c_str();
}

extern "C" int rf_ctx_stream(rf_ctx* ctx, void** stream)
{
    if (!ctx || !stream) return RF_ERR_INVALID;
    *stream = ctx->stream;
    return RF_OK;
}

namespace rfrt {
int check_device_error(rf_ctx* ctx)
{
    int e = 0;
    CUDA_TRY(ctx, cudaMemcpy(&e, ctx->dev_err, sizeof(int), cudaMemcpyDeviceToHost));
    return device_error(ctx, e);
}

int device_error(rf_ctx* ctx, int e)
{
    if (e) {
        cudaMemset(ctx->dev_err, 0, sizeof(int));
        const char* what = e == RF_DEVERR_PROBE ? "hash probe exhausted the table"
                           : e == RF_DEVERR_WAIT ? "bounded wait ran out"
                           : e == RF_DEVERR_RANGE ? "loop lower bound not found in the iterator column (Locate returned -1)"
                           : e == RF_DEVERR_OVERFLOW ? "output capacity exceeded"
                                                     : "unknown device error";
        return fail(ctx, RF_ERR_DEVICE, "device error %d: %s", e, what);
    }
    return RF_OK;
}
}  // namespace rfrt
using rfrt::check_device_error;

extern "C" int rf_ctx_sync(rf_ctx* ctx)
{
    if (!ctx) return RF_ERR_INVALID;
    cudaSetDevice(ctx->device);
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return check_device_error(ctx);
}

extern "C" int rf_ctx_launch_count(rf_ctx* ctx, int64_t* count)
{
    if (!ctx || !count) return RF_ERR_INVALID;
    *count = ctx->launches.load();
    return RF_OK;
}

extern "C" int rf_host_alloc(rf_ctx* ctx, size_t bytes, void** ptr)
{
    if (!ctx || !ptr) return RF_ERR_INVALID;
    cudaSetDevice(ctx->device);
    if (cudaHostAlloc(ptr, bytes ? bytes : 1, cudaHostAllocDefault) != cudaSuccess)
        return fail(ctx, RF_ERR_OOM, "cudaHostAlloc(%zu) failed", bytes);
    return RF_OK;
}

extern "C" int rf_host_free(rf_ctx* ctx, void* ptr)
{
    if (!ctx) return RF_ERR_INVALID;
    if (ptr) cudaFreeHost(ptr);
    return RF_OK;
}

// ------------------------------------------------------------------------------------------
// tables
// ------------------------------------------------------------------------------------------
namespace {

// copies `bytes` from host `src` into the allocation (*buf, *cap), growing it if needed;
// *active is set to the copy, or NULL when there is nothing to copy
int copy_in(rf_ctx* ctx, void** active, void** buf, size_t* cap, const void* src, size_t bytes, cudaStream_t s,
            std::vector<HostCopy>* defer, int width = 0)
{
    *active = nullptr;
    if (!src || bytes == 0) return RF_OK;
    if (!*buf || *cap < bytes) {
        if (*buf) cudaFreeAsync(*buf, s);
        *buf = nullptr;
        *cap = 0;
        // 16 bytes of slack: vector loads may touch the tail of the last element's 16-byte line
        if (pool_alloc(buf, bytes + 16, s) != cudaSuccess)
            return fail(ctx, RF_ERR_OOM, "device allocation of %zu bytes failed", bytes);
        *cap = bytes;
    }
    if (defer)
        defer->push_back({*buf, src, bytes, width});
    else
        CUDA_TRY(ctx, cudaMemcpyAsync(*buf, src, bytes, cudaMemcpyHostToDevice, s));
    *active = *buf;
    return RF_OK;
}

// Pinned staging ring: two halves of kStageSlots slots of kStageChunk bytes (128 MiB in all),
// allocated on first use and kept by the context.
constexpr size_t kStageChunk = size_t(4) << 20;
constexpr size_t kStageSlots = 16;

}  // namespace

namespace rfrt {

int staged_h2d(rf_ctx* ctx, const std::vector<HostCopy>& copies,
               const std::function<bool(void*, const void*, size_t)>& fill, cudaStream_t s)
{
    struct Piece {
        void* dst;
        const void* src;
        size_t n;
    };
    std::vector<Piece> pieces;
    for (const HostCopy& c : copies)
        for (size_t o = 0; o < c.bytes; o += kStageChunk)
            pieces.push_back({(char*)c.dst + o, (const char*)c.src + o, std::min(kStageChunk, c.bytes - o)});
    if (pieces.empty()) return RF_OK;
    std::lock_guard<std::mutex> g(ctx->stage_mu);
    if (!ctx->stage) {
        CUDA_TRY(ctx, cudaHostAlloc((void**)&ctx->stage, 2 * kStageSlots * kStageChunk, cudaHostAllocDefault));
        for (auto& e : ctx->stage_ev) CUDA_TRY(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    // fillers: every thread takes slots of the current round until none is left
    const size_t hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t nthreads = std::min({hw, size_t(16), pieces.size()});
    std::mutex m;
    std::condition_variable cv_work, cv_done;
    size_t gen = 0, lo = 0, hi = 0, pending = 0;
    unsigned char* base = nullptr;
    bool stop = false;
    std::atomic<size_t> next{0};
    std::atomic<bool> bad{false};
    auto run_round = [&](size_t l, size_t h, unsigned char* b) {
        for (size_t i; (i = l + next.fetch_add(1)) < h;)
            if (!fill(b + (i - l) * kStageChunk, pieces[i].src, pieces[i].n)) bad = true;
    };
    std::vector<std::thread> pool;
    for (size_t k = 0; nthreads > 1 && k < nthreads; k++)
        pool.emplace_back([&] {
            size_t seen = 0;
            for (;;) {
                size_t l, h;
                unsigned char* b;
                {
                    std::unique_lock<std::mutex> lk(m);
                    cv_work.wait(lk, [&] { return stop || gen != seen; });
                    if (stop) return;
                    seen = gen;
                    l = lo, h = hi, b = base;
                }
                run_round(l, h, b);
                std::lock_guard<std::mutex> lk(m);
                if (--pending == 0) cv_done.notify_one();
            }
        });
    int rc = RF_OK;
    bool used[2] = {false, false};
    const size_t rounds = (pieces.size() + kStageSlots - 1) / kStageSlots;
    for (size_t r = 0; r < rounds && rc == RF_OK; r++) {
        const int half = (int)(r & 1);
        unsigned char* b = ctx->stage + half * kStageSlots * kStageChunk;
        // the half is free once the copies out of it two rounds ago have landed
        if (used[half] && cudaEventSynchronize(ctx->stage_ev[half]) != cudaSuccess) {
            rc = fail(ctx, RF_ERR_CUDA, "staged copy: %s", cudaGetErrorString(cudaGetLastError()));
            break;
        }
        const size_t l = r * kStageSlots, h = std::min(pieces.size(), l + kStageSlots);
        next = 0;
        if (pool.empty()) {
            run_round(l, h, b);
        } else {
            {
                std::lock_guard<std::mutex> lk(m);
                lo = l, hi = h, base = b, pending = pool.size();
                gen++;
            }
            cv_work.notify_all();
            std::unique_lock<std::mutex> lk(m);
            cv_done.wait(lk, [&] { return pending == 0; });
        }
        if (bad) {
            rc = fail(ctx, RF_ERR_INVALID, "staged copy: reading the source failed");
            break;
        }
        for (size_t i = l; i < h && rc == RF_OK; i++) {
            cudaError_t e = cudaMemcpyAsync(pieces[i].dst, b + (i - l) * kStageChunk, pieces[i].n, cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) rc = fail(ctx, RF_ERR_CUDA, "staged copy: %s", cudaGetErrorString(e));
        }
        if (cudaEventRecord(ctx->stage_ev[half], s) != cudaSuccess && rc == RF_OK)
            rc = fail(ctx, RF_ERR_CUDA, "staged copy: event record failed");
        used[half] = true;
    }
    {
        std::lock_guard<std::mutex> lk(m);
        stop = true;
    }
    cv_work.notify_all();
    for (auto& t : pool) t.join();
    // the ring is free for the next caller only when every copy out of it has landed
    for (int half = 0; half < 2; half++)
        if (used[half] && cudaEventSynchronize(ctx->stage_ev[half]) != cudaSuccess && rc == RF_OK)
            rc = fail(ctx, RF_ERR_CUDA, "staged copy: %s", cudaGetErrorString(cudaGetLastError()));
    return rc;
}

}  // namespace rfrt

namespace {

// table buffers are pool allocations ordered on the context's stream
void free_table_mem(rf_table* t)
{
    cudaStream_t s = t->ctx ? t->ctx->stream : nullptr;
    for (auto& c : t->cols) {
        if (c.data_buf) cudaFreeAsync(c.data_buf, s);
        if (c.valid_buf) cudaFreeAsync(c.valid_buf, s);
        if (c.re_buf) cudaFreeAsync(c.re_buf, s);
        c.data_buf = c.valid_buf = c.re_buf = nullptr;
    }
    if (t->ix_slots) cudaFreeAsync(t->ix_slots, s);
    if (t->ix_special) cudaFreeAsync(t->ix_special, s);
    t->ix_slots = nullptr;
    t->ix_special = nullptr;
}

}  // namespace

namespace rfrt {

int upload(rf_ctx* ctx, const ArrowSchema* schema, const ArrowArray* array, int64_t dim, const int32_t* sel, int32_t nsel,
           void* stream, rf_table** out, rf_table* reuse, std::vector<HostCopy>* defer)
{
    if (!ctx || !schema || !array || !out) return fail(ctx, RF_ERR_INVALID, "null argument");
    *out = nullptr;
    cudaSetDevice(ctx->device);
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    if (!schema->format || std::string(schema->format) != "+s")
        return fail(ctx, RF_ERR_INVALID, "table schema must be a struct (+s), got %s", schema->format ? schema->format : "null");
    if (schema->n_children != array->n_children) return fail(ctx, RF_ERR_INVALID, "schema/array child count mismatch");
    if (array->offset != 0) return fail(ctx, RF_ERR_UNSUPPORTED, "arrays with an offset are not supported");
    long long n = schema->n_children;
    if (n > RF_MAX_COLS) return fail(ctx, RF_ERR_UNSUPPORTED, "table has %lld columns (max %d)", n, RF_MAX_COLS);
    std::unique_ptr<rf_table> owned;
    rf_table* t = reuse;
    if (t && (long long)t->cols.size() != n) {
        free_table_mem(t);
        t->cols.clear();
    }
    if (!t) {
        owned = std::make_unique<rf_table>();
        t = owned.get();
    }
    t->ctx = ctx;
    t->gen = next_table_gen();  // new contents: caches keyed on the table start over
    t->dim = dim;
    t->name = schema->name ? schema->name : "";
    t->has_index = false;
    t->null_count = 0;
    t->ndv.assign(n, -1);
    t->hot_ready = false;
    t->hot.clear();
    t->cols.resize(n);
    t->present.assign(n, 0);
    std::vector<char> want(n, sel ? 0 : 1);
    for (int i = 0; sel && i < nsel; i++)
        if (sel[i] >= 0 && sel[i] < n) want[sel[i]] = 1;
    for (long long c = 0; c < n; c++) {
        const ArrowSchema* cs = schema->children[c];
        const ArrowArray* ca = array->children[c];
        DevCol& dc = t->cols[c];
        dc.name = cs->name ? cs->name : "";
        if (ca->offset != 0) return fail(ctx, RF_ERR_UNSUPPORTED, "column %lld has an offset", c);
        std::string fmt = cs->format ? cs->format : "";
        if (fmt == "+r") {
            if (cs->n_children != 2 || ca->n_children != 2)
                return fail(ctx, RF_ERR_INVALID, "run-end column %lld needs 2 children", c);
            const ArrowArray* re = ca->children[0];
            const ArrowArray* va = ca->children[1];
            if (std::string(cs->children[0]->format) != "i")
                return fail(ctx, RF_ERR_UNSUPPORTED, "run ends must be int32 (column %lld)", c);
            if (!parse_format(cs->children[1]->format, dc.type))
                return fail(ctx, RF_ERR_UNSUPPORTED, "column %lld: format %s", c, cs->children[1]->format);
            dc.runend = true;
            dc.nvals = va->length;
            dc.logical = ca->length;
            if (re->length != va->length) return fail(ctx, RF_ERR_INVALID, "run ends and values differ in length");
            dc.data = nullptr;
            dc.valid = nullptr;
            dc.run_ends = nullptr;
            if (want[c]) {
                int rc;
                if ((rc = copy_in(ctx, (void**)&dc.run_ends, &dc.re_buf, &dc.re_cap, re->buffers[1], re->length * 4, s, defer)))
                    return rc;
                if ((rc = copy_in(ctx, &dc.data, &dc.data_buf, &dc.data_cap, va->buffers[1], va->length * dc.type.size(), s, defer)))
                    return rc;
                if (va->n_buffers > 0 && va->buffers[0] && va->null_count != 0)
                    if ((rc = copy_in(ctx, (void**)&dc.valid, &dc.valid_buf, &dc.valid_cap, va->buffers[0],
                                      ((va->length + 15) / 16) * 2, s, defer)))
                        return rc;
            }
        } else {
            if (!parse_format(cs->format, dc.type)) return fail(ctx, RF_ERR_UNSUPPORTED, "column %lld: format %s", c, cs->format);
            dc.runend = false;
            dc.nvals = ca->length;
            dc.logical = ca->length;
            dc.data = nullptr;
            dc.valid = nullptr;
            dc.run_ends = nullptr;
            if (want[c]) {
                int rc;
                if (ca->n_buffers < 2) return fail(ctx, RF_ERR_INVALID, "column %lld has no value buffer", c);
                if ((rc = copy_in(ctx, &dc.data, &dc.data_buf, &dc.data_cap, ca->buffers[1], ca->length * dc.type.size(), s, defer,
                                  (int)dc.type.size())))
                    return rc;
                if (ca->buffers[0] && ca->null_count != 0)
                    if ((rc = copy_in(ctx, (void**)&dc.valid, &dc.valid_buf, &dc.valid_cap, ca->buffers[0],
                                      ((ca->length + 15) / 16) * 2, s, defer, -1)))
                        return rc;
            }
        }
        t->present[c] = want[c];
    }
    if (owned) owned.release();
    *out = t;
    return RF_OK;
}

int build_index(rf_table* t, cudaStream_t s)
{
    rf_ctx* ctx = t->ctx;
    t->gen = next_table_gen();
    if (t->cols.empty()) return fail(ctx, RF_ERR_INVALID, "empty table");
    DevCol& c0 = t->cols[0];
    if (c0.type.btype != reffine::INT64)
        return fail(ctx, RF_ERR_UNSUPPORTED, "Data type not supported for indexing: %s", c0.type.str().c_str());
    if (!t->present[0]) return fail(ctx, RF_ERR_INVALID, "column 0 not on the device");
    unsigned long long cap = (unsigned long long)(2 * c0.nvals);  // load factor 0.5
    if (cap < 2) cap = 2;
    if (t->ix_slots) cudaFreeAsync(t->ix_slots, s);
    if (t->ix_special) cudaFreeAsync(t->ix_special, s);
    t->ix_slots = nullptr;
    t->ix_special = nullptr;
    if (pool_alloc((void**)&t->ix_slots, cap * 16, s) != cudaSuccess) return fail(ctx, RF_ERR_OOM, "index allocation failed");
    // [empty-key row, 8 B][repeated-key flag, 4 B]
    if (pool_alloc((void**)&t->ix_special, 16, s) != cudaSuccess) return fail(ctx, RF_ERR_OOM, "index allocation failed");
    t->ix_cap = cap;
    t->ix_unique = -1;
    int e = rf_k_index_build(c0.data, c0.valid, c0.nvals, t->ix_slots, cap, t->ix_special, ctx->dev_err,
                             (int*)(t->ix_special + 1), s);
    if (e) return fail(ctx, RF_ERR_CUDA, "index build launch failed: %s", cudaGetErrorString((cudaError_t)e));
    ctx->launches += c0.nvals > 0 ? 2 : 1;
    t->has_index = true;
    return RF_OK;
}

}  // namespace rfrt

extern "C" int rf_table_upload(rf_ctx* ctx, const ArrowSchema* schema, const ArrowArray* array, int64_t dim,
                               void* stream, rf_table** out)
{
    return upload(ctx, schema, array, dim, nullptr, 0, stream, out, nullptr);
}

extern "C" int rf_table_upload_cols(rf_ctx* ctx, const ArrowSchema* schema, const ArrowArray* array, int64_t dim,
                                    const int32_t* cols, int32_t n_cols, void* stream, rf_table** out)
{
    return upload(ctx, schema, array, dim, cols, n_cols, stream, out, nullptr);
}

extern "C" int rf_table_free(rf_table* t)
{
    if (!t) return RF_OK;
    cudaSetDevice(t->ctx->device);
    free_table_mem(t);  // stream-ordered: work already enqueued on the table still completes
    delete t;
    return RF_OK;
}

extern "C" int rf_table_build_index(rf_table* t, void* stream)
{
    if (!t) return RF_ERR_INVALID;
    cudaSetDevice(t->ctx->device);
    return build_index(t, stream ? (cudaStream_t)stream : t->ctx->stream);
}

extern "C" int rf_table_num_rows(rf_table* t, int64_t* rows)
{
    if (!t || !rows) return RF_ERR_INVALID;
    *rows = t->cols.empty() ? 0 : t->cols[0].logical;
    return RF_OK;
}

extern "C" int rf_table_num_cols(rf_table* t, int32_t* cols)
{
    if (!t || !cols) return RF_ERR_INVALID;
    *cols = (int32_t)t->cols.size();
    return RF_OK;
}

extern "C" int rf_table_null_count(rf_table* t, int64_t* nulls)
{
    if (!t || !nulls) return RF_ERR_INVALID;
    *nulls = t->null_count;
    return RF_OK;
}

extern "C" int rf_table_describe(rf_table* t, char* buf, size_t len, size_t* needed)
{
    if (!t) return RF_ERR_INVALID;
    std::string text;
    for (const DevCol& c : t->cols)
        text += c.name + "\t" + format_of(c.type) + "\t" + (c.runend ? "runend" : "flat") + "\n";
    if (needed) *needed = text.size() + 1;
    if (buf && len) {
        const size_t n = std::min(len - 1, text.size());
        std::memcpy(buf, text.data(), n);
        buf[n] = 0;
    }
    return RF_OK;
}

extern "C" int rf_table_column(rf_table* t, int32_t col, int32_t part, void** dev_ptr, int64_t* count)
{
    if (!t || !dev_ptr || col < 0 || col >= (int32_t)t->cols.size()) return RF_ERR_INVALID;
    auto& c = t->cols[col];
    if (part == 0) {
        *dev_ptr = c.data;
        if (count) *count = c.nvals;
    } else if (part == 1) {
        *dev_ptr = c.valid;
        if (count) *count = c.valid ? (c.nvals + 15) / 16 * 2 : 0;
    } else if (part == 2) {
        *dev_ptr = c.run_ends;
        if (count) *count = c.runend ? c.nvals : 0;
    } else {
        return RF_ERR_INVALID;
    }
    return RF_OK;
}

// ---- export: device table -> host Arrow C data (owned; released through callbacks) --------
namespace {

struct ExportSchemaPriv {
    std::string format, name;
    std::vector<ArrowSchema*> children;
    std::vector<ArrowSchema> child_store;
};
struct ExportArrayPriv {
    std::vector<void*> bufs;       // malloc'ed
    std::vector<const void*> buf_ptrs;
    std::vector<ArrowArray*> children;
    std::vector<ArrowArray> child_store;
};

void release_schema(ArrowSchema* s)
{
    if (!s || !s->release) return;
    auto* p = (ExportSchemaPriv*)s->private_data;
    if (p) {
        for (auto& c : p->child_store)
            if (c.release) c.release(&c);
        delete p;
    }
    s->release = nullptr;
}

void release_array(ArrowArray* a)
{
    if (!a || !a->release) return;
    auto* p = (ExportArrayPriv*)a->private_data;
    if (p) {
        for (auto& c : p->child_store)
            if (c.release) c.release(&c);
        for (void* b : p->bufs) free(b);
        delete p;
    }
    a->release = nullptr;
}

void init_schema(ArrowSchema* s, const std::string& fmt, const std::string& name, size_t nchildren)
{
    auto* p = new ExportSchemaPriv();
    p->format = fmt;
    p->name = name;
    p->child_store.resize(nchildren);
    p->children.resize(nchildren);
    for (size_t i = 0; i < nchildren; i++) p->children[i] = &p->child_store[i];
    memset(s, 0, sizeof(*s));
    s->format = p->format.c_str();
    s->name = p->name.c_str();
    s->flags = ARROW_FLAG_NULLABLE;
    s->n_children = (int64_t)nchildren;
    s->children = nchildren ? p->children.data() : nullptr;
    s->release = release_schema;
    s->private_data = p;
}

ExportArrayPriv* init_array(ArrowArray* a, long long length, long long nulls, size_t nbuffers, size_t nchildren)
{
    auto* p = new ExportArrayPriv();
    p->buf_ptrs.assign(nbuffers, nullptr);
    p->child_store.resize(nchildren);
    p->children.resize(nchildren);
    for (size_t i = 0; i < nchildren; i++) p->children[i] = &p->child_store[i];
    memset(a, 0, sizeof(*a));
    a->length = length;
    a->null_count = nulls;
    a->n_buffers = (int64_t)nbuffers;
    a->n_children = (int64_t)nchildren;
    a->buffers = nbuffers ? p->buf_ptrs.data() : nullptr;
    a->children = nchildren ? p->children.data() : nullptr;
    a->release = release_array;
    a->private_data = p;
    return p;
}

// Touches one byte of every page of [h, h + bytes) on up to 16 host threads.  A fresh host
// buffer is mapped page by page on first touch; a device-to-host copy into it then spends most
// of its time in page faults taken one at a time (116 MB on the GB300 machine: 5.5 ms copied fresh,
// 1.5 ms touched on 16 threads + 0.8 ms copied).
void touch_pages(void* h, size_t bytes)
{
    static const size_t page = (size_t)std::max(4096L, sysconf(_SC_PAGESIZE));
    const size_t npages = (bytes + page - 1) / page;
    const int nt = (int)std::min<size_t>({16, std::max(1u, std::thread::hardware_concurrency()), npages / 256 + 1});
    auto part = [&](int k) {
        for (size_t i = npages * k / nt; i < npages * (k + 1) / nt; i++) ((volatile char*)h)[i * page] = 0;
    };
    std::vector<std::thread> th;
    for (int k = 1; k < nt; k++) th.emplace_back(part, k);
    part(0);
    for (auto& x : th) x.join();
}

// one column buffer of an export: host memory of `bytes`, pages touched now, filled by the copy
// enqueued on the context's stream (the caller synchronises once after all copies)
int fetch(rf_ctx* ctx, ExportArrayPriv* p, int slot, const void* dsrc, size_t bytes)
{
    if (!dsrc || bytes == 0) return RF_OK;
    void* h = malloc(bytes);
    if (!h) return fail(ctx, RF_ERR_OOM, "host allocation failed");
    p->bufs.push_back(h);
    if (bytes >= ((size_t)1 << 22)) touch_pages(h, bytes);
    CUDA_TRY(ctx, cudaMemcpyAsync(h, dsrc, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    p->buf_ptrs[slot] = h;
    return RF_OK;
}

}  // namespace

extern "C" int rf_table_export(rf_table* t, ArrowSchema* so, ArrowArray* ao)
{
    if (!t || !so || !ao) return RF_ERR_INVALID;
    rf_ctx* ctx = t->ctx;
    cudaSetDevice(ctx->device);
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    size_t n = t->cols.size();
    long long rows = n ? t->cols[0].logical : 0;
    init_schema(so, "+s", t->name, n);
    auto* ap = init_array(ao, rows, 0, 1, n);
    for (size_t c = 0; c < n; c++) {
        auto& dc = t->cols[c];
        auto* sp = (ExportSchemaPriv*)so->private_data;
        ArrowSchema* cs = sp->children[c];
        ArrowArray* ca = ap->children[c];
        long long nulls = dc.valid ? t->null_count : 0;
        if (dc.runend) {
            init_schema(cs, "+r", dc.name, 2);
            auto* csp = (ExportSchemaPriv*)cs->private_data;
            init_schema(csp->children[0], "i", "run_ends", 0);
            init_schema(csp->children[1], format_of(dc.type), "values", 0);
            auto* cap = init_array(ca, dc.logical, 0, 0, 2);
            auto* rp = init_array(cap->children[0], dc.nvals, 0, 2, 0);
            auto* vp = init_array(cap->children[1], dc.nvals, nulls, 2, 0);
            int rc;
            if ((rc = fetch(ctx, rp, 1, dc.run_ends, dc.nvals * 4))) return rc;
            if ((rc = fetch(ctx, vp, 1, dc.data, dc.nvals * dc.type.size()))) return rc;
            if ((rc = fetch(ctx, vp, 0, dc.valid, (dc.nvals + 15) / 16 * 2))) return rc;
        } else {
            init_schema(cs, format_of(dc.type), dc.name, 0);
            auto* cp = init_array(ca, dc.nvals, nulls, 2, 0);
            int rc;
            if ((rc = fetch(ctx, cp, 1, dc.data, dc.nvals * dc.type.size()))) return rc;
            if ((rc = fetch(ctx, cp, 0, dc.valid, (dc.nvals + 15) / 16 * 2))) return rc;
        }
    }
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return RF_OK;
}

// ------------------------------------------------------------------------------------------
// plans
// ------------------------------------------------------------------------------------------
// Waves of resident blocks a reduce's work units fill.  More units balance uneven rows (the
// join's probe: 2.0 -> 1.6 ms at 200M rows with 8 waves) and let a row-chunked run launch a full
// wave per chunk; but every unit folds its block's slots into a partial and the last unit folds
// all partials, FP64 adds on GB300's narrow FP64 pipe: with 6 x 6 slots (the 60M-row group-by)
// 8 waves cost 1.27 -> 1.47 ms.  So plans with many slots keep one wave.
static int unit_waves(const rfg::Plan& pl)
{
    if (pl.kind == rfg::PlanKind::SCAN_REDUCE) return kUnitWaves;
    if (pl.kind == rfg::PlanKind::GROUP_REDUCE) return pl.groups * pl.aggs <= 16 ? kUnitWaves : 1;
    return 1;
}

namespace {
// The plan of `fn` at block size `threads`: lowered, its kernels compiled and loaded, its work
// units sized and its device buffers allocated (rf_plan_compile, and the autotuner's variants).
int build_plan(rf_ctx* ctx, const std::shared_ptr<reffine::Func>& fn, bool vectorize, int threads,
               std::unique_ptr<rf_plan>& p)
{
    p = std::make_unique<rf_plan>();
    p->ctx = ctx;
    try {
        p->plan = rfg::lower(fn, vectorize, threads);
    } catch (const rfg::LowerError& e) {
        return fail(ctx, e.unsupported ? RF_ERR_UNSUPPORTED : RF_ERR_INVALID, "%s", e.what());
    } catch (const std::exception& e) {
        return fail(ctx, RF_ERR_INVALID, "%s", e.what());
    }
    int rc = jit_compile(ctx, p->plan.key, p->plan.source, p->mod, nullptr);
    if (rc) return rc;
    for (auto& k : p->plan.kernels) {
        CUfunction f = nullptr;
        if (k.name.empty()) {  // a step run by the library's own kernels (kernels.cu)
            p->fns.push_back(nullptr);
            continue;
        }
        if ((rc = get_function(ctx, *p->mod, k.name, f))) return rc;
        if (k.smem > 0) {  // the default cap is 48 KiB minus the kernel's static shared memory
            CUresult cr = drv().FuncSetAttribute(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)k.smem);
            if (cr != CUDA_SUCCESS) return cu_fail(ctx, cr, "cuFuncSetAttribute");
        }
        p->fns.push_back(f);
    }
    // work units of the main kernel: enough resident blocks to fill the GPU once
    int per_sm = 1;
    for (size_t i = 0; i < p->plan.kernels.size(); i++) {
        if (p->plan.kernels[i].role != rfg::KernelSpec::MAIN) continue;
        CUresult cr = drv().OccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, p->fns[i], p->plan.kernels[i].threads,
                                                                      p->plan.kernels[i].smem);
        if (cr != CUDA_SUCCESS) return cu_fail(ctx, cr, "occupancy query");
        if (per_sm < 1) {
            int regs = -1, ssm = -1, maxt = -1, maxdyn = -1;
            drv().FuncGetAttribute(&regs, CU_FUNC_ATTRIBUTE_NUM_REGS, p->fns[i]);
            drv().FuncGetAttribute(&ssm, CU_FUNC_ATTRIBUTE_SHARED_SIZE_BYTES, p->fns[i]);
            drv().FuncGetAttribute(&maxt, CU_FUNC_ATTRIBUTE_MAX_THREADS_PER_BLOCK, p->fns[i]);
            drv().FuncGetAttribute(&maxdyn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, p->fns[i]);
            return fail(ctx, RF_ERR_JIT,
                        "kernel %s cannot be resident: %d threads, %zu B dynamic shared memory (allowed %d), %d B "
                        "static, %d registers, at most %d threads",
                        p->plan.kernels[i].name.c_str(), p->plan.kernels[i].threads, p->plan.kernels[i].smem, maxdyn,
                        ssm, regs, maxt);
        }
    }
    p->max_units = ctx->sm_count * per_sm;
    p->reduce_units = p->max_units * unit_waves(p->plan);
    if ((p->plan.kind == rfg::PlanKind::SCAN_REDUCE || p->plan.kind == rfg::PlanKind::GROUP_REDUCE) &&
        !p->plan.device_range) {
        const auto& mk = p->plan.kernels.back();
        CUfunction bf;
        if ((rc = get_function(ctx, *p->mod, "rf_batch", bf))) return rc;
        if (mk.smem > 0) {
            CUresult cr = drv().FuncSetAttribute(bf, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)mk.smem);
            if (cr != CUDA_SUCCESS) return cu_fail(ctx, cr, "cuFuncSetAttribute");
        }
        int bps = 1;
        CUresult cr = drv().OccupancyMaxActiveBlocksPerMultiprocessor(&bps, bf, mk.threads, mk.smem);
        if (cr != CUDA_SUCCESS) return cu_fail(ctx, cr, "occupancy query");
        p->batch_fn = bf;
        p->batch_grid = ctx->sm_count * std::max(1, bps);
        p->batch_smem = mk.smem;
        p->batch_threads = mk.threads;
    }
    // the plan's own device buffers, carved from one allocation of the context's stream-ordered
    // pool (compiling many plans costs no device-wide synchronisation):
    //   [partials of the units][completion counter 64 B][loop range 64 B][value result]
    //   [table outputs: column pointer array][results 64 B]
    p->partials_bytes = (size_t)p->reduce_units * (p->plan.acc_bytes ? p->plan.acc_bytes : 8);
    const size_t osz = p->plan.out_size ? p->plan.out_size : 8;
    auto al = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t o_counter = al(p->partials_bytes), o_range = o_counter + 256, o_out = o_range + 256;
    const size_t o_ptrs = o_out + al(osz), o_res = o_ptrs + al(sizeof(void*) * 2 * RF_MAX_COLS);
    const size_t total = p->plan.out_is_table ? o_res + 256 : o_ptrs;
    unsigned char* base = nullptr;
    CUDA_TRY(ctx, pool_alloc((void**)&base, total, ctx->stream));
    p->buf = base;
    p->partials = base;
    p->counter = (unsigned*)(base + o_counter);
    p->range = (long long*)(base + o_range);
    p->dout = base + o_out;
    if (p->plan.out_is_table) {
        p->d_ptrs = (void**)(base + o_ptrs);
        p->d_res = (long long*)(base + o_res);
    }
    CUDA_TRY(ctx, cudaMemsetAsync(p->counter, 0, 64, ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));  // ready for use on any stream
    return RF_OK;
}
}  // namespace

extern "C" int rf_plan_compile(rf_ctx* ctx, const char* text, int vectorize, rf_plan** out)
{
    if (!ctx || !text || !out) return fail(ctx, RF_ERR_INVALID, "null argument");
    *out = nullptr;
    cudaSetDevice(ctx->device);
    std::shared_ptr<reffine::Func> fn;
    std::string shape;
    try {
        fn = reffine::parse_text(text);
        shape = rfg::lower(fn, vectorize != 0).key;  // the query shape at the default block size
    } catch (const rfg::LowerError& e) {
        return fail(ctx, e.unsupported ? RF_ERR_UNSUPPORTED : RF_ERR_INVALID, "%s", e.what());
    } catch (const std::exception& e) {
        return fail(ctx, RF_ERR_INVALID, "%s", e.what());
    }
    // a block size the autotuner chose for this shape (kept as bucket -1 of the shape's entry)
    int threads = 256;
    {
        std::lock_guard<std::mutex> g(ctx->tune_mu);
        auto it = ctx->tune.find(shape);
        if (it != ctx->tune.end()) {
            auto jt = it->second.find(-1);
            if (jt != it->second.end()) threads = (int)jt->second;
        }
    }
    std::unique_ptr<rf_plan> p;
    int rc = build_plan(ctx, fn, vectorize != 0, threads, p);
    if (rc) return rc;
    p->text = text;
    p->shape = shape;
    *out = p.release();
    return RF_OK;
}

extern "C" int rf_plan_check(const char* text, int vectorize, char* buf, size_t buf_len)
{
    auto put = [&](const std::string& m) {
        if (buf && buf_len) {
            size_t n = std::min(buf_len - 1, m.size());
            memcpy(buf, m.data(), n);
            buf[n] = 0;
        }
    };
    if (!text) return RF_ERR_INVALID;
    rfg::Plan plan;
    try {
        plan = rfg::lower(reffine::parse_text(text), vectorize != 0);
    } catch (const rfg::LowerError& e) {
        put(e.what());
        return e.unsupported ? RF_ERR_UNSUPPORTED : RF_ERR_INVALID;
    } catch (const std::exception& e) {
        put(e.what());
        return RF_ERR_INVALID;
    }
    std::string cubin, log;
    if (!nvrtc_compile(plan.source, cubin, log)) {
        put(log);
        return RF_ERR_JIT;
    }
    put(plan.source);
    return RF_OK;
}

namespace rfrt {
void release_filtered_index(rf_plan* p, cudaStream_t s);
}

extern "C" int rf_plan_free(rf_plan* p)
{
    if (!p) return RF_OK;
    cudaSetDevice(p->ctx->device);
    {
        std::lock_guard<std::mutex> g(p->ctx->ixf_mu);
        rfrt::release_filtered_index(p, p->ctx->stream);
        if (p->ixf_ev) cudaEventDestroy(p->ixf_ev);
    }
    cudaStreamSynchronize(p->ctx->stream);
    if (p->buf) cudaFreeAsync(p->buf, p->ctx->stream);
    cudaFree(p->d_tiles);
    cudaFree(p->hg_keys);
    cudaFree(p->hg_acc);
    cudaFree(p->seg_woff);
    cudaFree(p->seg_tmp);
    cudaFree(p->seg_part);
    cudaFree(p->hg_img);
    cudaFreeHost(p->h_res);
    for (auto* t : p->staging)
        if (t) {
            free_table_mem(t);
            delete t;
        }
    rfrt::thunk_release(p);
    delete p;
    return RF_OK;
}

extern "C" const char* rf_plan_source(rf_plan* p) { return p ? p->plan.source.c_str() : ""; }

extern "C" int rf_plan_info(rf_plan* p, rf_plan_info_t* info)
{
    if (!p || !info) return RF_ERR_INVALID;
    memset(info, 0, sizeof(*info));
    info->kind = (int)p->plan.kind;
    info->n_inputs = p->plan.n_inputs;
    info->output_is_table = p->plan.out_is_table;
    info->n_groups = p->plan.groups;
    info->output_size = (int64_t)p->plan.out_size;
    for (int i = 0; i < p->plan.n_inputs && i < 8; i++) {
        long long b = 0;
        if (p->plan.input_types[i].is_vector())
            for (int c : p->plan.cols_read[i]) b += (long long)p->plan.input_types[i].dtypes[c].size();
        info->bytes_per_row[i] = b;
    }
    info->n_kernels = (int32_t)p->plan.kernels.size();
    info->vectorize = p->plan.vectorize;
    return RF_OK;
}

namespace rfrt {

// Tiling of a scan: the rows of one unit of work.  Scan and grouped-scan Reduce plans take the
// autotuner's choice for their shape and size bucket when there is one (rf_plan_tune); every
// path of a query (alone, batched, without allocation) asks here, so all use the same tiling and
// give the same result bits.
// A hash group-by's table: slots per 100 estimated distinct keys, the autotuner's choice for the
// plan's query shape and row-count bucket (the same tuning table as the scans' tiling), else 220
// (load 0.45, the best of 160 / 220 / 300 / 400 measured on 100M Zipf(1.1) rows).
int hg_factor_for(rf_plan* p, long long rows)
{
    if (p->hg_factor_override > 0) return p->hg_factor_override;
    int bucket = 0;
    while (bucket < 62 && (1LL << (bucket + 1)) <= rows) bucket++;
    std::lock_guard<std::mutex> g(p->ctx->tune_mu);
    auto it = p->ctx->tune.find(p->plan.key);
    if (it == p->ctx->tune.end()) return 220;
    auto jt = it->second.find(bucket);
    return jt == it->second.end() ? 220 : (int)jt->second;
}

long long tile_rows_for(rf_plan* p, long long rows)
{
    const rfg::Plan& pl = p->plan;
    if (pl.kind != rfg::PlanKind::SCAN_REDUCE && pl.kind != rfg::PlanKind::GROUP_REDUCE) return pl.tile_rows;
    if (p->tile_override > 0) return p->tile_override;
    int bucket = 0;
    while (bucket < 62 && (1LL << (bucket + 1)) <= rows) bucket++;
    std::lock_guard<std::mutex> g(p->ctx->tune_mu);
    auto it = p->ctx->tune.find(pl.key);
    if (it == p->ctx->tune.end()) return pl.tile_rows;
    auto jt = it->second.find(bucket);
    return jt == it->second.end() ? pl.tile_rows : jt->second;
}

int fill_params(rf_plan* p, const rf_arg* args, int n_args, RfParams& P, long long& lo, long long& hi,
                bool may_allocate)
{
    rf_ctx* ctx = p->ctx;
    const rfg::Plan& pl = p->plan;
    if (n_args != pl.n_inputs) return fail(ctx, RF_ERR_INVALID, "plan takes %d inputs, got %d", pl.n_inputs, n_args);
    memset(&P, 0, sizeof(P));
    for (int i = 0; i < n_args; i++) {
        const auto& ty = pl.input_types[i];
        if (ty.is_vector()) {
            if (args[i].kind != RF_ARG_TABLE || !args[i].table)
                return fail(ctx, RF_ERR_INVALID, "input %d must be a table", i);
            rf_table* t = args[i].table;
            if (t->cols.size() != ty.dtypes.size())
                return fail(ctx, RF_ERR_INVALID, "input %d: table has %zu columns, query expects %zu", i, t->cols.size(),
                            ty.dtypes.size());
            RfTab& T = P.t[pl.table_slot[i]];
            for (size_t c = 0; c < t->cols.size(); c++) {
                auto& dc = t->cols[c];
                if (dc.type.size() != ty.dtypes[c].size() || dc.type.is_float() != ty.dtypes[c].is_float())
                    return fail(ctx, RF_ERR_INVALID, "input %d column %zu: type %s, query expects %s", i, c,
                                dc.type.str().c_str(), ty.dtypes[c].str().c_str());
                if ((ty.encodings[c] == reffine::RUNEND) != dc.runend)
                    return fail(ctx, RF_ERR_INVALID, "input %d column %zu: encoding differs from the query's", i, c);
                T.col[c].data = dc.data;
                T.col[c].valid = dc.valid;
                T.col[c].run_ends = dc.run_ends;
                T.col[c].len = dc.nvals;
            }
            for (int c : pl.cols_read[i])
                if (!t->present[c]) return fail(ctx, RF_ERR_INVALID, "input %d: column %d is not on the device", i, c);
            if (pl.needs_index[i]) {
                if (!t->has_index) {
                    if (!may_allocate)
                        return fail(ctx, RF_ERR_INVALID, "input %d needs its index: call rf_table_build_index first", i);
                    int rc = build_index(t, ctx->stream);
                    if (rc) return rc;
                }
                T.ix.slots = t->ix_slots;
                T.ix.cap = t->ix_cap;
                T.ix.special = t->ix_special;
            }
            T.nrows = t->cols.empty() ? 0 : t->cols[0].logical;
        } else {
            int j = pl.scalar_slot[i];
            if (ty.is_float()) {
                double d = args[i].kind == RF_ARG_F64 ? args[i].f64 : (double)args[i].i64;
                memcpy(&P.s[j], &d, 8);
            } else {
                P.s[j] = args[i].kind == RF_ARG_F64 ? (long long)args[i].f64 : args[i].i64;
            }
        }
    }
    for (size_t k = 0; k < pl.consts.size(); k++) {
        if (pl.consts[k].is_float) P.k[k].f = pl.consts[k].f;
        else P.k[k].i = pl.consts[k].i;
    }
    bool ok = true;
    lo = eval_host(pl.row_lo, args, n_args, ok);
    hi = eval_host(pl.row_hi, args, n_args, ok);
    if (!ok) return fail(ctx, RF_ERR_INVALID, "cannot evaluate the loop bounds");
    if (pl.drive_input >= 0) {
        // never read past the driving table's columns (the reference would read out of bounds)
        rf_table* t = args[pl.drive_input].table;
        bool aligned = true;
        for (int c : pl.cols_read[pl.drive_input]) {
            if (t->cols[c].nvals < hi) hi = t->cols[c].nvals;
            aligned = aligned && ((uintptr_t)t->cols[c].data & 15) == 0;
        }
        if (lo < 0) lo = 0;
        // a scan's 4-row vector loads need every column it reads 16-byte aligned (a table loaded
        // from an IPC file may hold 8-byte aligned buffers; those take the one-row path)
        if (aligned) P.flags |= RF_FLAG_VEC4;
    }
    if (hi < lo) hi = lo;
    P.row_lo = lo;
    P.row_hi = hi;
    P.tile_rows = tile_rows_for(p, hi - lo);
    P.range = pl.device_range ? p->range : nullptr;
    P.partials = p->partials;
    P.counter = p->counter;
    P.out = p->dout;
    P.err = ctx->dev_err;
    return RF_OK;
}

bool index_role(int role)
{
    return role == rfg::KernelSpec::IXCOUNT || role == rfg::KernelSpec::IXINIT || role == rfg::KernelSpec::IXBUILD;
}

// Builds the plan's filtered index of the probed table T (its index entries whose row passes
// the pushed-down filter, see the lowering) on stream s, in memory taken from the stream-ordered
// pool for this run (*buf; the caller releases it after the probing kernel), and points `out`
// at it.  The number of entries kept is counted once per table (a synchronising read) and
// remembered; the entries come from T's rows when no key repeats, else from its index.
void release_filtered_index(rf_plan* p, cudaStream_t s);

// (the caller holds ctx->ixf_mu from here until the kernels that read the index are enqueued
// and, when the plan keeps the index, p->ixf_ev is recorded after them)
int filtered_index(rf_plan* p, rf_table* T, const RfParams& P, cudaStream_t s, RfIndex* out, void** buf)
{
    rf_ctx* ctx = p->ctx;
    const rfg::Plan& pl = p->plan;
    *buf = nullptr;
    CUfunction fc = nullptr, fi = nullptr, fb = nullptr;
    for (size_t i = 0; i < pl.kernels.size(); i++) {
        if (pl.kernels[i].role == rfg::KernelSpec::IXCOUNT) fc = p->fns[i];
        if (pl.kernels[i].role == rfg::KernelSpec::IXINIT) fi = p->fns[i];
        if (pl.kernels[i].role == rfg::KernelSpec::IXBUILD) fb = p->fns[i];
    }
    if (T->ix_unique < 0) {
        int dup = 0;
        CUDA_TRY(ctx, cudaMemcpyAsync(&dup, T->ix_special + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
        CUDA_TRY(ctx, cudaStreamSynchronize(s));
        T->ix_unique = dup ? 0 : 1;
    }
    const long long mode = T->ix_unique == 1 ? 1 : 0;
    const unsigned long long nent = mode ? (unsigned long long)T->cols[0].nvals : T->ix_cap;
    const int gfull = (int)std::min<unsigned long long>((nent + 1023) / 1024 + 1, (unsigned long long)ctx->sm_count * 8);
    int rc;
    if (p->ixf_for != T->gen) {
        unsigned long long* cnt = nullptr;
        CUDA_TRY(ctx, pool_alloc((void**)&cnt, 8, s));
        CUDA_TRY(ctx, cudaMemsetAsync(cnt, 0, 8, s));
        RfParams Q = P;
        Q.aux2 = cnt;
        Q.aux_n1 = mode;
        rc = launch(ctx, fc, gfull, 256, 0, s, &Q);
        unsigned long long n = 0;
        cudaError_t e = rc ? cudaSuccess : cudaMemcpyAsync(&n, cnt, 8, cudaMemcpyDeviceToHost, s);
        cudaFreeAsync(cnt, s);
        if (rc) return rc;
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return fail(ctx, RF_ERR_CUDA, "filtered index count: %s", cudaGetErrorString(e));
        p->ixf_count = (long long)n;
        p->ixf_for = T->gen;
    }
    // the index kept from this plan's last run on the same table (the table's generation
    // changes with every upload or index build, so a kept index is never stale)
    if (p->ixf_buf && p->ixf_buf_for == T->gen) {
        *out = p->ixf_ix;
        ctx->ixf_lru.remove(p);
        ctx->ixf_lru.push_back(p);
        return RF_OK;
    }
    unsigned long long cap = 64;
    while (cap < 2 * (unsigned long long)p->ixf_count) cap *= 2;
    if (pool_alloc(buf, cap * 16 + 256, s) != cudaSuccess) {
        *buf = nullptr;
        return fail(ctx, RF_ERR_OOM, "filtered index (%llu slots)", cap);
    }
    RfParams Q = P;
    Q.aux0 = *buf;
    Q.aux_n0 = (long long)cap;
    Q.aux1 = (unsigned char*)*buf + cap * 16;
    Q.aux_n1 = mode;
    const int gcap = (int)std::min<unsigned long long>((cap + 255) / 256, (unsigned long long)ctx->sm_count * 8);
    if ((rc = launch(ctx, fi, gcap, 256, 0, s, &Q))) return rc;
    if ((rc = launch(ctx, fb, gfull, 256, 0, s, &Q))) return rc;
    out->slots = (const long long*)*buf;
    out->cap = cap;
    out->special = (const long long*)Q.aux1;
    // keep it for the next run: the plan's previous index and, over the context's budget, the
    // indexes of the plans used longest ago are released in stream order after their last runs
    const size_t bytes = cap * 16 + 256;
    if (bytes > ctx->ixf_budget) return RF_OK;  // not kept: the caller releases it after this run
    if (!p->ixf_ev && cudaEventCreateWithFlags(&p->ixf_ev, cudaEventDisableTiming) != cudaSuccess) {
        p->ixf_ev = nullptr;
        return RF_OK;
    }
    release_filtered_index(p, s);
    while (ctx->ixf_bytes + bytes > ctx->ixf_budget && !ctx->ixf_lru.empty())
        release_filtered_index(ctx->ixf_lru.front(), s);
    p->ixf_buf = *buf;
    p->ixf_buf_bytes = bytes;
    p->ixf_buf_for = T->gen;
    p->ixf_ix = *out;
    ctx->ixf_bytes += bytes;
    ctx->ixf_lru.push_back(p);
    *buf = nullptr;
    return RF_OK;
}

// Releases the filtered index plan p keeps (caller holds ctx->ixf_mu): freed on s once p's last
// run that read it is done.
void release_filtered_index(rf_plan* p, cudaStream_t s)
{
    rf_ctx* ctx = p->ctx;
    if (!p->ixf_buf) return;
    if (p->ixf_ev) cudaStreamWaitEvent(s, p->ixf_ev, 0);
    cudaFreeAsync(p->ixf_buf, s);
    ctx->ixf_bytes -= p->ixf_buf_bytes;
    ctx->ixf_lru.remove(p);
    p->ixf_buf = nullptr;
    p->ixf_buf_bytes = 0;
    p->ixf_buf_for = 0;
}

int enqueue(rf_plan* p, const rf_arg* args, int n_args, cudaStream_t s, RfParams* Pout)
{
    rf_ctx* ctx = p->ctx;
    RfParams P;
    long long lo, hi;
    int rc = fill_params(p, args, n_args, P, lo, hi, true);
    if (rc) return rc;
    const rfg::Plan& pl = p->plan;
    long long ntiles = (hi - lo + P.tile_rows - 1) / P.tile_rows;
    int units = units_for(p, ntiles);
    P.nunits = units;
    void* ixbuf = nullptr;
    std::unique_lock<std::mutex> ixf_lock(ctx->ixf_mu, std::defer_lock);
    if (pl.ixf_input >= 0) {
        ixf_lock.lock();
        RfTab& tab = P.t[pl.table_slot[pl.ixf_input]];
        if ((rc = filtered_index(p, args[pl.ixf_input].table, P, s, &tab.ix, &ixbuf))) {
            if (ixbuf) cudaFreeAsync(ixbuf, s);
            return rc;
        }
    }
    for (size_t i = 0; i < pl.kernels.size() && !rc; i++) {
        const auto& k = pl.kernels[i];
        if (index_role(k.role)) continue;
        int grid = 1;
        switch (k.role) {
            case rfg::KernelSpec::RANGE: grid = 1; break;
            case rfg::KernelSpec::SCAN: grid = 1; break;
            case rfg::KernelSpec::STOP: grid = (int)std::min<long long>(std::max<long long>((hi - lo + 255) / 256, 1), ctx->sm_count * 8); break;
            case rfg::KernelSpec::MAIN: grid = units; break;
            default: grid = units; break;
        }
        rc = launch(ctx, p->fns[i], grid, k.threads, k.smem, s, &P);
    }
    if (ixbuf) cudaFreeAsync(ixbuf, s);  // after the kernels that read it, in stream order
    if (p->ixf_buf && ixf_lock.owns_lock()) cudaEventRecord(p->ixf_ev, s);  // the kept index's last use
    if (ixf_lock.owns_lock()) ixf_lock.unlock();
    if (rc) return rc;
    if (Pout) *Pout = P;
    return RF_OK;
}

bool streamable(rf_plan* p)
{
    const rfg::Plan& pl = p->plan;
    if (pl.out_is_table || pl.device_range || pl.drive_input < 0) return false;
    if (pl.kind != rfg::PlanKind::SCAN_REDUCE && pl.kind != rfg::PlanKind::GROUP_REDUCE) return false;
    const int d = pl.drive_input;
    if (pl.needs_index[d] || pl.random_read[d] || pl.ixf_input == d) return false;
    int mains = 0;
    for (const auto& k : pl.kernels) {
        if (index_role(k.role)) continue;
        if (k.role != rfg::KernelSpec::MAIN) return false;
        mains++;
    }
    return mains == 1;
}

int run_streamed(rf_plan* p, const rf_arg* args, int n_args, const std::vector<HostCopy>& drive, void* out)
{
    constexpr int kChunks = kUnitWaves;
    rf_ctx* ctx = p->ctx;
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    // Copies from pageable memory are not left to the copy engines alone (on this host the GPU
    // reads pageable memory through the host page tables and competes with the chunks' kernels),
    // so a driving table outside pinned memory is copied whole first: same units, same bits.
    bool pinned = !drive.empty();
    // chunks of at least one unit per SM: fewer units than that per chunk leave each chunk's
    // kernel as long as the whole run's, and its tail is not shortened
    int nchunks = 1;
    {
        RfParams P0;
        long long lo0, hi0;
        if (fill_params(p, args, n_args, P0, lo0, hi0, true) == RF_OK) {
            const int u = units_for(p, (hi0 - lo0 + P0.tile_rows - 1) / P0.tile_rows);
            nchunks = std::min(kChunks, u / std::max(1, ctx->sm_count));
        }
    }
    if (nchunks < 2) pinned = false;
    for (const HostCopy& c : drive) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, c.src) != cudaSuccess || a.type != cudaMemoryTypeHost) {
            cudaGetLastError();
            pinned = false;
            break;
        }
    }
    if (!pinned) {  // (or too few units to chunk)
        for (const HostCopy& c : drive)
            CUDA_TRY(ctx, cudaMemcpyAsync(c.dst, c.src, c.bytes, cudaMemcpyHostToDevice, s));
        return rf_plan_run(p, args, n_args, out, s);
    }
    if (!p->h_res && cudaHostAlloc((void**)&p->h_res, 16 + p->plan.out_size, cudaHostAllocDefault) != cudaSuccess)
        return fail(ctx, RF_ERR_OOM, "pinned result buffer");
    RfParams P;
    long long lo, hi;
    int rc = fill_params(p, args, n_args, P, lo, hi, true);
    if (rc) return rc;
    const rfg::Plan& pl = p->plan;
    const long long tr = P.tile_rows;
    const long long ntiles = (hi - lo + tr - 1) / tr;
    const int units = units_for(p, ntiles);
    P.nunits = units;
    size_t mi = 0;
    while (mi < pl.kernels.size() && (index_role(pl.kernels[mi].role) || pl.kernels[mi].role != rfg::KernelSpec::MAIN)) mi++;
    if (mi == pl.kernels.size()) return fail(ctx, RF_ERR_INVALID, "streamed run of a plan without a main kernel");
    std::lock_guard<std::mutex> g(ctx->pipe_mu);
    if (!ctx->copy_stream) {
        CUDA_TRY(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
        ctx->pipe_ev.assign(kChunks, nullptr);
        for (auto& e : ctx->pipe_ev) CUDA_TRY(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    cudaStream_t cs = ctx->copy_stream;
    void* ixbuf = nullptr;
    std::unique_lock<std::mutex> ixf_lock(ctx->ixf_mu, std::defer_lock);
    if (pl.ixf_input >= 0) {
        ixf_lock.lock();
        RfTab& tab = P.t[pl.table_slot[pl.ixf_input]];
        rc = filtered_index(p, args[pl.ixf_input].table, P, s, &tab.ix, &ixbuf);
    }
    // copies start after everything enqueued on the compute stream so far (the device buffers
    // of the driving table were allocated there)
    if (!rc && (cudaEventRecord(ctx->pipe_ev[0], s) != cudaSuccess || cudaStreamWaitEvent(cs, ctx->pipe_ev[0], 0) != cudaSuccess))
        rc = fail(ctx, RF_ERR_CUDA, "streamed run: ordering the copy stream");
    nchunks = std::min(nchunks, units);
    long long r0 = 0;  // rows of every driving column copied so far (the first chunk starts at row 0)
    for (int k = 0; k < nchunks && !rc; k++) {
        const int u0 = (int)((long long)units * k / nchunks), u1 = (int)((long long)units * (k + 1) / nchunks);
        const bool last = k == nchunks - 1;
        // units [u0, u1) read the rows of tiles [u0*ntiles/units, u1*ntiles/units)
        const long long r1 = lo + (long long)u1 * ntiles / units * tr;
        for (const HostCopy& c : drive) {
            size_t b0, b1;
            if (c.width == 0) {
                if (k) continue;  // not addressable by row: whole, before the first units
                b0 = 0, b1 = c.bytes;
            } else if (c.width > 0) {
                b0 = std::min(c.bytes, (size_t)r0 * (size_t)c.width);
                b1 = last ? c.bytes : std::min(c.bytes, (size_t)r1 * (size_t)c.width);
            } else {  // validity bitmap, read as 16-bit words: whole words, the boundary word twice
                b0 = std::min(c.bytes, (size_t)(r0 / 16) * 2);
                b1 = last ? c.bytes : std::min(c.bytes, (size_t)((r1 + 15) / 16) * 2);
            }
            if (b1 <= b0) continue;
            const cudaError_t e = cudaMemcpyAsync((char*)c.dst + b0, (const char*)c.src + b0, b1 - b0,
                                                  cudaMemcpyHostToDevice, cs);
            if (e != cudaSuccess) {
                rc = fail(ctx, RF_ERR_CUDA, "streamed run: copy: %s", cudaGetErrorString(e));
                break;
            }
        }
        if (rc) break;
        if (cudaEventRecord(ctx->pipe_ev[k], cs) != cudaSuccess || cudaStreamWaitEvent(s, ctx->pipe_ev[k], 0) != cudaSuccess) {
            rc = fail(ctx, RF_ERR_CUDA, "streamed run: chunk event");
            break;
        }
        RfParams Q = P;
        Q.unit0 = u0;
        rc = launch(ctx, p->fns[mi], u1 - u0, pl.kernels[mi].threads, pl.kernels[mi].smem, s, &Q);
        r0 = r1;
    }
    if (ixbuf) cudaFreeAsync(ixbuf, s);
    if (p->ixf_buf && ixf_lock.owns_lock()) cudaEventRecord(p->ixf_ev, s);  // the kept index's last use
    if (ixf_lock.owns_lock()) ixf_lock.unlock();
    if (rc) {
        // no copy may outlive the call (the caller owns the host memory), and the units that did
        // run left the merge ticket part-way
        cudaStreamSynchronize(cs);
        cudaStreamSynchronize(s);
        cudaMemsetAsync(p->counter, 0, sizeof(unsigned int), s);
        cudaStreamSynchronize(s);
        return rc;
    }
    CUDA_TRY(ctx, cudaMemcpyAsync(p->h_res, ctx->dev_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(ctx, cudaMemcpyAsync(p->h_res + 16, p->dout, pl.out_size, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(ctx, cudaStreamSynchronize(s));  // after the last chunk's event: every copy has landed too
    int e;
    memcpy(&e, p->h_res, sizeof(int));
    if ((rc = device_error(ctx, e))) return rc;
    if (out) memcpy(out, p->h_res + 16, pl.out_size);
    return RF_OK;
}

}  // namespace rfrt

namespace rfrt {
const rfg::Plan& plan_of(rf_plan* p) { return p->plan; }
rf_ctx* ctx_of(rf_plan* p) { return p->ctx; }
std::vector<rf_table*>& staging_of(rf_plan* p)
{
    if (p->staging.size() < (size_t)p->plan.n_inputs) p->staging.resize(p->plan.n_inputs, nullptr);
    return p->staging;
}
}  // namespace rfrt

// ------------------------------------------------------------------------------------------
// autotuner
// ------------------------------------------------------------------------------------------
// Hash group-by: times whole runs (each one's output freed) with the table at 160, 220 and 300
// slots per 100 estimated distinct keys and records the fastest, as slots per 100 keys, for the
// plan's query shape and the input's row-count bucket.  Its output's rows and their per-key
// counts do not depend on the sizing; a key's FP64 sum depends on the order its rows meet its
// slot in any case (atomics), and stays within the oracle's tolerance.
namespace {
int run_table(rf_plan* p, const rf_arg* args, int n_args, rf_table** out, cudaStream_t s);
}

static int tune_hash_table(rf_plan* p, const rf_arg* args, int n_args, int reps, int64_t* choice, double* ms)
{
    rf_ctx* ctx = p->ctx;
    const rfg::Plan& pl = p->plan;
    if (pl.drive_input < 0 || pl.drive_input >= n_args || !args || args[pl.drive_input].kind != RF_ARG_TABLE ||
        !args[pl.drive_input].table)
        return fail(ctx, RF_ERR_INVALID, "hash group-by tuning needs its input table");
    const long long rows = args[pl.drive_input].table->cols.empty() ? 0 : args[pl.drive_input].table->cols[0].logical;
    cudaStream_t s = ctx->stream;
    int best = 0, rc = RF_OK;
    double best_ms = 0;
    for (int f : {160, 220, 300}) {
        p->hg_factor_override = f;
        std::vector<double> v;
        for (int r = 0; r <= reps && !rc; r++) {
            rf_table* out = nullptr;
            const auto t0 = std::chrono::steady_clock::now();
            rc = run_table(p, args, n_args, &out, s);
            if (!rc && cudaStreamSynchronize(s) != cudaSuccess) rc = fail(ctx, RF_ERR_CUDA, "autotuner timing");
            const double x = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            if (out) rf_table_free(out);
            if (r) v.push_back(x);  // the first run is a warm-up
        }
        if (rc) break;
        std::sort(v.begin(), v.end());
        if (!best || v[v.size() / 2] < best_ms) {
            best = f;
            best_ms = v[v.size() / 2];
        }
    }
    p->hg_factor_override = 0;
    if (rc) return rc;
    int bucket = 0;
    while (bucket < 62 && (1LL << (bucket + 1)) <= rows) bucket++;
    {
        std::lock_guard<std::mutex> g(ctx->tune_mu);
        ctx->tune[pl.key][bucket] = best;
    }
    if (choice) *choice = best;
    if (ms) *ms = best_ms;
    return RF_OK;
}

namespace {
int tune_block_and_tiles(rf_plan* p, const rf_arg* args, int32_t n_args, int32_t reps, int64_t* tile_rows, double* ms);
}

extern "C" int rf_plan_tune(rf_plan* p, const rf_arg* args, int32_t n_args, int32_t reps, int64_t* tile_rows,
                            double* ms)
{
    if (!p) return RF_ERR_INVALID;
    rf_ctx* ctx = p->ctx;
    cudaSetDevice(ctx->device);
    const rfg::Plan& pl = p->plan;
    if (reps < 1) reps = 3;
    if (pl.kind == rfg::PlanKind::HASH_GROUP) return tune_hash_table(p, args, n_args, reps, tile_rows, ms);
    if (pl.out_is_table || (pl.kind != rfg::PlanKind::SCAN_REDUCE && pl.kind != rfg::PlanKind::GROUP_REDUCE))
        return fail(ctx, RF_ERR_UNSUPPORTED,
                    "the autotuner tunes the block size and tiling of Reduce scans and the table sizing of hash "
                    "group-bys");
    return tune_block_and_tiles(p, args, n_args, reps, tile_rows, ms);
}

namespace {
// the tiling of a Reduce scan at the plan's current kernels: tiles of 1K..32K rows timed on the
// given inputs, the fastest recorded for the plan's shape key and the inputs' size bucket
int tune_tiles(rf_plan* p, const rf_arg* args, int32_t n_args, int32_t reps, int64_t* tile_rows, double* ms)
{
    rf_ctx* ctx = p->ctx;
    const rfg::Plan& pl = p->plan;
    RfParams P;
    long long lo, hi;
    int rc = fill_params(p, args, n_args, P, lo, hi, true);
    if (rc) return rc;
    const long long rows = std::max<long long>(hi - lo, 1);
    cudaStream_t s = ctx->stream;
    cudaEvent_t e0, e1;
    CUDA_TRY(ctx, cudaEventCreate(&e0));
    CUDA_TRY(ctx, cudaEventCreate(&e1));
    long long best = 0;
    float best_ms = 0;
    // candidate tilings: 1K to 32K rows (no tile much larger than the input), and the tiles that
    // cut the rows into 1-4 whole waves of resident blocks (no partly filled last wave); a
    // multiple of 4 rows, so a tile starts where 4-row vector loads do
    std::vector<long long> cand;
    for (long long t = 1024; t <= 32768; t *= 2)
        if (t <= 2 * rows || cand.empty()) cand.push_back(t);
    for (int w = 1; w <= 4 && p->max_units > 0; w++) {
        const long long units = (long long)p->max_units * w;
        const long long t = ((rows + units - 1) / units + 3) & ~3LL;
        if (t >= 256 && t <= 65536 && std::find(cand.begin(), cand.end(), t) == cand.end()) cand.push_back(t);
    }
    // each timing runs k launches back to back (k such that they take about 2 ms: a short kernel
    // timed alone is mostly launch latency and its jitter), as a query stream runs them; the
    // median of `reps` timings, after one warm-up launch
    int k = 1;
    for (long long t : cand) {
        p->tile_override = t;
        std::vector<float> v;
        for (int r = 0; r <= reps && !rc; r++) {
            const int n = r ? k : 1;
            cudaEventRecord(e0, s);
            for (int i = 0; i < n && !rc; i++) rc = enqueue(p, args, n_args, s, nullptr);
            cudaEventRecord(e1, s);
            if (!rc && cudaEventSynchronize(e1) != cudaSuccess) rc = fail(ctx, RF_ERR_CUDA, "autotuner timing");
            float x = 0;
            cudaEventElapsedTime(&x, e0, e1);
            if (!r) {
                if (t == cand.front()) k = (int)std::max(1.0, std::min(64.0, std::ceil(2.0 / std::max(x, 1e-3f))));
                continue;  // the first run is a warm-up
            }
            v.push_back(x / (float)n);
        }
        if (rc) break;
        std::sort(v.begin(), v.end());
        const float med = v[v.size() / 2];
        if (!best || med < best_ms) {
            best = t;
            best_ms = med;
        }
    }
    p->tile_override = 0;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if ((rc = check_device_error(ctx))) return rc;
    int bucket = 0;
    while (bucket < 62 && (1LL << (bucket + 1)) <= rows) bucket++;
    {
        std::lock_guard<std::mutex> g(ctx->tune_mu);
        ctx->tune[pl.key][bucket] = best;
    }
    if (tile_rows) *tile_rows = best;
    if (ms) *ms = best_ms;
    return RF_OK;
}

// The plan's kernels and the buffers shaped by them, exchanged with a variant's (the variant
// then holds, and frees, the plan's former ones).
void swap_kernels(rf_plan* a, rf_plan* b)
{
    std::swap(a->plan, b->plan);
    std::swap(a->mod, b->mod);
    std::swap(a->fns, b->fns);
    std::swap(a->buf, b->buf);
    std::swap(a->partials, b->partials);
    std::swap(a->partials_bytes, b->partials_bytes);
    std::swap(a->counter, b->counter);
    std::swap(a->range, b->range);
    std::swap(a->dout, b->dout);
    std::swap(a->max_units, b->max_units);
    std::swap(a->reduce_units, b->reduce_units);
    std::swap(a->batch_fn, b->batch_fn);
    std::swap(a->batch_grid, b->batch_grid);
    std::swap(a->batch_smem, b->batch_smem);
    std::swap(a->batch_threads, b->batch_threads);
}

// Block size and tiling together: the plan's shape compiled at 128, 256 and 512 threads per block
// (a variant that cannot be resident is skipped), each variant's tiling tuned, and the fastest
// pair kept - the plan takes that variant's kernels, and later compiles of the same shape in
// this context start from that block size.  Results then come from the chosen kernels on every
// path (alone, batched, served), so they stay the same everywhere.
int tune_block_and_tiles(rf_plan* p, const rf_arg* args, int32_t n_args, int32_t reps, int64_t* tile_rows, double* ms)
{
    rf_ctx* ctx = p->ctx;
    int64_t best_tile = 0;
    double best_ms = 0;
    int best_threads = p->plan.threads;
    std::unique_ptr<rf_plan> best_variant;
    int rc = tune_tiles(p, args, n_args, reps, &best_tile, &best_ms);
    if (rc) return rc;
    if (!p->text.empty()) {
        std::shared_ptr<reffine::Func> fn;
        try {
            fn = reffine::parse_text(p->text);
        } catch (const std::exception& e) {
            return fail(ctx, RF_ERR_INVALID, "%s", e.what());
        }
        for (int threads : {128, 256, 512}) {
            if (threads == p->plan.threads) continue;
            std::unique_ptr<rf_plan> v;
            if (build_plan(ctx, fn, p->plan.vectorize, threads, v)) {
                if (v) rf_plan_free(v.release());
                continue;  // e.g. too much shared memory at this block size
            }
            int64_t t = 0;
            double m = 0;
            if (tune_tiles(v.get(), args, n_args, reps, &t, &m) == RF_OK && m < best_ms) {
                best_tile = t;
                best_ms = m;
                best_threads = threads;
                if (best_variant) rf_plan_free(best_variant.release());
                best_variant = std::move(v);
            } else {
                rf_plan_free(v.release());
            }
        }
        cudaGetLastError();
    }
    if (best_variant) {
        cudaStreamSynchronize(ctx->stream);
        swap_kernels(p, best_variant.get());
        rf_plan_free(best_variant.release());
    }
    if (!p->shape.empty()) {
        std::lock_guard<std::mutex> g(ctx->tune_mu);
        ctx->tune[p->shape][-1] = best_threads;
    }
    if (tile_rows) *tile_rows = best_tile;
    if (ms) *ms = best_ms;
    return RF_OK;
}
}  // namespace

extern "C" int rf_tune_export(rf_ctx* ctx, char* buf, size_t len, size_t* needed)
{
    if (!ctx) return RF_ERR_INVALID;
    std::string t;
    {
        std::lock_guard<std::mutex> g(ctx->tune_mu);
        for (auto& kv : ctx->tune)
            for (auto& b : kv.second) t += kv.first + " " + std::to_string(b.first) + " " + std::to_string(b.second) + "\n";
    }
    if (needed) *needed = t.size() + 1;
    if (buf && len) {
        size_t n = std::min(len - 1, t.size());
        memcpy(buf, t.data(), n);
        buf[n] = 0;
        if (n < t.size()) return fail(ctx, RF_ERR_INVALID, "buffer of %zu bytes holds %zu of the tuning table", len, n);
    }
    return RF_OK;
}

extern "C" int rf_tune_import(rf_ctx* ctx, const char* text)
{
    if (!ctx || !text) return RF_ERR_INVALID;
    std::istringstream in(text);
    std::string key;
    int bucket;
    long long tile;
    std::map<std::string, std::map<int, long long>> add;
    while (in >> key >> bucket >> tile) {
        const bool block = bucket == -1;  // the shape's block size
        if (block ? (tile != 128 && tile != 256 && tile != 512)
                  : (bucket < 0 || bucket > 62 || tile < 32 || tile > (1LL << 30)))
            return fail(ctx, RF_ERR_INVALID, "tuning entry %s %d %lld out of range", key.c_str(), bucket, tile);
        add[key][bucket] = tile;
    }
    if (!in.eof()) return fail(ctx, RF_ERR_INVALID, "malformed tuning table");
    std::lock_guard<std::mutex> g(ctx->tune_mu);
    for (auto& kv : add)
        for (auto& b : kv.second) ctx->tune[kv.first][b.first] = b.second;
    return RF_OK;
}

extern "C" int rf_plan_launch(rf_plan* p, const rf_arg* args, int32_t n_args, void* dev_out, void* stream)
{
    if (!p) return RF_ERR_INVALID;
    rf_ctx* ctx = p->ctx;
    cudaSetDevice(ctx->device);
    if (p->plan.out_is_table) return fail(ctx, RF_ERR_INVALID, "rf_plan_launch takes value-output plans");
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    int rc = enqueue(p, args, n_args, s, nullptr);
    if (rc) return rc;
    if (dev_out) CUDA_TRY(ctx, cudaMemcpyAsync(dev_out, p->dout, p->plan.out_size, cudaMemcpyDeviceToDevice, s));
    return RF_OK;
}

namespace rfrt {

// Distinct values of an int64 column, estimated with HyperLogLog (kernels.cu) and cached on the
// table (a table statistic, as a database keeps one; computed once per uploaded table).
// The most frequent keys of a flat int64 column 0, from a sample of up to 2^16 rows, most
// frequent first (keys seen at least twice when every row is sampled, else three times).
// Cached in the table.  The sample is counted in an open-addressing table (no sort of the
// sample: a table re-uploaded for every call of a query function pays this each time); which
// keys come out hot only decides which rows take the warp-fold path, never a result.
int hot_keys(rf_table* t, cudaStream_t s)
{
    std::lock_guard<std::mutex> g(t->stats_mu);
    if (t->hot_ready) return RF_OK;
    rf_ctx* ctx = t->ctx;
    DevCol& dc = t->cols[0];
    const long long n = dc.nvals, m = std::min<long long>(n, 1LL << 16);
    std::vector<long long> h((size_t)std::max<long long>(m, 0));
    if (m > 0) {
        long long* d = nullptr;
        CUDA_TRY(ctx, pool_alloc((void**)&d, (size_t)m * 8, s));
        int e = rf_k_sample_keys(dc.data, dc.valid, n, m, d, s);
        cudaError_t ce = (cudaError_t)e;
        if (ce == cudaSuccess) ce = cudaMemcpyAsync(h.data(), d, (size_t)m * 8, cudaMemcpyDeviceToHost, s);
        cudaFreeAsync(d, s);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
        if (ce != cudaSuccess) return fail(ctx, RF_ERR_CUDA, "key sample: %s", cudaGetErrorString(ce));
        ctx->launches += 1;
    }
    const long long minc = m == n ? 2 : 3;
    size_t cap = 16;
    while (cap < 2 * h.size()) cap *= 2;
    std::vector<long long> tk(cap, RF_EMPTY_KEY), tc(cap, 0);
    for (long long k : h) {
        if (k == RF_EMPTY_KEY) continue;
        size_t i = (size_t)(((unsigned long long)k * 0x9E3779B97F4A7C15ULL) >> 17) & (cap - 1);
        while (tk[i] != RF_EMPTY_KEY && tk[i] != k) i = (i + 1) & (cap - 1);
        tk[i] = k;
        tc[i]++;
    }
    std::vector<std::pair<long long, long long>> cnt;  // (count, key)
    for (size_t i = 0; i < cap; i++)
        if (tk[i] != RF_EMPTY_KEY && tc[i] >= minc) cnt.push_back({tc[i], tk[i]});
    std::sort(cnt.begin(), cnt.end(), [](const std::pair<long long, long long>& a, const std::pair<long long, long long>& b) {
        return a.first != b.first ? a.first > b.first : a.second < b.second;
    });
    if (cnt.size() > 8192) cnt.resize(8192);
    t->hot.clear();
    for (auto& c : cnt) t->hot.push_back(c.second);
    t->hot_ready = true;
    return RF_OK;
}

// The hot-key image a hash group-by plan's aggregation kernel copies into shared memory: an
// open-addressing index (capacity 2HK, a power of two; linear probing; the kernel's 32-bit
// multiplicative hash of the folded key) of the HK hottest keys with ids 0..HK-1, laid out
//   hk[2HK] i64 | hid[2HK] i32.
// Only which rows take which path depends on it, never a result.  Null: no hot keys.
static inline unsigned host_h32(long long key, unsigned mult, int bits)
{
    const unsigned f = (unsigned)key ^ (unsigned)((unsigned long long)key >> 32);
    return (f * mult) >> (32 - bits);
}

// The hot-key image the aggregation kernel copies to shared memory:
//   [u32 multiplier][u32 0] [i64 key of each of RF_HG_SLOTS_PER_KEY*HK slots] [u8 hot id per slot]
// The hottest keys are placed in hotness order, each in the single slot its hash names: the kernel
// finds a key with one probe and no loop.  Among 64 odd multipliers the one that places the most
// keys is used; a key whose slot is taken stays cold (it takes the global table's path).
int hot_image(rf_plan* p, rf_table* vt, cudaStream_t s, void** img)
{
    *img = nullptr;
    const int HK = p->plan.hg_hot;
    if (HK == 0) return RF_OK;
    int rc = hot_keys(vt, s);
    if (rc) return rc;
    if (p->hg_img_for == vt->gen) {
        *img = p->hg_img_some ? p->hg_img : nullptr;
        return RF_OK;
    }
    std::vector<long long> keys;
    {
        std::lock_guard<std::mutex> g(vt->stats_mu);
        keys = vt->hot;
    }
    p->hg_img_for = vt->gen;
    p->hg_img_some = !keys.empty();
    if (keys.empty()) return RF_OK;
    if ((int)keys.size() > HK) keys.resize(HK);
    const size_t HKS = (size_t)rfg::kHotSlotsPerKey * HK, bytes = 8 + HKS * 9;
    int bits = 0;
    while (((size_t)1 << bits) < HKS) bits++;
    std::vector<unsigned char> buf(bytes, 0);
    long long* hk = (long long*)(buf.data() + 8);
    unsigned char* hid = buf.data() + 8 + HKS * 8;
    unsigned best_mult = 0x9E3779B1u;
    size_t best_placed = 0;
    std::vector<char> used(HKS);
    for (unsigned t = 0; t < 64 && best_placed < keys.size(); t++) {
        const unsigned mult = 0x9E3779B1u + 2u * t * 0x10001u;
        std::fill(used.begin(), used.end(), 0);
        size_t placed = 0;
        for (long long k : keys) {
            const unsigned h = host_h32(k, mult, bits);
            if (!used[h]) used[h] = 1, placed++;
        }
        if (placed > best_placed) best_placed = placed, best_mult = mult;
    }
    std::fill(hk, hk + HKS, RF_EMPTY_KEY);
    for (size_t i = 0; i < keys.size(); i++) {
        const unsigned h = host_h32(keys[i], best_mult, bits);
        if (hk[h] != RF_EMPTY_KEY) continue;  // taken by a hotter key: this one stays cold
        hk[h] = keys[i];
        hid[h] = (unsigned char)i;
    }
    std::memcpy(buf.data(), &best_mult, 4);
    if (!grow(&p->hg_img, &p->hg_img_cap, bytes, s)) {
        p->hg_img_for = 0;
        return fail(p->ctx, RF_ERR_OOM, "hot-key image");
    }
    CUDA_TRY(p->ctx, cudaMemcpyAsync(p->hg_img, buf.data(), bytes, cudaMemcpyHostToDevice, s));
    CUDA_TRY(p->ctx, cudaStreamSynchronize(s));  // buf is released on return
    *img = p->hg_img;
    return RF_OK;
}

int ndv_estimate(rf_table* t, int col, cudaStream_t s, long long* out)
{
    std::lock_guard<std::mutex> g(t->stats_mu);
    rf_ctx* ctx = t->ctx;
    if ((int)t->ndv.size() <= col) t->ndv.resize(col + 1, -1);
    if (t->ndv[col] >= 0) {
        *out = t->ndv[col];
        return RF_OK;
    }
    DevCol& dc = t->cols[col];
    unsigned* regs = nullptr;
    CUDA_TRY(ctx, pool_alloc((void**)&regs, RF_HLL_M * sizeof(unsigned), s));
    int e = rf_k_hll(dc.data, dc.valid, dc.nvals, regs, s);
    if (e) {
        cudaFreeAsync(regs, s);
        return fail(ctx, RF_ERR_CUDA, "distinct-count sketch launch: %s", cudaGetErrorString((cudaError_t)e));
    }
    ctx->launches += 1;
    std::vector<unsigned> h(RF_HLL_M);
    cudaError_t ce = cudaMemcpyAsync(h.data(), regs, RF_HLL_M * sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(regs, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) return fail(ctx, RF_ERR_CUDA, "distinct-count sketch: %s", cudaGetErrorString(ce));
    double sum = 0, m = RF_HLL_M;
    int zeros = 0;
    for (unsigned r : h) {
        sum += std::ldexp(1.0, -(int)r);
        zeros += r == 0;
    }
    double est = 0.7213 / (1.0 + 1.079 / m) * m * m / sum;
    if (est <= 2.5 * m && zeros) est = m * std::log(m / zeros);
    long long v = (long long)(est + 0.5);
    if (v > dc.nvals) v = dc.nvals;
    t->ndv[col] = v;
    *out = v;
    return RF_OK;
}

}  // namespace rfrt

namespace {

// Runs an Op plan: allocates the output table (capacity = the loop's row range, so no 1e8-row
// preallocation as in loopgen.cpp:115), launches the materialisation kernels and sizes the table
// from the device counters (finalize_vector, vinstr.h:113-135).
int run_table(rf_plan* p, const rf_arg* args, int n_args, rf_table** out, cudaStream_t s)
{
    rf_ctx* ctx = p->ctx;
    const rfg::Plan& pl = p->plan;
    // a hash group-by's table lives for the run only (see below); an overflow's rerun grows it
    // first, and whichever table is current when the outermost run returns goes back to the pool
    struct ReleaseHashTable {
        rf_plan* p;
        cudaStream_t s;
        ~ReleaseHashTable()
        {
            if (p->hg_keys) cudaFreeAsync(p->hg_keys, s);
            p->hg_keys = nullptr;
            p->hg_keys_cap = 0;
        }
    };
    std::unique_ptr<ReleaseHashTable> release_hash;
    if (pl.kind == rfg::PlanKind::HASH_GROUP) release_hash.reset(new ReleaseHashTable{p, s});
    RfParams P;
    long long lo, hi;
    int rc = fill_params(p, args, n_args, P, lo, hi, true);
    if (rc) return rc;
    long long hg_cap = 0;
    if (pl.kind == rfg::PlanKind::HASH_GROUP) {
        // hash table of hg_factor_for() slots per 100 estimated distinct keys (default 220: load
        // 0.45, i.e. 0.5 with a 10% margin on the estimate); a probe overflow reruns with twice
        // the capacity
        rf_table* vt = args[pl.drive_input].table;
        long long ndv = 0;
        if ((rc = ndv_estimate(vt, 0, s, &ndv))) return rc;
        const int factor = hg_factor_for(p, vt->cols[0].logical);
        hg_cap = std::max<long long>(1024, (long long)((double)factor / 100.0 * (double)ndv));
        if (p->hg_retry_cap > hg_cap) hg_cap = p->hg_retry_cap;
        // slots of pl.acc_bytes bytes: {key, accumulators} (array of structs).  The table is
        // taken from the pool for this run and handed back when the run ends (stream-ordered):
        // a serving mix holds thousands of hash group-by plans (one per query's constants), and
        // each keeping its table measured 52 GB for 722 plans.
        if (!grow(&p->hg_keys, &p->hg_keys_cap, (size_t)(hg_cap + 1) * pl.acc_bytes, s))
            return fail(ctx, RF_ERR_OOM, "hash table allocation (%lld slots)", hg_cap);
        P.aux4 = p->hg_keys;
        P.aux_n0 = vt->cols[0].logical;
        P.aux_n1 = hg_cap;
        if ((rc = hot_image(p, vt, s, &P.aux5))) return rc;
        lo = 0;
        hi = hg_cap + 1;
        P.row_lo = lo;
        P.row_hi = hi;
    }
    long long cap = hi - lo;
    size_t nc = pl.out_cols.size();
    auto t = std::make_unique<rf_table>();
    t->ctx = ctx;
    t->dim = pl.out_dim;
    t->name = "out";
    t->cols.resize(nc);
    t->present.assign(nc, 1);
    std::vector<void*> hptrs(2 * RF_MAX_COLS, nullptr);
    // output columns of `rows` rows (validity bitmaps when vectorised)
    auto alloc_cols = [&](long long rows) -> int {
        for (size_t c = 0; c < nc; c++) {
            DevCol& dc = t->cols[c];
            dc.type = pl.out_cols[c];
            dc.name = (c < (size_t)pl.out_dim ? "it" : "out") +
                      std::to_string(c < (size_t)pl.out_dim ? c : c - pl.out_dim);
            size_t bytes = (size_t)std::max<long long>(rows, 1) * dc.type.size();
            if (pool_alloc(&dc.data_buf, bytes + 16, s) != cudaSuccess)
                return fail(ctx, RF_ERR_OOM, "output column allocation (%zu bytes) failed", bytes);
            dc.data_cap = bytes;
            dc.data = dc.data_buf;
            hptrs[c] = dc.data_buf;
            if (pl.vectorize) {
                size_t vb = (size_t)((std::max<long long>(rows, 1) + 31) / 32) * 4;
                if (pool_alloc(&dc.valid_buf, vb + 16, s) != cudaSuccess)
                    return fail(ctx, RF_ERR_OOM, "output bitmap allocation failed");
                dc.valid_cap = vb;
                CUDA_TRY(ctx, cudaMemsetAsync(dc.valid_buf, 0, vb + 16, s));
                hptrs[RF_MAX_COLS + c] = dc.valid_buf;
            }
        }
        CUDA_TRY(ctx, cudaMemcpyAsync(p->d_ptrs, hptrs.data(), sizeof(void*) * hptrs.size(), cudaMemcpyHostToDevice, s));
        return RF_OK;
    };
    // A compacting materialisation (count, scan, scatter) learns its row count from the scan: the
    // columns are then allocated at exactly that size before the scatter, so an output holds its
    // rows, not the loop's range (a hash group-by's slot table is ~2.2x the distinct keys).  A
    // vectorised one writes every visited element and is allocated at the range up front.
    // (a union merge knows its row count only after its scan, vectorised or not)
    const bool union_merge = pl.kind == rfg::PlanKind::UNION_MERGE;
    int iscatter = -1;
    for (size_t i = 0; i < pl.kernels.size(); i++)
        if (pl.kernels[i].role == rfg::KernelSpec::SCATTER && (!pl.vectorize || union_merge)) iscatter = (int)i;
    if (iscatter < 0 && (rc = alloc_cols(cap))) {
        free_table_mem(t.get());
        return rc;
    }
    long long ntiles = (hi - lo + P.tile_rows - 1) / P.tile_rows;
    if ((size_t)std::max<long long>(ntiles, 1) * 8 > p->tiles_cap) {  // tiles_cap: bytes
        if (!grow((void**)&p->d_tiles, &p->tiles_cap, (size_t)std::max<long long>(ntiles, 1024) * 8, s)) {
            free_table_mem(t.get());
            return fail(ctx, RF_ERR_OOM, "tile buffer allocation failed");
        }
    }
    CUDA_TRY(ctx, cudaMemsetAsync(p->d_res, 0, 64, s));
    P.aux0 = p->d_ptrs;
    P.aux1 = p->d_ptrs + RF_MAX_COLS;
    P.aux2 = p->d_tiles;
    P.aux3 = p->d_res;
    long long nruns = 0;
    if (pl.kind == rfg::PlanKind::SEG_REDUCE) {
        rf_table* vt = args[pl.drive_input].table;
        nruns = vt->cols[0].nvals;
        long long nrows = vt->cols[0].logical;
        size_t wmax = (size_t)(nruns + (nrows + pl.seg_chunk - 1) / pl.seg_chunk + 2);
        if (!grow((void**)&p->seg_woff, &p->seg_runs_cap, (size_t)(nruns + 2) * 8, s) ||
            !grow((void**)&p->seg_tmp, &p->seg_tmp_cap, (size_t)(nruns / 2048 + 4) * 8, s) ||
            !grow(&p->seg_part, &p->seg_part_cap, wmax * pl.acc_bytes, s)) {
            free_table_mem(t.get());
            return fail(ctx, RF_ERR_OOM, "segmented-reduce buffers");
        }
        P.aux4 = p->seg_woff;
        P.aux5 = p->seg_part;
    }
    if (union_merge) {
        // paired-row counts of the first vector, scanned in place (nA + 1 entries)
        rf_table* ta = args[pl.union_inputs[0]].table;
        rf_table* tb = args[pl.union_inputs[1]].table;
        if (!pl.vectorize && (ta->cols[0].valid || tb->cols[0].valid)) {
            free_table_mem(t.get());
            return fail(ctx, RF_ERR_UNSUPPORTED,
                        "a union over iterator columns with nulls is lowered in the vectorised form only");
        }
        nruns = ta->cols[0].nvals + 1;
        if (!grow((void**)&p->seg_woff, &p->seg_runs_cap, (size_t)(nruns + 1) * 8, s) ||
            !grow((void**)&p->seg_tmp, &p->seg_tmp_cap, (size_t)(nruns / 2048 + 4) * 8, s)) {
            free_table_mem(t.get());
            return fail(ctx, RF_ERR_OOM, "union merge buffers");
        }
        P.aux4 = p->seg_woff;
    }
    int units = units_for(p, ntiles);
    P.nunits = units;
    for (size_t i = 0; i < pl.kernels.size(); i++) {
        const auto& k = pl.kernels[i];
        if ((int)i == iscatter) {
            long long total = 0;
            CUDA_TRY(ctx, cudaMemcpyAsync(&total, p->d_res, 8, cudaMemcpyDeviceToHost, s));
            CUDA_TRY(ctx, cudaStreamSynchronize(s));
            if ((rc = check_device_error(ctx))) {
                free_table_mem(t.get());
                if (pl.kind == rfg::PlanKind::HASH_GROUP && rc == RF_ERR_DEVICE && hg_cap < (1LL << 34) &&
                    std::string(rf_last_error(ctx)).find("capacity") != std::string::npos) {
                    p->hg_retry_cap = hg_cap * 2;  // the estimate was low: grow and rerun
                    return run_table(p, args, n_args, out, s);
                }
                return rc;
            }
            if (total < 0 || total > cap) {
                free_table_mem(t.get());
                return fail(ctx, RF_ERR_DEVICE, "materialisation counted %lld rows of %lld", total, cap);
            }
            if ((rc = alloc_cols(total))) {
                free_table_mem(t.get());
                return rc;
            }
            cap = total;
        }
        if (k.role == rfg::KernelSpec::SEGSCAN) {
            int e = rf_k_scan_excl(p->seg_woff, nruns, p->seg_tmp, s);
            if (e) {
                free_table_mem(t.get());
                return fail(ctx, RF_ERR_CUDA, "segment scan launch: %s", cudaGetErrorString((cudaError_t)e));
            }
            ctx->launches += 3;
            continue;
        }
        int grid = units;
        if (k.role == rfg::KernelSpec::SEGCOUNT || k.role == rfg::KernelSpec::SEGREDUCE ||
            k.role == rfg::KernelSpec::INIT)
            grid = ctx->sm_count * 8;
        if (pl.kind == rfg::PlanKind::HASH_GROUP && k.role == rfg::KernelSpec::MAIN)
            grid = std::max(1, p->max_units * t_grid_share / 100);
        if (k.role == rfg::KernelSpec::RANGE || k.role == rfg::KernelSpec::SCAN) grid = 1;
        if (k.role == rfg::KernelSpec::STOP)
            grid = (int)std::min<long long>(std::max<long long>((hi - lo + 255) / 256, 1), ctx->sm_count * 8);
        if ((rc = launch(ctx, p->fns[i], grid, k.threads, k.smem, s, &P))) {
            free_table_mem(t.get());
            return rc;
        }
    }
    long long res[2] = {0, 0}, rng[2] = {lo, hi};
    CUDA_TRY(ctx, cudaMemcpyAsync(res, p->d_res, 16, cudaMemcpyDeviceToHost, s));
    if (pl.device_range) CUDA_TRY(ctx, cudaMemcpyAsync(rng, p->range, 16, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(ctx, cudaStreamSynchronize(s));
    rc = check_device_error(ctx);
    if (rc) {
        free_table_mem(t.get());
        if (pl.kind == rfg::PlanKind::HASH_GROUP && rc == RF_ERR_DEVICE && hg_cap < (1LL << 34) &&
            std::string(rf_last_error(ctx)).find("capacity") != std::string::npos) {
            p->hg_retry_cap = hg_cap * 2;  // the estimate was low: grow and rerun
            return run_table(p, args, n_args, out, s);
        }
        return rc;
    }
    long long rows = res[0];
    if (pl.vectorize && !union_merge) {
        long long a = std::max(lo, rng[0]), b = std::min(hi, rng[1]);
        rows = b > a ? b - a : 0;
    }
    if (rows > cap) {
        free_table_mem(t.get());
        return fail(ctx, RF_ERR_DEVICE, "materialisation wrote %lld rows into %lld", rows, cap);
    }
    t->null_count = pl.vectorize ? res[1] : 0;
    for (auto& dc : t->cols) {
        dc.nvals = rows;
        dc.logical = rows;
        // finalize_vector: no bitmap when nothing is null
        dc.valid = (pl.vectorize && t->null_count > 0) ? (unsigned short*)dc.valid_buf : nullptr;
    }
    *out = t.release();
    return RF_OK;
}

}  // namespace

extern "C" int rf_plan_run_noalloc(rf_plan* p, const rf_arg* args, int32_t n_args, void* host_out, void* stream)
{
    if (!p) return RF_ERR_INVALID;
    rf_ctx* ctx = p->ctx;
    cudaSetDevice(ctx->device);
    const rfg::Plan& pl = p->plan;
    if (pl.out_is_table || (pl.kind != rfg::PlanKind::SCAN_REDUCE && pl.kind != rfg::PlanKind::GROUP_REDUCE))
        return fail(ctx, RF_ERR_UNSUPPORTED, "rf_plan_run_noalloc runs Reduce (value-output) plans only");
    if (!host_out) return fail(ctx, RF_ERR_INVALID, "host_out is required");
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    void* base = nullptr;
    size_t cap = 0;
    int e = rf_k_noalloc_scratch(ctx->device, &base, &cap);
    if (e) return fail(ctx, RF_ERR_CUDA, "scratch address lookup failed: %s", cudaGetErrorString((cudaError_t)e));
    // RF_NOALLOC_LIMIT (bytes) can only lower the usable part of the array
    if (const char* lim = getenv("RF_NOALLOC_LIMIT")) {
        long long v = atoll(lim);
        if (v > 0 && (size_t)v < cap) cap = (size_t)v;
    }
    RfParams P;
    long long lo, hi;
    int rc = fill_params(p, args, n_args, P, lo, hi, false);
    if (rc) return rc;
    long long ntiles = (hi - lo + P.tile_rows - 1) / P.tile_rows;
    int units = units_for(p, ntiles);
    // layout: [counter 256][loop bounds 256][error word at 752][result at 768, 256-aligned]
    // [partials: units x max(acc_bytes, 8); every unit writes at least one 8-byte accumulator]
    const size_t err_at = 752, out_at = 768;
    size_t out_bytes = (pl.out_size + 255) / 256 * 256;
    size_t acc = pl.acc_bytes ? pl.acc_bytes : 8;
    size_t need = out_at + out_bytes + (size_t)units * acc;
    if (need > cap)
        return fail(ctx, RF_ERR_INVALID,
                    "rf_plan_run_noalloc: this run needs %zu bytes of scratch, the fixed array holds %zu "
                    "(use rf_plan_run)", need, cap);
    unsigned char* b = (unsigned char*)base;
    P.counter = (unsigned int*)b;
    P.range = pl.device_range ? (long long*)(b + 256) : nullptr;
    P.out = b + out_at;
    P.partials = b + out_at + out_bytes;
    P.nunits = units;
    // the last-unit-done merge counts arrivals from zero
    CUDA_TRY(ctx, cudaMemsetAsync(P.counter, 0, sizeof(unsigned int), s));
    for (size_t i = 0; i < pl.kernels.size(); i++) {
        const auto& k = pl.kernels[i];
        if (index_role(k.role)) continue;  // runs on the full index: same result, no allocation
        int grid = k.role == rfg::KernelSpec::RANGE ? 1
                   : k.role == rfg::KernelSpec::STOP
                       ? (int)std::min<long long>(std::max<long long>((hi - lo + 255) / 256, 1), ctx->sm_count * 8)
                       : units;
        if ((rc = launch(ctx, p->fns[i], grid, k.threads, k.smem, s, &P))) return rc;
    }
    // the error word is placed just before the result, so one copy brings back both; the result
    // reaches host_out only once the error word says the run succeeded (as in rf_plan_run)
    CUDA_TRY(ctx, cudaMemcpyAsync(b + err_at, ctx->dev_err, sizeof(int), cudaMemcpyDeviceToDevice, s));
    unsigned char small[16 + 4096];
    const bool one_copy = pl.out_size <= sizeof(small) - 16;
    const size_t back = one_copy ? 16 + pl.out_size : 16;
    CUDA_TRY(ctx, cudaMemcpyAsync(small, b + err_at, back, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(ctx, cudaStreamSynchronize(s));
    int err;
    memcpy(&err, small, sizeof(int));
    if ((rc = device_error(ctx, err))) return rc;
    if (one_copy) {
        memcpy(host_out, small + 16, pl.out_size);
    } else {  // a result larger than the stack buffer: a second copy, after the check
        CUDA_TRY(ctx, cudaMemcpyAsync(host_out, P.out, pl.out_size, cudaMemcpyDeviceToHost, s));
        CUDA_TRY(ctx, cudaStreamSynchronize(s));
    }
    return RF_OK;
}

extern "C" int rf_plan_run(rf_plan* p, const rf_arg* args, int32_t n_args, void* out, void* stream)
{
    if (!p) return RF_ERR_INVALID;
    rf_ctx* ctx = p->ctx;
    cudaSetDevice(ctx->device);
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    if (p->plan.out_is_table) {
        if (!out) return fail(ctx, RF_ERR_INVALID, "table output needs an rf_table** out");
        *(rf_table**)out = nullptr;
        return run_table(p, args, n_args, (rf_table**)out, s);
    }
    if (!p->h_res) {
        if (cudaHostAlloc((void**)&p->h_res, 16 + p->plan.out_size, cudaHostAllocDefault) != cudaSuccess)
            return fail(ctx, RF_ERR_OOM, "pinned result buffer");
    }
    int rc = enqueue(p, args, n_args, s, nullptr);
    if (rc) return rc;
    // the error word and the result come back in one round trip
    CUDA_TRY(ctx, cudaMemcpyAsync(p->h_res, ctx->dev_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(ctx, cudaMemcpyAsync(p->h_res + 16, p->dout, p->plan.out_size, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(ctx, cudaStreamSynchronize(s));
    int e;
    memcpy(&e, p->h_res, sizeof(int));
    if ((rc = device_error(ctx, e))) return rc;
    if (out) memcpy(out, p->h_res + 16, p->plan.out_size);
    return RF_OK;
}
