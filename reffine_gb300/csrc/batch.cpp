// Batched execution: many queries, one persistent launch per query shape, replayed as a CUDA
// graph (rf_batch_*).
//
// The reference runs one query per call (compile_op's function, include/reffine/utils/utils.h:
// 47-54) and has no batching; this is the GB300 side's serving primitive.  A batch holds Reduce
// queries of any shapes.  Queries sharing a compiled shape run in one launch of that shape's
// rf_batch kernel (device/rf_templates.cuh), a persistent kernel whose blocks walk a work list
// of (query, unit) items; every query is cut into the units of its stand-alone launch and folded
// in the same order, so each result has the same bits alone or in the mix.  The launch sequence
// (parameter and work-list copies, counter reset, one kernel per shape, result copy) is built
// as a CUDA graph the first time a set of shapes is seen at a given size class and replayed
// afterwards.
#include <cuda_runtime_api.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "objects.h"
#include "runtime.h"

namespace {

struct Item {
    rf_plan* plan;
    RfParams P;
    void* host_out;
    int units;
    size_t out_off, part_off;
    int group;
};

struct Group {
    CUfunction fn;
    int grid, threads;
    size_t smem;
    std::vector<int> work;  // flattened {query, unit} pairs
};

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

size_t size_class(size_t n)
{
    size_t c = 16;
    while (c < n) c *= 2;
    return c;
}

}  // namespace

struct rf_batch {
    rf_ctx* ctx = nullptr;
    int cap = 0;
    std::vector<Item> items;
    std::vector<rf_plan*> groups_plan;
    // device buffers
    RfParams* d_params = nullptr;
    int* d_work = nullptr;      // per group: [count][pairs...], at group offsets
    unsigned char* d_scratch = nullptr;
    size_t work_cap = 0, scratch_cap = 0;
    // pinned host mirrors
    RfParams* h_params = nullptr;
    int* h_work = nullptr;
    unsigned char* h_out = nullptr;
    size_t h_work_cap = 0, h_out_cap = 0;
    // graph cache: signature -> executable graph
    std::map<std::string, cudaGraphExec_t> graphs;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    cudaEvent_t ctx_ready = nullptr;  // the context stream's work (uploads, index builds) so far
    cudaStream_t last_stream = nullptr;  // the stream of the previous launch
    int share_pct = 100;              // at most this share of a shape's resident blocks per launch
    bool in_flight = false;
    size_t out_bytes = 0, counters_bytes = 0;
};

using namespace rfrt;

namespace {

// Device buffers grow stream-ordered: the old one is released after the previous launch on
// `last` (the stream that used it), the new one is ready in `s`'s order; no device-wide sync.
int grow_dev(rf_ctx* ctx, void** p, size_t* cap, size_t bytes, cudaStream_t last, cudaStream_t s)
{
    if (*p && *cap >= bytes) return RF_OK;
    if (*p) cudaFreeAsync(*p, last);
    *p = nullptr;
    *cap = 0;
    bytes += bytes / 2;  // room to grow
    if (pool_alloc(p, bytes, s) != cudaSuccess)
        return fail(ctx, RF_ERR_OOM, "batch device buffer (%zu bytes)", bytes);
    *cap = bytes;
    return RF_OK;
}

int grow_host(rf_ctx* ctx, void** p, size_t* cap, size_t bytes)
{
    if (*p && *cap >= bytes) return RF_OK;
    if (*p) cudaFreeHost(*p);
    *p = nullptr;
    *cap = 0;
    bytes += bytes / 2;
    if (cudaHostAlloc(p, bytes, cudaHostAllocDefault) != cudaSuccess)
        return fail(ctx, RF_ERR_OOM, "batch pinned buffer (%zu bytes)", bytes);
    *cap = bytes;
    return RF_OK;
}

void drop_graphs(rf_batch* b)
{
    for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
    b->graphs.clear();
}

}  // namespace

extern "C" int rf_batch_create(rf_ctx* ctx, int32_t capacity, rf_batch** out)
{
    if (!ctx || !out || capacity <= 0) return RF_ERR_INVALID;
    *out = nullptr;
    cudaSetDevice(ctx->device);
    auto b = std::make_unique<rf_batch>();
    b->ctx = ctx;
    b->cap = capacity;
    CUDA_TRY(ctx, cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    CUDA_TRY(ctx, cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming));
    CUDA_TRY(ctx, cudaEventCreateWithFlags(&b->ctx_ready, cudaEventDisableTiming));
    CUDA_TRY(ctx, cudaMalloc((void**)&b->d_params, sizeof(RfParams) * (size_t)capacity));
    CUDA_TRY(ctx, cudaHostAlloc((void**)&b->h_params, sizeof(RfParams) * (size_t)capacity, cudaHostAllocDefault));
    b->items.reserve(capacity);
    *out = b.release();
    return RF_OK;
}

extern "C" int rf_batch_free(rf_batch* b)
{
    if (!b) return RF_OK;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->stream);
    drop_graphs(b);
    cudaFree(b->d_params);
    cudaFree(b->d_work);
    cudaFree(b->d_scratch);
    cudaFreeHost(b->h_params);
    cudaFreeHost(b->h_work);
    cudaFreeHost(b->h_out);
    cudaEventDestroy(b->done);
    cudaEventDestroy(b->ctx_ready);
    cudaStreamDestroy(b->stream);
    delete b;
    return RF_OK;
}

extern "C" int rf_batch_add(rf_batch* b, rf_plan* plan, const rf_arg* args, int32_t n_args, void* host_out)
{
    if (!b || !plan) return RF_ERR_INVALID;
    rf_ctx* ctx = b->ctx;
    if (b->in_flight) return fail(ctx, RF_ERR_BUSY, "batch is in flight: wait and reset it first");
    if ((int)b->items.size() >= b->cap) return fail(ctx, RF_ERR_BUSY, "batch is full (%d queries)", b->cap);
    if (!plan->batch_fn)
        return fail(ctx, RF_ERR_UNSUPPORTED, "only Reduce plans without device-computed loop bounds are batched");
    Item it{};
    it.plan = plan;
    it.host_out = host_out;
    long long lo, hi;
    int rc = fill_params(plan, args, n_args, it.P, lo, hi, true);
    if (rc) return rc;
    long long ntiles = (hi - lo + it.P.tile_rows - 1) / it.P.tile_rows;
    it.units = units_for(plan, ntiles);
    it.P.nunits = it.units;
    b->items.push_back(it);
    return RF_OK;
}

extern "C" int rf_batch_launch(rf_batch* b, void* stream)
{
    if (!b) return RF_ERR_INVALID;
    rf_ctx* ctx = b->ctx;
    cudaSetDevice(ctx->device);
    if (b->in_flight) return fail(ctx, RF_ERR_BUSY, "batch already launched");
    cudaStream_t s = stream ? (cudaStream_t)stream : b->stream;
    size_t n = b->items.size();
    if (n == 0) return RF_OK;
    // groups: one per compiled shape (module)
    std::vector<Group> groups;
    std::map<CUfunction, int> gid;
    for (auto& it : b->items) {
        auto f = gid.find(it.plan->batch_fn);
        if (f == gid.end()) {
            gid[it.plan->batch_fn] = (int)groups.size();
            groups.push_back({it.plan->batch_fn, it.plan->batch_grid, it.plan->batch_threads, it.plan->batch_smem, {}});
            f = gid.find(it.plan->batch_fn);
        }
        it.group = f->second;
    }
    // scratch layout, fixed by the size class so a replayed graph copies the right ranges:
    //   [error word, 16 B][ncls counters of 16 B][ncls result slots of OS B][partials of each query]
    // The first two parts are zeroed and the first three copied back by every launch.
    size_t ncls = size_class(n);
    size_t os = 16;
    for (auto& it : b->items) os = std::max(os, size_class(it.plan->plan.out_size));
    size_t counters_bytes = align_up(16 + 16 * ncls, 256);
    size_t outs_base = counters_bytes;
    size_t off = outs_base + align_up(ncls * os, 256);
    for (size_t i = 0; i < n; i++) {
        auto& it = b->items[i];
        it.out_off = outs_base + i * os;
        it.part_off = off;
        off = align_up(off + (size_t)it.units * it.plan->plan.acc_bytes, 16);
    }
    size_t scratch_need = off;
    void* scr = b->d_scratch;
    cudaStream_t last = b->last_stream ? b->last_stream : s;
    int rc = grow_dev(ctx, &scr, &b->scratch_cap, scratch_need, last, s);
    if (rc) return rc;
    if (scr != (void*)b->d_scratch) drop_graphs(b);
    b->d_scratch = (unsigned char*)scr;
    // work lists: per group [count, pad, pairs...]
    std::vector<size_t> goff(groups.size());
    size_t words = 0;
    for (size_t i = 0; i < n; i++) {
        auto& it = b->items[i];
        for (int u = 0; u < it.units; u++) {
            groups[it.group].work.push_back((int)i);
            groups[it.group].work.push_back(u);
        }
    }
    for (size_t g = 0; g < groups.size(); g++) {
        goff[g] = words;
        words += 2 + size_class(groups[g].work.size() / 2) * 2;
    }
    void* w = b->d_work;
    if ((rc = grow_dev(ctx, &w, &b->work_cap, words * 4, last, s))) return rc;
    if (w != (void*)b->d_work) drop_graphs(b);
    b->d_work = (int*)w;
    void* hw = b->h_work;
    if ((rc = grow_host(ctx, &hw, &b->h_work_cap, words * 4))) return rc;
    if (hw != (void*)b->h_work) drop_graphs(b);
    b->h_work = (int*)hw;
    for (size_t g = 0; g < groups.size(); g++) {
        int* p = b->h_work + goff[g];
        p[0] = (int)(groups[g].work.size() / 2);
        p[1] = 0;
        std::memcpy(p + 2, groups[g].work.data(), groups[g].work.size() * 4);
    }
    // parameter blocks point into the batch's scratch
    for (size_t i = 0; i < n; i++) {
        auto& it = b->items[i];
        RfParams P = it.P;
        P.counter = (unsigned int*)(b->d_scratch + 16 + 16 * i);
        P.err = (int*)b->d_scratch;
        P.out = b->d_scratch + it.out_off;
        P.partials = b->d_scratch + it.part_off;
        P.range = nullptr;
        b->h_params[i] = P;
    }
    b->out_bytes = ncls * os;
    b->counters_bytes = counters_bytes;
    void* ho = b->h_out;
    if ((rc = grow_host(ctx, &ho, &b->h_out_cap, counters_bytes + b->out_bytes))) return rc;
    if (ho != (void*)b->h_out) drop_graphs(b);
    b->h_out = (unsigned char*)ho;
    // graph: signature = shapes + size classes (copies are sized to the class)
    std::string sig = std::to_string(ncls) + ":" + std::to_string(b->out_bytes);
    for (size_t g = 0; g < groups.size(); g++)
        sig += "|" + std::to_string((uintptr_t)groups[g].fn) + "@" + std::to_string(goff[g]) + "/" +
               std::to_string(size_class(groups[g].work.size() / 2));
    auto gi = b->graphs.find(sig);
    if (gi == b->graphs.end()) {
        // built node by node (no stream capture, which would interact with other threads'
        // synchronising calls): three setup nodes, one kernel node per shape (the shapes run
        // concurrently), then the copy of error word, counters and results back to the host
        cudaGraph_t graph;
        CUDA_TRY(ctx, cudaGraphCreate(&graph, 0));
        cudaGraphNode_t setup[3], out_node;
        std::vector<cudaGraphNode_t> kn(groups.size());
        cudaMemsetParams ms{};
        ms.dst = b->d_scratch;
        ms.value = 0;
        ms.elementSize = 1;
        ms.width = counters_bytes;
        ms.height = 1;
        cudaError_t e = cudaGraphAddMemcpyNode1D(&setup[0], graph, nullptr, 0, b->d_params, b->h_params,
                                                 sizeof(RfParams) * std::min(ncls, (size_t)b->cap),
                                                 cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaGraphAddMemcpyNode1D(&setup[1], graph, nullptr, 0, b->d_work, b->h_work, words * 4,
                                         cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaGraphAddMemsetNode(&setup[2], graph, nullptr, 0, &ms);
        CUresult cr = CUDA_SUCCESS;
        for (size_t g = 0; g < groups.size() && e == cudaSuccess && cr == CUDA_SUCCESS; g++) {
            const RfParams* pp = b->d_params;
            const int* wl = b->d_work + goff[g] + 2;
            const int* nw = b->d_work + goff[g];
            void* kargs[] = {&pp, &wl, &nw};
            CUDA_KERNEL_NODE_PARAMS kp{};
            kp.func = groups[g].fn;
            int cap = std::max(1, groups[g].grid * b->share_pct / 100);
            kp.gridDimX = (unsigned)std::max(1, std::min(cap, (int)size_class(groups[g].work.size() / 2)));
            kp.gridDimY = kp.gridDimZ = 1;
            kp.blockDimX = (unsigned)groups[g].threads;
            kp.blockDimY = kp.blockDimZ = 1;
            kp.sharedMemBytes = (unsigned)groups[g].smem;
            kp.kernelParams = kargs;
            cr = drv().GraphAddKernelNode((CUgraphNode*)&kn[g], (CUgraph)graph, (const CUgraphNode*)setup, 3, &kp);
        }
        if (e == cudaSuccess && cr == CUDA_SUCCESS)
            e = cudaGraphAddMemcpyNode1D(&out_node, graph, kn.data(), kn.size(), b->h_out, b->d_scratch,
                                         counters_bytes + b->out_bytes, cudaMemcpyDeviceToHost);
        cudaGraphExec_t exec = nullptr;
        if (e == cudaSuccess && cr == CUDA_SUCCESS) e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (cr != CUDA_SUCCESS) return cu_fail(ctx, cr, "batch graph kernel node");
        if (e != cudaSuccess) return fail(ctx, RF_ERR_CUDA, "batch graph: %s", cudaGetErrorString(e));
        gi = b->graphs.emplace(sig, exec).first;
    }
    // the batch runs after everything already queued on the context stream (table uploads,
    // stream-ordered allocations, the index builds rf_batch_add may have enqueued)
    if (s != ctx->stream) {
        CUDA_TRY(ctx, cudaEventRecord(b->ctx_ready, ctx->stream));
        CUDA_TRY(ctx, cudaStreamWaitEvent(s, b->ctx_ready, 0));
    }
    CUDA_TRY(ctx, cudaGraphLaunch(gi->second, s));
    CUDA_TRY(ctx, cudaEventRecord(b->done, s));
    b->last_stream = s;
    ctx->launches += (long long)groups.size();
    b->in_flight = true;
    b->groups_plan.clear();
    return RF_OK;
}

extern "C" int rf_batch_wait(rf_batch* b)
{
    if (!b) return RF_ERR_INVALID;
    rf_ctx* ctx = b->ctx;
    cudaSetDevice(ctx->device);
    if (!b->in_flight) return RF_OK;
    CUDA_TRY(ctx, cudaEventSynchronize(b->done));
    b->in_flight = false;
    int e = 0;
    std::memcpy(&e, b->h_out, sizeof(int));
    if (e) return fail(ctx, RF_ERR_DEVICE, "device error %d in a batched query", e);
    for (auto& it : b->items)
        if (it.host_out) std::memcpy(it.host_out, b->h_out + it.out_off, it.plan->plan.out_size);
    return RF_OK;
}

extern "C" int rf_batch_poll(rf_batch* b, int32_t* done)
{
    if (!b || !done) return RF_ERR_INVALID;
    cudaSetDevice(b->ctx->device);
    if (!b->in_flight) {
        *done = 1;
        return RF_OK;
    }
    cudaError_t e = cudaEventQuery(b->done);
    if (e == cudaErrorNotReady) {
        *done = 0;
        return RF_OK;
    }
    *done = 1;
    return rf_batch_wait(b);
}

namespace rfrt {
// A launch of this batch fills at most `pct` percent of the block slots its kernels could hold,
// leaving the rest of every SM to batches launched beside it.  The grid only changes which
// block runs a work item, not the items or their fold order, so results are unchanged.
void batch_set_share(rf_batch* b, int pct)
{
    b->share_pct = std::min(100, std::max(1, pct));
    drop_graphs(b);
}
}  // namespace rfrt

extern "C" int rf_batch_reset(rf_batch* b)
{
    if (!b) return RF_ERR_INVALID;
    if (b->in_flight) return fail(b->ctx, RF_ERR_BUSY, "batch in flight: wait first");
    b->items.clear();
    return RF_OK;
}
