/*
 * rf_gpu.h - C-ABI of the GB300 execution backend for Reffine compiled queries.
 *
 * Plain C types only.  Every entry point returns an rf_status (0 = RF_OK) and never aborts or
 * exits; the message of the last failure on a context is rf_last_error(ctx).  Streams are
 * passed as `void*` (a cudaStream_t; NULL = the context's own stream).
 *
 * Reference interfaces these replace (Reffine, file:line):
 *   rf_gpu_init / rf_gpu_shutdown   ExecEngine::Get (src/engine/engine.cpp:24-39) and
 *                                   CudaEngine::Get (src/engine/cuda_engine.cpp:25-43)
 *   rf_table_upload / rf_table_free ArrowTable over ArrowArray/ArrowSchema (include/reffine/arrow/abi.h:56-69,
 *                                   include/reffine/arrow/table.h:15-151), made device-resident
 *   rf_table_build_index            ArrowTable2::build_index (include/reffine/arrow/table.h:107-138)
 *   rf_table_export                 the output ArrowTable handed back by make_vector/finalize_vector
 *                                   (src/vinstr/external.cpp:6-11, include/reffine/vinstr/vinstr.h:113-135)
 *   rf_plan_compile                 compile_op<FnTy>(Func, vectorize) (include/reffine/utils/utils.h:47-54):
 *                                   LoopGen + passes + codegen + ExecEngine::AddModule
 *   rf_plan_run / rf_plan_launch    calling the generated `extern "C" void fn(OutT* output_addr, inputs...)`
 *                                   (src/pass/cemitter.cpp:227-252, src/pass/canonpass.cpp:55-61)
 *   rf_plan_check                   the same lowering + compile, without a device (codegen checks)
 *   rf_plan_thunk                   ExecEngine::Lookup<FnTy>(name) (include/reffine/engine/engine.h:61-66):
 *                                   a host function pointer with the generated function's signature
 *   rf_batch_*                      no counterpart: batching of many queries into one persistent launch
 *   rf_server_*                     no counterpart: continuous-batching request loop
 *   rf_plan_tune, rf_tune_*         no counterpart: autotuner (scan tiling, hash-table sizing)
 *   rf_ipc_read, rf_table_load_ipc  load_arrow_file (src/utils/utils.cpp:11-34), without Arrow C++
 *   rf_last_error                   no counterpart: the reference exits or aborts on errors
 *                                   (src/engine/cuda_engine.cpp:10-23)
 */
#ifndef RF_GPU_H_
#define RF_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

struct ArrowSchema;
struct ArrowArray;

typedef struct rf_ctx rf_ctx;
typedef struct rf_table rf_table;
typedef struct rf_plan rf_plan;
typedef struct rf_batch rf_batch;

typedef enum rf_status {
    RF_OK = 0,
    RF_ERR_INVALID = 1,     /* malformed argument, IR text or table */
    RF_ERR_UNSUPPORTED = 2, /* query shape the GPU lowering does not map to a kernel template */
    RF_ERR_CUDA = 3,        /* CUDA runtime/driver error */
    RF_ERR_JIT = 4,         /* NVRTC compile or module load error */
    RF_ERR_OOM = 5,         /* device or pinned-host allocation failed */
    RF_ERR_DEVICE = 6,      /* a kernel reported an error (bounded wait or probe ran out) */
    RF_ERR_BUSY = 7,        /* a batch or queue is full */
    RF_ERR_CANCELLED = 8    /* a served request cancelled before it started */
} rf_status;

/* Argument of a plan run: a table or a scalar, in the Func's input order. */
typedef enum rf_arg_kind { RF_ARG_TABLE = 0, RF_ARG_I64 = 1, RF_ARG_F64 = 2 } rf_arg_kind;
typedef struct rf_arg {
    int32_t kind;     /* rf_arg_kind */
    int32_t pad_;
    rf_table* table;  /* RF_ARG_TABLE */
    int64_t i64;      /* RF_ARG_I64 (every integer / idx / bool scalar) */
    double f64;       /* RF_ARG_F64 (f32 / f64 scalars) */
} rf_arg;

/* Plan description, filled by rf_plan_info. */
typedef struct rf_plan_info_t {
    int32_t kind;             /* 1 = scan-reduce, 2 = grouped scan-reduce, 3 = materialise (Op),
                                 4 = run-end segmented reduce, 5 = hash group-by, 6 = merge join */
    int32_t n_inputs;         /* Func inputs */
    int32_t output_is_table;  /* 1: the Func returns a vector (rf_table*), 0: a value */
    int32_t n_groups;         /* grouped plans: number of key groups */
    int64_t output_size;      /* value outputs: bytes of the output struct (C layout) */
    int64_t bytes_per_row[8]; /* algorithmic input bytes per row, per table input (columns read) */
    int32_t n_kernels;        /* kernels one run launches */
    int32_t vectorize;
} rf_plan_info_t;

/* ---- context ---------------------------------------------------------------------------- */
int rf_gpu_init(int device, rf_ctx** out);
int rf_gpu_shutdown(rf_ctx* ctx);
const char* rf_last_error(rf_ctx* ctx);
/* The stream the context launches on when a call passes NULL. */
int rf_ctx_stream(rf_ctx* ctx, void** stream);
/* Synchronise the context's stream; reports device-side errors raised by earlier launches. */
int rf_ctx_sync(rf_ctx* ctx);
/* Counters: kernels launched by this context since creation (for launch accounting). */
int rf_ctx_launch_count(rf_ctx* ctx, int64_t* count);

/* Pinned host memory (for end-to-end host<->device staging). */
int rf_host_alloc(rf_ctx* ctx, size_t bytes, void** ptr);
int rf_host_free(rf_ctx* ctx, void* ptr);

/* ---- device-resident tables ------------------------------------------------------------- */
/* Copies a Reffine table (a struct array "+s" of flat or run-end encoded "+r" children, as
 * ArrowTable2 lays it out) to device memory.  `dim` is the number of iterator columns.  Host
 * buffers may be pageable or pinned (rf_host_alloc).  Arrays with a non-zero offset are
 * rejected (the reference ignores offsets). */
int rf_table_upload(rf_ctx* ctx, const struct ArrowSchema* schema, const struct ArrowArray* array,
                    int64_t dim, void* stream, rf_table** out);
/* Same, but copies only the listed columns (others stay absent on the device). */
int rf_table_upload_cols(rf_ctx* ctx, const struct ArrowSchema* schema, const struct ArrowArray* array,
                         int64_t dim, const int32_t* cols, int32_t n_cols, void* stream, rf_table** out);
int rf_table_free(rf_table* t);
/* Device hash index on column 0 (int64; run values for a run-end column): open addressing at
 * load factor 0.5, first occurrence wins, invalid rows skipped (table.h:107-138). */
int rf_table_build_index(rf_table* t, void* stream);
int rf_table_num_rows(rf_table* t, int64_t* rows);
int rf_table_num_cols(rf_table* t, int32_t* cols);
/* Device address and element count of a column buffer: part 0 = values (run values for a
 * run-end column), 1 = validity bitmap (NULL if all valid), 2 = run ends. */
int rf_table_column(rf_table* t, int32_t col, int32_t part, void** dev_ptr, int64_t* count);
/* Copies a device table back to host memory as Arrow C data (the caller releases both structs
 * through their release callbacks).  The output of an Op plan carries names "it0..", "out0..". */
int rf_table_export(rf_table* t, struct ArrowSchema* schema_out, struct ArrowArray* array_out);
/* Null count of the table (vectorised Op outputs mark filtered rows invalid). */
int rf_table_null_count(rf_table* t, int64_t* nulls);
/* One line per column, "name<TAB>format<TAB>flat|runend\n" (Arrow format strings: "l" int64,
 * "g" double, ...; a run-end column gives its values' format), written to buf (NUL-terminated,
 * truncated to len); *needed = the full text's length + 1.  The column types of
 * ArrowTable2::get_data_type (table.h:64-80) for a table that has no host-side schema. */
int rf_table_describe(rf_table* t, char* buf, size_t len, size_t* needed);
/* Arrow IPC ingest (load_arrow_file, src/utils/utils.cpp:11-34): record batch 0 of an Arrow
 * IPC file - integer, float and run-end encoded columns, uncompressed, no dictionaries.
 * rf_ipc_read needs no GPU: it returns the batch as Arrow C data (a "+s" struct of the
 * columns, as ArrowTable2 holds it; release both objects to free it); on failure `err` holds
 * the reason.  rf_table_load_ipc reads the file straight into a device table. */
int rf_ipc_read(const char* path, struct ArrowSchema* schema, struct ArrowArray* array, char* err, size_t err_len);
int rf_table_load_ipc(rf_ctx* ctx, const char* path, int64_t dim, void* stream, rf_table** out);

/* ---- plans -------------------------------------------------------------------------------- */
/* Lowers a Reffine Func (its text form, include/reffine_gb300/ir.h) onto a kernel template,
 * generates the query's device fragment and compiles it for sm_103a.  Queries that differ only
 * in constants share one compiled module.  `vectorize` has the meaning of compile_op's flag. */
int rf_plan_compile(rf_ctx* ctx, const char* func_text, int vectorize, rf_plan** out);
int rf_plan_free(rf_plan* plan);
/* The compile half of rf_plan_compile without a device: lowers `func_text` and compiles the
 * generated source for sm_103a with NVRTC.  On return `buf` (if not NULL) holds the generated
 * source, or the error message.  Needs no GPU and no context. */
int rf_plan_check(const char* func_text, int vectorize, char* buf, size_t buf_len);
int rf_plan_info(rf_plan* plan, rf_plan_info_t* info);
/* The generated CUDA source of a plan (valid while the plan lives). */
const char* rf_plan_source(rf_plan* plan);
/* Runs a plan over device tables and scalars and waits for it.
 *   value output: `out` points to host memory of rf_plan_info.output_size bytes receiving the
 *                 result in the C layout of the reference's output struct;
 *   table output: `out` is an rf_table** receiving a new device table. */
int rf_plan_run(rf_plan* plan, const rf_arg* args, int32_t n_args, void* out, void* stream);
/* Enqueues a run without waiting.  Value outputs land in device memory `dev_out`
 * (output_size bytes); table outputs are not allowed here. */
int rf_plan_launch(rf_plan* plan, const rf_arg* args, int32_t n_args, void* dev_out, void* stream);
/* rf_plan_run for callers that cannot allocate device memory while running queries - a host
 * with a fixed device-memory budget decided at start-up, or a latency-critical loop where a
 * cudaMalloc/cudaFree would synchronise the device.  It allocates nothing: the plan's partial
 * results, completion counter, loop bounds and result live in one fixed array of 4 MiB that the
 * library holds in device memory (on every device that loads it, until the process exits);
 * runs needing more are rejected with RF_ERR_INVALID and a message saying so (the environment
 * variable RF_NOALLOC_LIMIT, in bytes, lowers that limit; it cannot raise it).  Value-output
 * (Reduce) plans only, and every table a plan probes must already have its index
 * (rf_table_build_index), since building one allocates.  `host_out` receives the result, as in
 * rf_plan_run, and is left untouched when the run fails; the call waits for it.  The array is
 * set up by rf_gpu_init: it loads the module that holds the array and looks up its device
 * address (cudaGetSymbolAddress) with the device current, so no run does either.  All calls
 * share the array, which keeps the last call's contents (each run clears what must start at
 * zero): calls that overlap on the GPU (other threads or streams) race and must be serialised
 * by the caller.
 * No counterpart in the reference (its generated code runs on the host). */
int rf_plan_run_noalloc(rf_plan* plan, const rf_arg* args, int32_t n_args, void* host_out, void* stream);
/* A host function with the signature of the reference's generated query function:
 *   void fn(OutT* output_addr, ArrowTable* in0, ..., int64/double scalars ...)
 * Each call copies its host tables' referenced columns to the device, runs the plan and writes
 * the result to *output_addr (for a table output: a host ArrowTable* owned by the plan). */
int rf_plan_thunk(rf_plan* plan, void** fn);

/* ---- batching: many queries, one persistent launch -------------------------------------- */
int rf_batch_create(rf_ctx* ctx, int32_t capacity, rf_batch** out);
int rf_batch_free(rf_batch* b);
/* Adds a value-output run of `plan`; results land in host memory `host_out` after
 * rf_batch_wait.  Returns RF_ERR_BUSY when the batch is full. */
int rf_batch_add(rf_batch* b, rf_plan* plan, const rf_arg* args, int32_t n_args, void* host_out);
/* Launches everything added so far: one persistent kernel per query shape, in a CUDA graph
 * built once per set of shapes and size class and replayed when it recurs.  Ordered after the
 * work already queued on the context stream. */
int rf_batch_launch(rf_batch* b, void* stream);
int rf_batch_wait(rf_batch* b);
/* Non-blocking: *done = 1 once the launched batch has finished (its results are then copied as
 * by rf_batch_wait), 0 while it runs. */
int rf_batch_poll(rf_batch* b, int32_t* done);
int rf_batch_reset(rf_batch* b);

/* ---- autotuner (no reference counterpart) --------------------------------------------------
 * Times, on the given inputs, the tiling of a Reduce scan (rows per unit of work, 1K..32K), or
 * the table sizing of a hash group-by (160, 220 or 300 slots per 100 estimated distinct keys),
 * and records the fastest for the plan's query shape and the input's log2 row-count bucket;
 * every later run of that shape and bucket in this context (alone, batched, served) uses it.
 * *tile_rows receives the choice (tile rows, or slots per 100 keys).  Other table-output plans
 * are refused (RF_ERR_UNSUPPORTED).  The table of choices is exported and imported as text lines
 * "shape-key bucket choice". */
int rf_plan_tune(rf_plan* plan, const rf_arg* args, int32_t n_args, int32_t reps, int64_t* tile_rows, double* ms);
int rf_tune_export(rf_ctx* ctx, char* buf, size_t len, size_t* needed);
int rf_tune_import(rf_ctx* ctx, const char* text);

/* ---- serving: continuous batching over resident tables (no reference counterpart) ---------
 * A server owns a scheduler thread.  Batched mode packs the pending Reduce queries into
 * rf_batch launches on `lanes` streams as lanes free up (queries arriving while batches run
 * are launched as soon as a lane is free) and runs table-result queries one at a time on a
 * separate stream.  Per-query mode runs every request with rf_plan_run in arrival order (the
 * baseline).  Requests are admitted while the device scratch in flight stays within
 * hbm_budget_bytes; submit refuses with RF_ERR_BUSY once queue_capacity requests are pending.
 * Tables and plans must outlive the requests that use them; indexes must be built beforehand. */
typedef struct rf_server rf_server;
enum { RF_SERVE_BATCHED = 0, RF_SERVE_PER_QUERY = 1 };
typedef struct rf_server_config {
    int32_t mode;             /* RF_SERVE_BATCHED or RF_SERVE_PER_QUERY */
    int32_t max_batch;        /* queries per launch; 0: 256 */
    int32_t lanes;            /* batches in flight at once; 0: 2 */
    int32_t queue_capacity;   /* pending requests; 0: 65536 */
    int64_t hbm_budget_bytes; /* device scratch in flight; 0: 8 GiB */
    int32_t lane_share_pct;   /* a lane's launch fills at most this % of the block slots; 0: 75 */
    int32_t table_lanes;      /* batched mode: table-result queries running at once; 0: 1 */
    int32_t table_priority;   /* table-result lanes' streams: >= 0 the device's highest priority
                                 (default: their long single queries are not held behind batch
                                 blocks), < 0 normal priority */
    int32_t table_share_pct;  /* a table lane's hash aggregation fills at most this % of the block
                                 slots, leaving room for the batch lanes; 0: 100 */
} rf_server_config;
typedef struct rf_completion {
    uint64_t tag;             /* the submitter's tag */
    int32_t status;           /* rf_status of the run */
    int32_t batch_queries;    /* queries in the launch that carried it (1: alone) */
    int64_t t_submit_ns, t_launch_ns, t_done_ns; /* rf_clock_ns() times */
} rf_completion;
typedef struct rf_server_stats {
    int64_t submitted, completed, failed, cancelled, rejected;
    int64_t batches, batched_queries;
    int64_t queue_depth, max_queue_depth;
    int64_t inflight_bytes, peak_inflight_bytes, inflight_queries;
} rf_server_stats;
int64_t rf_clock_ns(void); /* monotonic clock of the completion records */
int rf_server_create(rf_ctx* ctx, const rf_server_config* cfg, rf_server** out);
/* Queues a run of `plan`; its value result (or, for a table result, its rf_table*) is written
 * to host_out before the completion with `tag` is delivered.  args are copied. */
int rf_server_submit(rf_server* s, rf_plan* plan, const rf_arg* args, int32_t n_args, void* host_out, uint64_t tag);
/* paused != 0: no queued request starts until resumed (requests on the GPU finish); submit,
 * cancel and poll keep working.  For draining, and to hold a queue in a known state. */
int rf_server_pause(rf_server* s, int32_t paused);
/* Removes a request that has not started; it completes with RF_ERR_CANCELLED. */
int rf_server_cancel(rf_server* s, uint64_t tag);
/* Takes up to max completions, waiting up to timeout_us for the first. */
int rf_server_poll(rf_server* s, rf_completion* out, int32_t max, int32_t* n_out, int32_t timeout_us);
int rf_server_get_stats(rf_server* s, rf_server_stats* out);
/* Pending requests complete as cancelled, work on the GPU finishes, then the server is freed. */
int rf_server_free(rf_server* s);
/* Open-loop load generator: submits request i at arrival_ns[i] after the call starts (tag i)
 * and returns when all have completed, with records[i] = request i's completion. */
int rf_server_replay(rf_server* s, int32_t n, rf_plan* const* plans, const rf_arg* const* args,
                     const int32_t* n_args, void* const* outs, const int64_t* arrival_ns, rf_completion* records);

#ifdef __cplusplus
}
#endif

#endif /* RF_GPU_H_ */
