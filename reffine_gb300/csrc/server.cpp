// Continuous-batching query server over resident tables (rf_server_*).
//
// The reference has no serving path: a compiled query is one synchronous host call
// (compile_op's function, include/reffine/utils/utils.h:47-54) and ExecEngine is an unlocked
// singleton (src/engine/engine.cpp:24-39).  This server is the GB300 side's request loop.
//
//   client threads --submit--> pending queues --scheduler--> lanes (rf_batch, one stream each)
//                                              \--solo thread--> rf_plan_run (table outputs)
//
// Batched mode.  Value-result (Reduce) queries are packed into rf_batch launches: whenever a
// lane is free the scheduler takes the pending queries in arrival order, as many as fit the
// batch size and the device-memory budget, and launches them at once (one persistent kernel per
// query shape, a replayed CUDA graph).  Queries that arrive while batches run wait only for a
// free lane, not for the running batches to end, and the lanes' streams overlap on the device.
// Table-result queries (Op, hash group-by) run on table lanes beside the batches: cfg.table_lanes
// threads, each on its own stream, each taking the oldest pending table request whose plan no
// other lane is running (a plan's buffers serve one run at a time).  The table lanes' streams have
// the device's highest priority unless cfg.table_priority < 0: a table query is one long request,
// and behind the blocks of two batch lanes it set the tail (10k-request mix at the per-query
// path's capacity: p99 121 ms at normal priority, 5.8 ms at high, against 14.7 ms per-query).
//
// Per-query mode (the baseline).  One worker runs every request with rf_plan_run in arrival
// order: the reference's calling pattern, one call per query, on the same kernels.
//
// Admission by device memory.  Each request is charged the device scratch it needs while in
// flight (per-unit partials and result slots for a Reduce; output columns, tile counts and hash
// slots for a table result).  A request waits until the scratch in flight plus its own is within
// the budget; one that is larger than the whole budget runs alone once nothing else is in flight.
#include <cuda_runtime_api.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "objects.h"
#include "runtime.h"

using namespace rfrt;

namespace {

int64_t now_ns()
{
    return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

struct Req {
    rf_plan* plan = nullptr;
    std::vector<rf_arg> args;
    void* host_out = nullptr;
    uint64_t tag = 0;
    int64_t t_submit = 0, t_launch = 0;
    size_t footprint = 0;
};

struct Lane {
    rf_batch* batch = nullptr;
    cudaStream_t stream = nullptr;
    std::vector<Req> reqs;
    size_t footprint = 0;
    bool busy = false;
};

// device scratch a request holds while in flight
size_t footprint_of(rf_plan* p, long long lo, long long hi)
{
    const rfg::Plan& pl = p->plan;
    long long rows = std::max<long long>(hi - lo, 0);
    if (!pl.out_is_table) {
        long long ntiles = (rows + pl.tile_rows - 1) / pl.tile_rows;
        long long units = units_for(p, ntiles);
        return (size_t)units * pl.acc_bytes + 2 * std::max<size_t>(pl.out_size, 16) + sizeof(RfParams);
    }
    size_t row_bytes = 8;
    for (auto& c : pl.out_cols) row_bytes += c.size();
    size_t bytes = (size_t)rows * row_bytes + (size_t)(rows / pl.tile_rows + 2) * 8;
    if (pl.kind == rfg::PlanKind::HASH_GROUP) bytes += (size_t)rows * 2 * (8 + pl.acc_bytes);
    return bytes;
}

}  // namespace

struct rf_server {
    rf_ctx* ctx = nullptr;
    rf_server_config cfg{};
    std::mutex mu;
    std::condition_variable work_cv;  // new requests, stop
    std::condition_variable done_cv;  // new completions
    std::deque<Req> pend_batch;       // batched mode: Reduce queries; per-query mode: everything
    std::deque<Req> pend_solo;        // batched mode: table-result queries
    std::deque<rf_completion> done;
    size_t inflight_bytes = 0;
    size_t reserved = 0;              // scratch held for the table-result request waiting to start
    int inflight_reqs = 0;
    bool stop = false;
    bool paused = false;              // no new work starts (work in flight finishes)
    std::thread sched;
    std::vector<std::thread> solos;   // table lanes (batched mode) or the one per-query worker
    std::vector<Lane> lanes;
    std::vector<cudaStream_t> solo_streams;
    std::vector<rf_plan*> solo_busy;  // plans running on a table lane now
    rf_server_stats st{};
};

namespace {

void push_done(rf_server* S, const Req& r, int status, int batch_queries, int64_t t_done)
{
    rf_completion c{};
    c.tag = r.tag;
    c.status = status;
    c.batch_queries = batch_queries;
    c.t_submit_ns = r.t_submit;
    c.t_launch_ns = r.t_launch;
    c.t_done_ns = t_done;
    S->done.push_back(c);
    if (status == RF_OK) S->st.completed++;
    else if (status == RF_ERR_CANCELLED) S->st.cancelled++;
    else S->st.failed++;
}

// under S->mu: may a batched request of `fp` bytes start now, `taken` bytes already picked for
// the same launch?  Scratch that a waiting table-result request has reserved counts as used, so
// a stream of small queries cannot hold a large one back for ever.
bool fits(rf_server* S, size_t fp, size_t taken)
{
    size_t budget = (size_t)S->cfg.hbm_budget_bytes;
    if (S->inflight_bytes + taken + fp + S->reserved <= budget) return true;
    return S->inflight_bytes + taken == 0 && S->reserved == 0;  // larger than the budget: alone
}

bool fits_solo(rf_server* S, size_t fp)
{
    return S->inflight_bytes + fp <= (size_t)S->cfg.hbm_budget_bytes || S->inflight_bytes == 0;
}

void charge(rf_server* S, size_t fp, int n)
{
    S->inflight_bytes += fp;
    S->inflight_reqs += n;
    S->st.peak_inflight_bytes = std::max<int64_t>(S->st.peak_inflight_bytes, (int64_t)S->inflight_bytes);
}

void release(rf_server* S, size_t fp, int n)
{
    S->inflight_bytes -= fp;
    S->inflight_reqs -= n;
}

// Batched mode's scheduler: retire finished lanes, then fill free lanes.
void sched_loop(rf_server* S)
{
    cudaSetDevice(S->ctx->device);
    for (;;) {
        bool progressed = false;
        for (auto& ln : S->lanes) {
            if (!ln.busy) continue;
            int32_t fin = 0;
            int rc = rf_batch_poll(ln.batch, &fin);
            if (!rc && !fin) continue;
            int64_t t = now_ns();
            rf_batch_reset(ln.batch);
            std::lock_guard<std::mutex> lk(S->mu);
            for (auto& r : ln.reqs) push_done(S, r, rc, (int)ln.reqs.size(), t);
            release(S, ln.footprint, (int)ln.reqs.size());
            ln.reqs.clear();
            ln.footprint = 0;
            ln.busy = false;
            progressed = true;
            S->done_cv.notify_all();
            S->work_cv.notify_all();  // the solo thread may be waiting for budget
        }
        for (auto& ln : S->lanes) {
            if (ln.busy) continue;
            {
                std::lock_guard<std::mutex> lk(S->mu);
                if (S->paused) break;
                size_t taken = 0;
                while (!S->pend_batch.empty() && (int)ln.reqs.size() < S->cfg.max_batch &&
                       fits(S, S->pend_batch.front().footprint, taken)) {
                    taken += S->pend_batch.front().footprint;
                    ln.reqs.push_back(std::move(S->pend_batch.front()));
                    S->pend_batch.pop_front();
                }
                if (ln.reqs.empty()) break;
                charge(S, taken, (int)ln.reqs.size());
                ln.footprint = taken;
            }
            int64_t t = now_ns();
            std::vector<int> bad(ln.reqs.size(), 0);
            int added = 0;
            for (size_t i = 0; i < ln.reqs.size(); i++) {
                auto& r = ln.reqs[i];
                r.t_launch = t;
                bad[i] = rf_batch_add(ln.batch, r.plan, r.args.data(), (int32_t)r.args.size(), r.host_out);
                if (!bad[i]) added++;
            }
            int lrc = added ? rf_batch_launch(ln.batch, ln.stream) : RF_OK;
            std::lock_guard<std::mutex> lk(S->mu);
            if (lrc || added < (int)ln.reqs.size()) {
                // requests the batch refused (and all of them if the launch failed) end here
                std::vector<Req> keep;
                size_t keep_fp = 0;
                int64_t td = now_ns();
                for (size_t i = 0; i < ln.reqs.size(); i++) {
                    if (bad[i] || lrc) push_done(S, ln.reqs[i], bad[i] ? bad[i] : lrc, (int)ln.reqs.size(), td);
                    else {
                        keep_fp += ln.reqs[i].footprint;
                        keep.push_back(std::move(ln.reqs[i]));
                    }
                }
                release(S, ln.footprint - keep_fp, (int)(ln.reqs.size() - keep.size()));
                ln.reqs = std::move(keep);
                ln.footprint = keep_fp;
                if (lrc) rf_batch_reset(ln.batch);
                S->done_cv.notify_all();
            }
            if (!ln.reqs.empty()) {
                ln.busy = true;
                S->st.batches++;
                S->st.batched_queries += (int64_t)ln.reqs.size();
            }
            progressed = true;
        }
        if (progressed) continue;
        bool any_busy = false;
        for (auto& ln : S->lanes) any_busy |= ln.busy;
        if (any_busy) {
            std::this_thread::yield();  // completion is seen by polling the lanes' events
            continue;
        }
        std::unique_lock<std::mutex> lk(S->mu);
        if (S->stop && S->pend_batch.empty()) return;
        S->work_cv.wait_for(lk, std::chrono::milliseconds(2), [&] {
            return S->stop ||
                   (!S->paused && !S->pend_batch.empty() && fits(S, S->pend_batch.front().footprint, 0));
        });
    }
}

// Runs requests one at a time with rf_plan_run: a table lane of batched mode (several may run
// beside each other), or the whole of per-query mode (one worker, arrival order).
void solo_loop(rf_server* S, std::deque<Req>* q, cudaStream_t stream)
{
    cudaSetDevice(S->ctx->device);
    if (S->cfg.mode == RF_SERVE_BATCHED) set_thread_grid_share(S->cfg.table_share_pct);
    auto busy = [&](rf_plan* p) {
        return std::find(S->solo_busy.begin(), S->solo_busy.end(), p) != S->solo_busy.end();
    };
    for (;;) {
        Req r;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            for (;;) {
                auto it = q->begin();
                while (it != q->end() && busy(it->plan)) ++it;
                if (it == q->end()) {
                    if (q->empty()) S->reserved = 0;
                    if (S->stop && q->empty()) return;
                    S->work_cv.wait(lk);
                    continue;
                }
                if (S->paused && !S->stop) {
                    S->work_cv.wait(lk);
                    continue;
                }
                if (fits_solo(S, it->footprint)) {
                    if (it->footprint >= S->reserved) S->reserved = 0;  // the request that reserved
                    r = std::move(*it);
                    q->erase(it);
                    break;
                }
                S->reserved = std::max(S->reserved, it->footprint);
                S->work_cv.wait(lk);
            }
            S->solo_busy.push_back(r.plan);
            charge(S, r.footprint, 1);
        }
        r.t_launch = now_ns();
        int rc = rf_plan_run(r.plan, r.args.data(), (int32_t)r.args.size(), r.host_out, stream);
        int64_t t = now_ns();
        std::lock_guard<std::mutex> lk(S->mu);
        S->solo_busy.erase(std::find(S->solo_busy.begin(), S->solo_busy.end(), r.plan));
        push_done(S, r, rc, 1, t);
        release(S, r.footprint, 1);
        S->done_cv.notify_all();
        S->work_cv.notify_all();
    }
}

}  // namespace

extern "C" int64_t rf_clock_ns(void) { return now_ns(); }

extern "C" int rf_server_create(rf_ctx* ctx, const rf_server_config* cfg, rf_server** out)
{
    if (!ctx || !out) return RF_ERR_INVALID;
    *out = nullptr;
    cudaSetDevice(ctx->device);
    auto S = std::make_unique<rf_server>();
    S->ctx = ctx;
    rf_server_config c{};
    if (cfg) c = *cfg;
    if (c.max_batch <= 0) c.max_batch = 256;
    if (c.lanes <= 0) c.lanes = 2;
    if (c.lanes > 16) c.lanes = 16;
    if (c.queue_capacity <= 0) c.queue_capacity = 1 << 16;
    if (c.hbm_budget_bytes <= 0) c.hbm_budget_bytes = (int64_t)8 << 30;
    if (c.lane_share_pct <= 0 || c.lane_share_pct > 100) c.lane_share_pct = 75;
    if (c.table_lanes <= 0) c.table_lanes = 1;
    if (c.table_share_pct <= 0 || c.table_share_pct > 100) c.table_share_pct = 100;
    if (c.table_lanes > 16) c.table_lanes = 16;
    if (c.mode == RF_SERVE_PER_QUERY) c.table_lanes = 1;  // the baseline: one call at a time
    if (c.mode != RF_SERVE_BATCHED && c.mode != RF_SERVE_PER_QUERY)
        return fail(ctx, RF_ERR_INVALID, "unknown serving mode %d", c.mode);
    S->cfg = c;
    if (c.mode == RF_SERVE_BATCHED) {
        S->lanes.resize(c.lanes);
        for (auto& ln : S->lanes) {
            int rc = rf_batch_create(ctx, c.max_batch, &ln.batch);
            if (rc) {
                for (auto& l2 : S->lanes)
                    if (l2.batch) rf_batch_free(l2.batch);
                return rc;
            }
            batch_set_share(ln.batch, c.lane_share_pct);
            CUDA_TRY(ctx, cudaStreamCreateWithFlags(&ln.stream, cudaStreamNonBlocking));
        }
    }
    int prio_least = 0, prio_greatest = 0;
    if (c.table_priority >= 0 && c.mode == RF_SERVE_BATCHED) cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
    S->solo_streams.resize(c.table_lanes, nullptr);
    for (auto& st : S->solo_streams)
        CUDA_TRY(ctx, cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, prio_greatest));
    rf_server* raw = S.release();
    if (c.mode == RF_SERVE_BATCHED) {
        raw->sched = std::thread(sched_loop, raw);
        for (auto st : raw->solo_streams) raw->solos.emplace_back(solo_loop, raw, &raw->pend_solo, st);
    } else {
        raw->solos.emplace_back(solo_loop, raw, &raw->pend_batch, raw->solo_streams[0]);
    }
    *out = raw;
    return RF_OK;
}

extern "C" int rf_server_submit(rf_server* S, rf_plan* plan, const rf_arg* args, int32_t n_args, void* host_out,
                                uint64_t tag)
{
    if (!S || !plan || (n_args > 0 && !args)) return RF_ERR_INVALID;
    Req r;
    r.t_submit = now_ns();
    r.plan = plan;
    r.args.assign(args, args + n_args);
    r.host_out = host_out;
    r.tag = tag;
    // validate now (inputs, bound indexes) and size the request's scratch
    RfParams P;
    long long lo, hi;
    int rc = fill_params(plan, args, n_args, P, lo, hi, false);
    if (rc) return rc;
    r.footprint = footprint_of(plan, lo, hi);
    // batched: Reduce plans with host-known loop bounds; the rest run on the solo lane
    bool batched = S->cfg.mode == RF_SERVE_BATCHED && plan->batch_fn;
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return fail(S->ctx, RF_ERR_INVALID, "server is shutting down");
    size_t depth = S->pend_batch.size() + S->pend_solo.size();
    if ((int64_t)depth >= S->cfg.queue_capacity) {
        S->st.rejected++;
        return fail(S->ctx, RF_ERR_BUSY, "request queue full (%d)", S->cfg.queue_capacity);
    }
    (batched || S->cfg.mode == RF_SERVE_PER_QUERY ? S->pend_batch : S->pend_solo).push_back(std::move(r));
    S->st.submitted++;
    S->st.max_queue_depth = std::max<int64_t>(S->st.max_queue_depth, (int64_t)depth + 1);
    S->work_cv.notify_all();
    return RF_OK;
}

extern "C" int rf_server_pause(rf_server* S, int32_t paused)
{
    if (!S) return RF_ERR_INVALID;
    std::lock_guard<std::mutex> lk(S->mu);
    S->paused = paused != 0;
    S->work_cv.notify_all();
    return RF_OK;
}

extern "C" int rf_server_cancel(rf_server* S, uint64_t tag)
{
    if (!S) return RF_ERR_INVALID;
    std::lock_guard<std::mutex> lk(S->mu);
    for (auto* q : {&S->pend_batch, &S->pend_solo}) {
        for (auto it = q->begin(); it != q->end(); ++it) {
            if (it->tag != tag) continue;
            push_done(S, *it, RF_ERR_CANCELLED, 0, now_ns());
            q->erase(it);
            S->done_cv.notify_all();
            return RF_OK;
        }
    }
    return fail(S->ctx, RF_ERR_INVALID, "request %llu is not pending (already started or unknown)",
                (unsigned long long)tag);
}

extern "C" int rf_server_poll(rf_server* S, rf_completion* out, int32_t max, int32_t* n_out, int32_t timeout_us)
{
    if (!S || !n_out || (max > 0 && !out)) return RF_ERR_INVALID;
    *n_out = 0;
    std::unique_lock<std::mutex> lk(S->mu);
    if (S->done.empty() && timeout_us > 0)
        S->done_cv.wait_for(lk, std::chrono::microseconds(timeout_us), [&] { return !S->done.empty(); });
    int32_t n = 0;
    while (n < max && !S->done.empty()) {
        out[n++] = S->done.front();
        S->done.pop_front();
    }
    *n_out = n;
    return RF_OK;
}

extern "C" int rf_server_get_stats(rf_server* S, rf_server_stats* st)
{
    if (!S || !st) return RF_ERR_INVALID;
    std::lock_guard<std::mutex> lk(S->mu);
    *st = S->st;
    st->queue_depth = (int64_t)(S->pend_batch.size() + S->pend_solo.size());
    st->inflight_bytes = (int64_t)S->inflight_bytes;
    st->inflight_queries = S->inflight_reqs;
    return RF_OK;
}

extern "C" int rf_server_free(rf_server* S)
{
    if (!S) return RF_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        // pending requests end as cancelled; work already on the GPU finishes
        for (auto* q : {&S->pend_batch, &S->pend_solo}) {
            for (auto& r : *q) push_done(S, r, RF_ERR_CANCELLED, 0, now_ns());
            q->clear();
        }
        S->stop = true;
        S->work_cv.notify_all();
    }
    if (S->sched.joinable()) S->sched.join();
    for (auto& th : S->solos)
        if (th.joinable()) th.join();
    cudaSetDevice(S->ctx->device);
    for (auto& ln : S->lanes) {
        rf_batch_free(ln.batch);
        cudaStreamDestroy(ln.stream);
    }
    for (auto st : S->solo_streams) cudaStreamDestroy(st);
    delete S;
    return RF_OK;
}

extern "C" int rf_server_replay(rf_server* S, int32_t n, rf_plan* const* plans, const rf_arg* const* args,
                                const int32_t* n_args, void* const* outs, const int64_t* arrival_ns,
                                rf_completion* records)
{
    if (!S || n < 0 || (n > 0 && (!plans || !args || !n_args || !outs || !arrival_ns || !records)))
        return RF_ERR_INVALID;
    std::vector<char> seen(n, 0);
    int32_t finished = 0;
    std::vector<rf_completion> buf(256);
    auto drain = [&](int32_t timeout_us) {
        int32_t got = 0;
        rf_server_poll(S, buf.data(), (int32_t)buf.size(), &got, timeout_us);
        for (int32_t k = 0; k < got; k++) {
            uint64_t i = buf[k].tag;
            if (i < (uint64_t)n && !seen[i]) {
                seen[i] = 1;
                records[i] = buf[k];
                finished++;
            }
        }
    };
    int64_t t0 = now_ns(), last = t0;
    for (int32_t i = 0; i < n; i++) {
        int64_t due = t0 + arrival_ns[i];
        for (int64_t t = now_ns(); t < due; t = now_ns()) {
            if (t - last > 50000) {  // collect completions now and then, off the server's lock otherwise
                drain(0);
                last = t;
            }
        }
        int rc = rf_server_submit(S, plans[i], args[i], n_args[i], outs[i], (uint64_t)i);
        if (rc) {
            // refused at admission (queue full, invalid input): recorded, not retried
            rf_completion c{};
            c.tag = (uint64_t)i;
            c.status = rc;
            c.t_submit_ns = c.t_launch_ns = c.t_done_ns = now_ns();
            records[i] = c;
            seen[i] = 1;
            finished++;
        }
    }
    while (finished < n) drain(1000);
    return RF_OK;
}
