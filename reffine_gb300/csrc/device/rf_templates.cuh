// Kernel templates of the GB300 backend.  Included by a generated query source AFTER the
// query's fragment (the templates use the fragment's types and functions), once per source.
#pragma once

// loads a lane issues ahead of its combines in the last unit's fold over all units' partials
#ifndef RF_FOLD
#define RF_FOLD 16
#endif
#ifndef RF_FOLD_ACC
#define RF_FOLD_ACC 4
#endif

// ---------------------------------------------------------------------------------------
// Template 1: fused scan-filter-project-reduce.
//   The fragment defines: struct RfAcc (8-byte aligned fields, size a multiple of 8),
//   rf_acc_init(P, A), rf_acc_combine(A, B) (A <- A op B), rf_acc_shfl(A, off),
//   rf_row(P, r, A) (one row) and rf_finish(P, A, out).
// Work is split into fixed tiles of P.tile_rows rows; unit u takes the contiguous tiles
// [u*ntiles/nunits, (u+1)*ntiles/nunits).  Each unit's accumulator goes to P.partials[u]; the
// last unit to finish folds the partials in a fixed order.  So the result depends only on (rows,
// tile_rows, nunits, threads), not on scheduling: a query gives the same bits alone, batched with
// others, or launched a range of units at a time as its rows arrive (P.unit0).
// ---------------------------------------------------------------------------------------
#ifdef RF_SCAN_REDUCE
template <int T>
RF_DEV void rf_scan_reduce_rows(const RfParams& P, int unit, int nunits, RfAcc& acc)
{
    long long lo = P.row_lo, hi = P.row_hi;
    if (P.range) {
        long long b = P.range[0], e = P.range[1];
        lo = b > lo ? b : lo;
        hi = e < hi ? e : hi;
    }
    const long long tr = P.tile_rows;
    const long long ntiles = (P.row_hi - P.row_lo + tr - 1) / tr;
    const long long t_end = (long long)(unit + 1) * ntiles / nunits;
    for (long long tile = (long long)unit * ntiles / nunits; tile < t_end; tile++) {
        long long r0 = P.row_lo + tile * tr, r1 = r0 + tr;
        if (r1 > hi) r1 = hi;
        if (r0 < lo) r0 = lo;
#ifdef RF_VEC4
        if ((P.flags & RF_FLAG_VEC4) && r0 >= 0) {
            // a thread takes 4 consecutive rows per step (one 16-byte load per column), in row
            // order; the rows before the first multiple of 4 and after the last go one by one
            long long a = (r0 + 3) & ~3LL;
            if (a > r1) a = r1;
            const long long b = a + ((r1 - a) & ~3LL);
            for (long long r = r0 + threadIdx.x; r < a; r += T) rf_row(P, r, acc);
#pragma unroll 2
            for (long long r = a + 4 * (long long)threadIdx.x; r < b; r += 4LL * T) rf_row4(P, r, acc);
            for (long long r = b + threadIdx.x; r < r1; r += T) rf_row(P, r, acc);
            continue;
        }
#endif
#pragma unroll 4
        for (long long r = r0 + threadIdx.x; r < r1; r += T) rf_row(P, r, acc);
    }
}

template <int T>
RF_DEV void rf_scan_reduce_merge(const RfParams& P, int unit, int nunits, RfAcc& acc)
{
    __shared__ RfAcc warp_acc[T / 32];
    __shared__ int last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        RfAcc o = rf_acc_shfl(acc, off);
        rf_acc_combine(acc, o);
    }
    if (lane == 0) warp_acc[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        RfAcc tot = warp_acc[0];
        for (int w = 1; w < T / 32; w++) rf_acc_combine(tot, warp_acc[w]);
        rf_st_words((RfAcc*)P.partials + unit, &tot, (int)sizeof(RfAcc));
        __threadfence();
        unsigned int ticket = atomicAdd(P.counter, 1u);
        last = (ticket == (unsigned int)nunits - 1u);
    }
    __syncthreads();
    if (last) {
        __threadfence();
        // the whole block folds the units' partials: thread t takes units t, t+T, t+2T, ... in
        // that order (their loads issued RF_FOLD_ACC at a time ahead of the combines), then the
        // lanes of each warp by shuffles and the warps in order - a fixed order on every path
        RfAcc tot;
        rf_acc_init(P, tot);
        int u = threadIdx.x;
        for (; u + T * (RF_FOLD_ACC - 1) < nunits; u += T * RF_FOLD_ACC) {
            RfAcc v[RF_FOLD_ACC];
#pragma unroll
            for (int k = 0; k < RF_FOLD_ACC; k++)
                rf_ld_words(&v[k], (const RfAcc*)P.partials + u + T * k, (int)sizeof(RfAcc));
#pragma unroll
            for (int k = 0; k < RF_FOLD_ACC; k++) rf_acc_combine(tot, v[k]);
        }
        for (; u < nunits; u += T) {
            RfAcc p;
            rf_ld_words(&p, (const RfAcc*)P.partials + u, (int)sizeof(RfAcc));
            rf_acc_combine(tot, p);
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            RfAcc o = rf_acc_shfl(tot, off);
            rf_acc_combine(tot, o);
        }
        if (lane == 0) warp_acc[warp] = tot;
        __syncthreads();
        if (threadIdx.x == 0) {
            RfAcc all = warp_acc[0];
            for (int w = 1; w < T / 32; w++) rf_acc_combine(all, warp_acc[w]);
            rf_finish(P, all, P.out);
            *P.counter = 0u;
        }
    }
    __syncthreads();  // shared state is reused by the next work item of a persistent block
}

// Batched form: one persistent launch runs the work units of many queries of this shape.
// work[w] = {query, unit}; params[query] is the query's parameter block.  A query's units are
// the ones its stand-alone launch would run, folded in the same order: same bits either way.
#define RF_SCAN_REDUCE_KERNEL(NAME, T)                                                      \
    extern "C" __global__ void __launch_bounds__(T) NAME(const __grid_constant__ RfParams P) \
    {                                                                                       \
        RfAcc acc;                                                                          \
        rf_acc_init(P, acc);                                                                \
        rf_scan_reduce_rows<T>(P, P.unit0 + (int)blockIdx.x, P.nunits, acc);                \
        rf_scan_reduce_merge<T>(P, P.unit0 + (int)blockIdx.x, P.nunits, acc);               \
    }                                                                                       \
    extern "C" __global__ void __launch_bounds__(T)                                         \
        rf_batch(const RfParams* __restrict__ params, const int2* __restrict__ work, const int* nwork) \
    {                                                                                       \
        const int n = *nwork;                                                               \
        for (int w = blockIdx.x; w < n; w += gridDim.x) {                                   \
            const int2 it = work[w];                                                        \
            const RfParams& Q = params[it.x];                                               \
            if (it.y < 0 || it.y >= Q.nunits) { /* a malformed work item: report, skip */  \
                if (threadIdx.x == 0) atomicExch(Q.err, RF_DEVERR_RANGE);                    \
                continue;                                                                   \
            }                                                                               \
            RfAcc acc;                                                                      \
            rf_acc_init(Q, acc);                                                            \
            rf_scan_reduce_rows<T>(Q, it.y, Q.nunits, acc);                                 \
            rf_scan_reduce_merge<T>(Q, it.y, Q.nunits, acc);                                \
        }                                                                                   \
    }
#endif  // RF_SCAN_REDUCE

// ---------------------------------------------------------------------------------------
// Template 2: grouped scan-reduce with shared-memory privatised accumulators.
//   The fragment defines RF_G groups x RF_M aggregates, struct RfVals, rf_group(P, r, V)
//   (group id or -1, and the row's aggregate inputs), rf_slot_init(m) (64-bit identity),
//   rf_slot_combine(m, a, b), rf_slot_add(S, g, t, V, df), rf_slots_done(S, t, df) (df: the
//   thread keeps its FP64 sums as double-floats, see rf_device.cuh) and
//   rf_finish_groups(P, tot, out).  With RF_GROUP_SPLIT it also defines the row's loads apart,
//   struct RfRowLd, rf_group_ld(P, r, L) and rf_group_v(P, r, L, V) (rf_group is the two in turn).
// Each thread owns a private column of G*M 64-bit slots in shared memory (slot (q, t) at
// S[q * T + t]): no atomics and no bank conflicts on the per-row update.  At the end every
// slot column is folded over the block in a fixed order, then over units by the last unit.
// ---------------------------------------------------------------------------------------
#ifdef RF_GROUP_REDUCE
template <int T>
RF_DEV void rf_group_reduce(const RfParams& P, int unit, int nunits)
{
    extern __shared__ unsigned long long S[];
    __shared__ int last;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int Q = RF_G * RF_M;
    for (int q = 0; q < Q; q++) S[q * T + tid] = rf_slot_init(P, q % RF_M);
    bool df = true;  // the thread's FP64 sum slots hold double-floats (rf_slot_add, rf_slots_done)
    long long lo = P.row_lo, hi = P.row_hi;
    if (P.range) {
        long long b = P.range[0], e = P.range[1];
        lo = b > lo ? b : lo;
        hi = e < hi ? e : hi;
    }
    const long long tr = P.tile_rows;
    const long long ntiles = (P.row_hi - P.row_lo + tr - 1) / tr;
#ifdef RF_COMPACT
    // per-warp queue (64 rows) behind the slots: rows passing the cheap prefix of the condition
    long long* q = (long long*)(S + (size_t)Q * T) + (size_t)warp * 64;
#endif
    const long long t_end = (long long)(unit + 1) * ntiles / nunits;
    for (long long tile = (long long)unit * ntiles / nunits; tile < t_end; tile++) {
        long long r0 = P.row_lo + tile * tr, r1 = r0 + tr;
        if (r1 > hi) r1 = hi;
        if (r0 < lo) r0 = lo;
#ifdef RF_PREFETCH
        // the next tile's rows of the row's columns into L2 while this one is read
        if (tid == 0 && tile + 1 < t_end) {
            const long long n0 = P.row_lo + (tile + 1) * tr;
            long long n1 = n0 + tr;
            if (n1 > hi) n1 = hi;
            rf_prefetch_rows(P, n0, n1);
        }
#endif
#ifdef RF_COMPACT
        // warp-uniform steps of 8 chunks of 32 rows: the cheap tests of all 8 are issued together
        constexpr int U = 8;
        int qn = 0;
        for (long long b = r0 + 32 * U * warp; b < r1; b += (long long)T * U) {
            bool c[U];
#pragma unroll
            for (int j = 0; j < U; j++) {
                const long long r = b + 32 * j + lane;
                c[j] = r < r1 && rf_cheap(P, r);
            }
#pragma unroll
            for (int j = 0; j < U; j++) {
                const unsigned m = __ballot_sync(0xffffffffu, c[j]);
                if (c[j]) q[qn + __popc(m & ((1u << lane) - 1u))] = b + 32 * j + lane;
                qn += __popc(m);
                __syncwarp();
                if (qn >= 32) {
                    RfVals V;
                    const int g = rf_group(P, q[lane], V);
                    if (g >= 0) rf_slot_add(S, g, tid, V, df);
                    __syncwarp();
                    if (lane < qn - 32) q[lane] = q[32 + lane];
                    __syncwarp();
                    qn -= 32;
                }
            }
        }
        if (lane < qn) {
            RfVals V;
            const int g = rf_group(P, q[lane], V);
            if (g >= 0) rf_slot_add(S, g, tid, V, df);
        }
        __syncwarp();
#else
#if defined(RF_GROUP_ROWS) && defined(RF_GROUP_SPLIT)
        // RF_GROUP_ROWS rows a thread per iteration: all their loads (rf_group_ld) issued before
        // any row is evaluated (rf_group_v), so a warp has that many rows' loads in flight
#pragma unroll 1
        for (long long r = r0 + tid; r < r1; r += (long long)RF_GROUP_ROWS * T) {
            RfRowLd L[RF_GROUP_ROWS];
#pragma unroll
            for (int k = 0; k < RF_GROUP_ROWS; k++)
                if (r + (long long)k * T < r1) rf_group_ld(P, r + (long long)k * T, L[k]);
#pragma unroll
            for (int k = 0; k < RF_GROUP_ROWS; k++) {
                if (r + (long long)k * T >= r1) break;
                RfVals V;
                const int g = rf_group_v(P, r + (long long)k * T, L[k], V);
                if (g >= 0) rf_slot_add(S, g, tid, V, df);
            }
        }
#else
        // RF_GROUP_UNROLL 1 (a fragment with double-float sums): one row per iteration - the slot
        // update is long, and unrolled rows (whose loads the compiler does not move above the
        // previous row's branches) cost registers the row's own latencies need (the 6-group
        // group-by, its value loads after its filter: 0.775 ms against 0.789 / 0.800 ms unrolled
        // 2 / 4)
#if defined(RF_GROUP_UNROLL) && RF_GROUP_UNROLL == 1
#pragma unroll 1
#else
#pragma unroll 4
#endif
        for (long long r = r0 + tid; r < r1; r += T) {
            RfVals V;
            int g = rf_group(P, r, V);
            if (g >= 0) rf_slot_add(S, g, tid, V, df);
        }
#endif
#endif
    }
    rf_slots_done(S, tid, df);
    __syncthreads();
    unsigned long long* part = (unsigned long long*)P.partials;
    for (int q = warp; q < Q; q += T / 32) {
        const int m = q % RF_M;
        unsigned long long a = S[q * T + lane];
        for (int k = 1; k < T / 32; k++) a = rf_slot_combine(m, a, S[q * T + lane + 32 * k]);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) a = rf_slot_combine(m, a, __shfl_down_sync(0xffffffffu, a, off));
        if (lane == 0) __stcg(part + (long long)unit * Q + q, a);
    }
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        unsigned int ticket = atomicAdd(P.counter, 1u);
        last = (ticket == (unsigned int)nunits - 1u);
    }
    __syncthreads();
    if (last) {
        __threadfence();
        for (int q = warp; q < Q; q += T / 32) {
            const int m = q % RF_M;
            // units lane, lane+32, ... folded in that order; their loads are issued RF_FOLD at a
            // time ahead of the combines
            unsigned long long a = rf_slot_init(P, m);
            int u = lane;
            for (; u + 32 * (RF_FOLD - 1) < nunits; u += 32 * RF_FOLD) {
                unsigned long long v[RF_FOLD];
#pragma unroll
                for (int k = 0; k < RF_FOLD; k++) v[k] = __ldcg(part + (long long)(u + 32 * k) * Q + q);
#pragma unroll
                for (int k = 0; k < RF_FOLD; k++) a = rf_slot_combine(m, a, v[k]);
            }
            for (; u < nunits; u += 32) a = rf_slot_combine(m, a, __ldcg(part + (long long)u * Q + q));
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) a = rf_slot_combine(m, a, __shfl_down_sync(0xffffffffu, a, off));
            if (lane == 0) S[q] = a;
        }
        __syncthreads();
        if (tid == 0) {
            rf_finish_groups(P, S, P.out);
            *P.counter = 0u;
        }
    }
    __syncthreads();  // shared state is reused by the next work item of a persistent block
}

// RF_MINB (set by the fragment): the blocks per SM the registers must allow; unset, the bound
// names the block size alone (a minimum of 1 block measured slower for the join's probe kernel:
// 1.11 -> 1.39 ms, as the compiler then takes registers freely)
#ifdef RF_MINB
#define RF_GROUP_BOUNDS(T) __launch_bounds__(T, RF_MINB)
#else
#define RF_GROUP_BOUNDS(T) __launch_bounds__(T)
#endif
#define RF_GROUP_REDUCE_KERNEL(NAME, T)                                                     \
    extern "C" __global__ void RF_GROUP_BOUNDS(T) NAME(const __grid_constant__ RfParams P) \
    {                                                                                       \
        rf_group_reduce<T>(P, P.unit0 + (int)blockIdx.x, P.nunits);                         \
    }                                                                                       \
    extern "C" __global__ void RF_GROUP_BOUNDS(T)                                           \
        rf_batch(const RfParams* __restrict__ params, const int2* __restrict__ work, const int* nwork) \
    {                                                                                       \
        const int n = *nwork;                                                               \
        for (int w = blockIdx.x; w < n; w += gridDim.x) {                                   \
            const int2 it = work[w];                                                        \
            if (it.y < 0 || it.y >= params[it.x].nunits) { /* malformed work item */       \
                if (threadIdx.x == 0) atomicExch(params[it.x].err, RF_DEVERR_RANGE);         \
                continue;                                                                   \
            }                                                                               \
            rf_group_reduce<T>(params[it.x], it.y, params[it.x].nunits);                    \
        }                                                                                   \
    }
#endif  // RF_GROUP_REDUCE


// ---------------------------------------------------------------------------------------
// Template 3: Op materialisation (LoopGen::visit(Op), loopgen.cpp:113-204, and
// finalize_vector, vinstr.h:113-135).
//   The fragment defines rf_cond(P, r) (the iteration condition of element r) and
//   rf_emit(P, r, o) (computes the element's iterators and outputs, writes them at output row o).
//   Output columns: ((void**)P.aux0)[c]; validity words: ((unsigned**)P.aux1)[c];
//   per-tile counts / offsets: (long long*)P.aux2; results (long long*)P.aux3:
//   [0] = rows written, [1] = null count.
//   Compaction (vectorize off) keeps passing elements in loop order: count per tile, one
//   exclusive scan over tiles, then a scatter that ranks elements inside each tile with warp
//   ballots.  Vectorised (on): every visited element is written; its condition becomes the
//   validity bit.
// ---------------------------------------------------------------------------------------
#ifdef RF_MATERIALIZE
RF_DEV void rf_mat_bounds(const RfParams& P, long long& lo, long long& hi)
{
    lo = P.row_lo;
    hi = P.row_hi;
    if (P.range) {
        long long b = P.range[0], e = P.range[1];
        lo = b > lo ? b : lo;
        hi = e < hi ? e : hi;
    }
}

RF_DEV long long rf_mat_ntiles(const RfParams& P)
{
    return (P.row_hi - P.row_lo + P.tile_rows - 1) / P.tile_rows;
}

template <int T>
RF_DEV int rf_block_sum_int(int v, int* sh)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = __reduce_add_sync(0xffffffffu, v);
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    int t = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < T / 32; w++) t += sh[w];
    __syncthreads();
    return t;
}

template <int T>
RF_DEV void rf_mat_count(const RfParams& P)
{
    __shared__ int sh[T / 32];
    long long lo, hi;
    rf_mat_bounds(P, lo, hi);
    long long* cnt = (long long*)P.aux2;
    const long long nt = rf_mat_ntiles(P);
    for (long long tile = blockIdx.x; tile < nt; tile += gridDim.x) {
        long long r0 = P.row_lo + tile * P.tile_rows, r1 = r0 + P.tile_rows;
        if (r1 > hi) r1 = hi;
        if (r0 < lo) r0 = lo;
        int c = 0;
        for (long long r = r0 + threadIdx.x; r < r1; r += T) c += rf_cond(P, r) ? 1 : 0;
        int t = rf_block_sum_int<T>(c, sh);
        if (threadIdx.x == 0) cnt[tile] = t;
    }
}

// exclusive scan of the tile counts in place (one block); total -> aux3[0]
RF_DEV void rf_mat_scan(const RfParams& P)
{
    __shared__ long long wsum[32];
    __shared__ long long carry;
    long long* cnt = (long long*)P.aux2;
    const long long nt = rf_mat_ntiles(P);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (long long base = 0; base < nt; base += blockDim.x) {
        long long i = base + threadIdx.x;
        long long v = i < nt ? cnt[i] : 0;
        long long x = v;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            long long y = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        if (warp == 0) {
            long long w = lane < nw ? wsum[lane] : 0;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                long long y = __shfl_up_sync(0xffffffffu, w, off);
                if (lane >= off) w += y;
            }
            if (lane < nw) wsum[lane] = w;
        }
        __syncthreads();
        long long excl = carry + (warp ? wsum[warp - 1] : 0) + x - v;
        if (i < nt) cnt[i] = excl;
        __syncthreads();
        if (threadIdx.x == 0) carry += wsum[nw - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) ((long long*)P.aux3)[0] = carry;
}

template <int T>
RF_DEV void rf_mat_scatter(const RfParams& P)
{
    __shared__ int wcnt[T / 32];
    __shared__ int woff[T / 32 + 1];
    long long lo, hi;
    rf_mat_bounds(P, lo, hi);
    const long long* off = (const long long*)P.aux2;
    const long long nt = rf_mat_ntiles(P);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (long long tile = blockIdx.x; tile < nt; tile += gridDim.x) {
        long long r0 = P.row_lo + tile * P.tile_rows, r1 = r0 + P.tile_rows;
        if (r1 > hi) r1 = hi;
        if (r0 < lo) r0 = lo;
        long long base = off[tile];
        for (long long c0 = r0; c0 < r1; c0 += T) {
            long long r = c0 + threadIdx.x;
            bool c = r < r1 && rf_cond(P, r);
            unsigned m = __ballot_sync(0xffffffffu, c);
            if (lane == 0) wcnt[warp] = __popc(m);
            __syncthreads();
            if (threadIdx.x == 0) {
                int s = 0;
                for (int w = 0; w < T / 32; w++) {
                    woff[w] = s;
                    s += wcnt[w];
                }
                woff[T / 32] = s;
            }
            __syncthreads();
            if (c) rf_emit(P, r, base + woff[warp] + __popc(m & ((1u << lane) - 1u)));
            base += woff[T / 32];
            __syncthreads();
        }
    }
}

template <int T>
RF_DEV void rf_mat_write_all(const RfParams& P, int ncols)
{
    long long lo, hi;
    rf_mat_bounds(P, lo, hi);
    const long long nt = rf_mat_ntiles(P);
    const int lane = threadIdx.x & 31;
    long long nulls = 0;
    for (long long tile = blockIdx.x; tile < nt; tile += gridDim.x) {
        long long r0 = P.row_lo + tile * P.tile_rows, r1 = r0 + P.tile_rows;
        if (r1 > hi) r1 = hi;
        if (r0 < lo) r0 = lo;
        for (long long c0 = r0; c0 < r1; c0 += T) {
            long long r = c0 + threadIdx.x;
            bool in = r < r1;
            bool c = in && rf_cond(P, r);
            if (in) rf_emit(P, r, r - lo);
            unsigned m = __ballot_sync(0xffffffffu, c);
            unsigned act = __ballot_sync(0xffffffffu, in);
            nulls += (lane == 0) ? __popc(act & ~m) : 0;
            // lanes of a warp hold consecutive elements: their bits land in at most two words
            long long o0 = __shfl_sync(0xffffffffu, r - lo, 0);
            if (lane == 0 && act) {
                long long w = o0 >> 5;
                int sft = (int)(o0 & 31);
                for (int col = 0; col < ncols; col++) {
                    unsigned* bm = ((unsigned**)P.aux1)[col];
                    atomicOr(bm + w, m << sft);
                    if (sft && (m >> (32 - sft))) atomicOr(bm + w + 1, m >> (32 - sft));
                }
            }
        }
    }
    if (lane == 0 && nulls) atomicAdd((unsigned long long*)P.aux3 + 1, (unsigned long long)nulls);
}

#define RF_MATERIALIZE_KERNELS(T, NCOLS)                                                                  \
    extern "C" __global__ void __launch_bounds__(T) rf_count(const __grid_constant__ RfParams P)         \
    {                                                                                                    \
        rf_mat_count<T>(P);                                                                              \
    }                                                                                                    \
    extern "C" __global__ void __launch_bounds__(1024) rf_scan(const __grid_constant__ RfParams P)      \
    {                                                                                                    \
        rf_mat_scan(P);                                                                                  \
    }                                                                                                    \
    extern "C" __global__ void __launch_bounds__(T) rf_scatter(const __grid_constant__ RfParams P)       \
    {                                                                                                    \
        rf_mat_scatter<T>(P);                                                                            \
    }                                                                                                    \
    extern "C" __global__ void __launch_bounds__(T) rf_write_all(const __grid_constant__ RfParams P)     \
    {                                                                                                    \
        rf_mat_write_all<T>(P, NCOLS);                                                                   \
    }
#endif  // RF_MATERIALIZE
