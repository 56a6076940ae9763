// Query-independent device kernels, compiled ahead of time with nvcc for sm_103a.
//
//   rf_index_*   the device hash index of a table's iterator column: the GPU form of
//                ArrowTable2::build_index (include/reffine/arrow/table.h:107-138), an
//                std::unordered_map<int64, row> built serially there.  Here: open addressing,
//                linear probing, load factor 0.5, {key, row} slots of 16 bytes (one load per
//                probe); the lowest row of a duplicated key wins (emplace keeps the first).
#include <cuda_runtime.h>

#include "device/rf_device.cuh"
#include "kernels.h"

namespace {

__global__ void index_init_kernel(long long* slots, unsigned long long cap, long long* special, int* dup)
{
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (; i < cap; i += stride) {
        longlong2 v;
        v.x = RF_EMPTY_KEY;
        v.y = RF_INT64_MAX;
        reinterpret_cast<longlong2*>(slots)[i] = v;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *special = RF_INT64_MAX;
        if (dup) *dup = 0;
    }
}

// keys: int64 column 0 (run values for a run-end column), n entries, validity bitmap or NULL
__global__ void index_build_kernel(const long long* __restrict__ keys, const unsigned short* __restrict__ valid,
                                   long long n, long long* slots, unsigned long long cap, long long* special,
                                   int* err, int* dup)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += stride) {
        if (!rf_valid(valid, i)) continue;
        long long k = __ldg(keys + i);
        if (k == RF_EMPTY_KEY) {
            if (atomicMin(special, i) != RF_INT64_MAX && dup) *dup = 1;
            continue;
        }
        unsigned long long h = rf_home(k, cap);
        bool done = false;
        // bounded: at most `cap` probes (the table is half empty, so a few in practice)
        for (unsigned long long p = 0; p < cap; ++p) {
            unsigned long long* kp = reinterpret_cast<unsigned long long*>(slots + 2 * h);
            // read first: duplicated keys find their slot without an atomic on the key word
            unsigned long long old = __ldcg(kp);
            if (old == (unsigned long long)RF_EMPTY_KEY)
                old = atomicCAS(kp, (unsigned long long)RF_EMPTY_KEY, (unsigned long long)k);
            if (old == (unsigned long long)RF_EMPTY_KEY || old == (unsigned long long)k) {
                if (old == (unsigned long long)k && dup) *dup = 1;  // a repeated key
                if (__ldcg(slots + 2 * h + 1) > i) atomicMin(slots + 2 * h + 1, i);
                done = true;
                break;
            }
            if (++h == cap) h = 0;
        }
        if (!done && err) atomicCAS(err, 0, RF_DEVERR_PROBE);
    }
}

int grid_for(long long n, int threads)
{
    long long b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > 152 * 16) b = 152 * 16;
    return (int)b;
}

}  // namespace

extern "C" int rf_k_index_build(const void* keys, const unsigned short* valid, long long n, long long* slots,
                                unsigned long long cap, long long* special, int* err, int* dup, cudaStream_t stream)
{
    index_init_kernel<<<grid_for((long long)cap, 256), 256, 0, stream>>>(slots, cap, special, dup);
    if (n > 0)
        index_build_kernel<<<grid_for(n, 256), 256, 0, stream>>>(static_cast<const long long*>(keys), valid, n, slots,
                                                                 cap, special, err, dup);
    return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// Exclusive prefix sum of n int64 values, in place; data[n] receives the total.
// Three launches: per-block sums, a one-block scan of those sums, per-block scans plus offset.
// ---------------------------------------------------------------------------------------
namespace {

constexpr int kScanT = 1024;
constexpr int kScanPer = 2 * kScanT;

__device__ long long block_incl_scan(long long x, long long* wsum)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        long long y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        long long w = wsum[lane];
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            long long y = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) w += y;
        }
        wsum[lane] = w;
    }
    __syncthreads();
    long long r = x + (warp ? wsum[warp - 1] : 0);
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kScanT) scan_sums_kernel(const long long* data, long long n, long long* sums)
{
    __shared__ long long wsum[32];
    long long base = (long long)blockIdx.x * kScanPer;
    long long a = base + 2 * threadIdx.x;
    long long v = (a < n ? data[a] : 0) + (a + 1 < n ? data[a + 1] : 0);
    long long s = block_incl_scan(v, wsum);
    if (threadIdx.x == kScanT - 1) sums[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kScanT) scan_top_kernel(long long* sums, long long nb)
{
    __shared__ long long wsum[32];
    __shared__ long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (long long b = 0; b < nb; b += kScanT) {
        long long i = b + threadIdx.x;
        long long v = i < nb ? sums[i] : 0;
        long long s = block_incl_scan(v, wsum);
        if (i < nb) sums[i] = carry + s - v;
        __syncthreads();
        if (threadIdx.x == kScanT - 1) carry += s;
        __syncthreads();
    }
    if (threadIdx.x == 0) sums[nb] = carry;
}

__global__ void __launch_bounds__(kScanT) scan_apply_kernel(long long* data, long long n, const long long* sums,
                                                            long long nb)
{
    __shared__ long long wsum[32];
    long long base = (long long)blockIdx.x * kScanPer;
    long long a = base + 2 * threadIdx.x;
    long long v0 = a < n ? data[a] : 0, v1 = a + 1 < n ? data[a + 1] : 0;
    long long s = block_incl_scan(v0 + v1, wsum);
    long long off = sums[blockIdx.x] + s - (v0 + v1);
    if (a < n) data[a] = off;
    if (a + 1 < n) data[a + 1] = off + v0;
    if (blockIdx.x == 0 && threadIdx.x == 0) data[n] = sums[nb];
}

}  // namespace

extern "C" int rf_k_scan_excl(long long* data, long long n, long long* tmp, cudaStream_t stream)
{
    long long nb = (n + kScanPer - 1) / kScanPer;
    if (nb < 1) nb = 1;
    scan_sums_kernel<<<(unsigned)nb, kScanT, 0, stream>>>(data, n, tmp);
    scan_top_kernel<<<1, kScanT, 0, stream>>>(tmp, nb);
    scan_apply_kernel<<<(unsigned)nb, kScanT, 0, stream>>>(data, n, tmp, nb);
    return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// Distinct-count sketch of an int64 column: HyperLogLog (Flajolet, Fusy, Gandouet, Meunier,
// 2007) with 2^14 registers, used to size hash tables.  Register j holds the largest rank
// (leading zeros + 1) of the hashed keys whose top 14 bits are j.  Registers are kept per block
// in shared memory (a register is only written when its value grows) and merged with atomicMax.
// ---------------------------------------------------------------------------------------
namespace {

constexpr int kHllBits = 14;
constexpr int kHllM = 1 << kHllBits;

__global__ void __launch_bounds__(512) hll_kernel(const long long* __restrict__ keys, const unsigned short* __restrict__ valid,
                                                  long long n, unsigned* regs)
{
    __shared__ unsigned r[kHllM];
    for (int i = threadIdx.x; i < kHllM; i += blockDim.x) r[i] = 0;
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        if (!rf_valid(valid, i)) continue;
        unsigned long long h = rf_mix64((unsigned long long)__ldg(keys + i));
        unsigned j = (unsigned)(h >> (64 - kHllBits));
        unsigned long long w = (h << kHllBits) | (1ULL << (kHllBits - 1));
        unsigned rank = (unsigned)__clzll((long long)w) + 1u;
        if (rank > r[j]) atomicMax(&r[j], rank);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kHllM; i += blockDim.x)
        if (r[i]) atomicMax(&regs[i], r[i]);
}

// the m sampled rows are i * n / m; a null key samples as RF_EMPTY_KEY
__global__ void __launch_bounds__(256) sample_kernel(const long long* __restrict__ keys, const unsigned short* __restrict__ valid,
                                                     long long n, long long m, long long* __restrict__ out)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x) {
        const long long r = i * n / m;
        out[i] = rf_valid(valid, r) ? __ldg(keys + r) : RF_EMPTY_KEY;
    }
}

}  // namespace

extern "C" int rf_k_sample_keys(const void* keys, const unsigned short* valid, long long n, long long m, long long* out,
                                cudaStream_t stream)
{
    if (m <= 0 || n <= 0) return 0;
    const int blocks = (int)std::min<long long>((m + 255) / 256, 1024);
    sample_kernel<<<blocks, 256, 0, stream>>>(static_cast<const long long*>(keys), valid, n, m, out);
    return (int)cudaGetLastError();
}

extern "C" int rf_k_hll(const void* keys, const unsigned short* valid, long long n, unsigned* regs, cudaStream_t stream)
{
    cudaMemsetAsync(regs, 0, sizeof(unsigned) * kHllM, stream);
    int blocks = grid_for(n, 512);
    if (blocks > 152 * 2) blocks = 152 * 2;
    hll_kernel<<<blocks, 512, 0, stream>>>(static_cast<const long long*>(keys), valid, n, regs);
    return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// Fixed scratch for rf_plan_run_noalloc: callers that may not allocate device memory on the
// query path run value-output plans with their partials, completion counter, loop bounds and
// result placed here.  The array exists on every device that loads this library, for the life
// of the process.  In host code `rf_noalloc_scratch` only names the variable; its device
// address comes from cudaGetSymbolAddress, looked up once per device with that device current.
// ---------------------------------------------------------------------------------------
#include <mutex>

#define RF_NOALLOC_SCRATCH_BYTES (4u << 20)
static __device__ __align__(256) unsigned char rf_noalloc_scratch[RF_NOALLOC_SCRATCH_BYTES];

extern "C" int rf_k_noalloc_scratch(int device, void** ptr, size_t* bytes)
{
    static std::mutex mu;
    static void* addr[256] = {};
    if (device < 0 || device >= 256) return (int)cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> g(mu);
    if (!addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, rf_noalloc_scratch);
        if (e != cudaSuccess) return (int)e;
        addr[device] = p;
    }
    *ptr = addr[device];
    *bytes = RF_NOALLOC_SCRATCH_BYTES;
    return 0;
}
