// Host launchers of the ahead-of-time kernels in kernels.cu.
#pragma once

#include <cuda_runtime_api.h>

#ifdef __cplusplus
extern "C" {
#endif

// Builds the device hash index of an int64 key column (2 launches); *dup (if not NULL) ends 1
// when a key occurs more than once.  Returns a cudaError_t.
int rf_k_index_build(const void* keys, const unsigned short* valid, long long n, long long* slots,
                     unsigned long long cap, long long* special, int* err, int* dup, cudaStream_t stream);

// Exclusive prefix sum of n int64 values in place (3 launches); data must hold n+1 entries, the
// last receives the total.  tmp must hold ceil(n / 2048) + 1 entries.
int rf_k_scan_excl(long long* data, long long n, long long* tmp, cudaStream_t stream);

// HyperLogLog registers (2^14 unsigned, device) of an int64 column (2 launches).
#define RF_HLL_M 16384
int rf_k_hll(const void* keys, const unsigned short* valid, long long n, unsigned* regs, cudaStream_t stream);

// m keys of an int64 column sampled at rows i * n / m (null keys as RF_EMPTY_KEY), 1 launch.
int rf_k_sample_keys(const void* keys, const unsigned short* valid, long long n, long long m, long long* out,
                     cudaStream_t stream);

// Device address (with the calling thread's current device = `device`) and size of the fixed
// scratch array of rf_plan_run_noalloc.  The address is looked up once per device.
int rf_k_noalloc_scratch(int device, void** ptr, size_t* bytes);

#ifdef __cplusplus
}
#endif
