// Internal interface between the runtime's translation units.
#pragma once

#include <cuda_runtime_api.h>

#include <functional>
#include <vector>

#include "device/rf_params.h"
#include "rf_gpu.h"

namespace rfrt {

// enqueues the kernels of one plan run on stream `s` (no synchronisation)
int enqueue(rf_plan* p, const rf_arg* args, int n_args, cudaStream_t s, RfParams* P);
// fills the parameter block of a plan run; lo/hi = tiling range
int fill_params(rf_plan* p, const rf_arg* args, int n_args, RfParams& P, long long& lo, long long& hi,
                bool may_allocate);
// one host-to-device copy that upload() leaves to its caller (see `defer`)
struct HostCopy {
    void* dst;
    const void* src;
    size_t bytes;
    int width;  // > 0: a flat column's values, `width` bytes per row; -1: its validity bitmap;
                // 0: not addressable by row (run ends, run values)
};
// copies the columns of Arrow C data into a device table; with `defer`, the device buffers are
// allocated but the copies are appended to *defer instead of being issued
int upload(rf_ctx* ctx, const struct ArrowSchema* schema, const struct ArrowArray* array, int64_t dim,
           const int32_t* sel, int32_t nsel, void* stream, rf_table** out, rf_table* reuse,
           std::vector<HostCopy>* defer = nullptr);
// Issues `copies` through the context's pinned staging ring: host threads fill(dst_pinned, src,
// bytes) chunks into one half of the ring while the other half's DMA runs.  Returns after the
// last copy is enqueued on `s` and every staging slot it used is free again.
int staged_h2d(rf_ctx* ctx, const std::vector<HostCopy>& copies,
               const std::function<bool(void*, const void*, size_t)>& fill, cudaStream_t s);
int build_index(rf_table* t, cudaStream_t s);
// whether a value-result plan can run while its driving table is still arriving: one main
// kernel of a scan or grouped reduce, reading the driving table only at the loop's own rows
bool streamable(rf_plan* p);
// runs such a plan with the driving input's columns copied from host memory in row chunks on
// the context's copy stream; each chunk's units launch as soon as their rows have landed.
// `drive` = the driving input's copies as upload(..., defer) listed them.  Same units, same
// fold order as rf_plan_run: same bits.
int run_streamed(rf_plan* p, const rf_arg* args, int n_args, const std::vector<HostCopy>& drive, void* out);
void thunk_release(rf_plan* p);

}  // namespace rfrt
