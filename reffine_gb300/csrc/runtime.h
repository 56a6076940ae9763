// Internal interface between the runtime's translation units.
#pragma once

#include <cuda_runtime_api.h>

#include "device/rf_params.h"
#include "rf_gpu.h"

namespace rfrt {

// enqueues the kernels of one plan run on stream `s` (no synchronisation)
int enqueue(rf_plan* p, const rf_arg* args, int n_args, cudaStream_t s, RfParams* P);
// fills the parameter block of a plan run; lo/hi = tiling range
int fill_params(rf_plan* p, const rf_arg* args, int n_args, RfParams& P, long long& lo, long long& hi,
                bool may_allocate);
int upload(rf_ctx* ctx, const struct ArrowSchema* schema, const struct ArrowArray* array, int64_t dim,
           const int32_t* sel, int32_t nsel, void* stream, rf_table** out, rf_table* reuse);
int build_index(rf_table* t, cudaStream_t s);
void thunk_release(rf_plan* p);

}  // namespace rfrt
