// Batched execution: many queries in one persistent launch (rf_batch_*).
#include "rf_gpu.h"

struct rf_batch {
    rf_ctx* ctx;
};

extern "C" int rf_batch_create(rf_ctx* ctx, int32_t capacity, rf_batch** out)
{
    (void)ctx;
    (void)capacity;
    if (out) *out = nullptr;
    return RF_ERR_UNSUPPORTED;
}
extern "C" int rf_batch_free(rf_batch* b)
{
    delete b;
    return RF_OK;
}
extern "C" int rf_batch_add(rf_batch*, rf_plan*, const rf_arg*, int32_t, void*) { return RF_ERR_UNSUPPORTED; }
extern "C" int rf_batch_launch(rf_batch*, void*) { return RF_ERR_UNSUPPORTED; }
extern "C" int rf_batch_wait(rf_batch*) { return RF_ERR_UNSUPPORTED; }
extern "C" int rf_batch_reset(rf_batch*) { return RF_ERR_UNSUPPORTED; }
