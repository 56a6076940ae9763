// Binding of Reffine's own IR to the GPU backend, for programs built against Reffine's headers
// (include/reffine/...): the IR builder (src/builder, src/ir) stays as it is; only the compile
// call changes.
//
//   #include "reffine/builder/reffiner.h"
//   #include "reffine_gb300/ref_binding.h"
//   auto fn = reffine_gb300::compile_op<void (*)(int64_t*, ArrowTable*)>(op, vectorize);
//
// func_text(fn) prints a reffine::Func (include/reffine/ir/stmt.h:8-27) in the text form that
// rf_plan_compile reads: the same expression graph, node for node.  A Reduce's init and
// accumulator functions (include/reffine/ir/op.h:89-112) are applied once to fresh state and
// value symbols, as the reference's own passes apply them.
//
// compile_op<FnTy> replaces the reference's compile_op (include/reffine/utils/utils.h:47-54): it
// compiles the Func for the GPU and returns a host function of the same type FnTy, which takes
// host ArrowTable* inputs and writes *output_addr as the reference's generated function does.
// Errors are thrown as std::runtime_error (the reference's passes throw it too).
//
// This header cannot be included together with reffine_gb300/ir.h or reffine_gb300/utils.h:
// those re-declare the IR for programs that do not link Reffine.
#pragma once

#include <cstdlib>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>

#include "reffine/ir/stmt.h"
#include "rf_gpu.h"

namespace reffine_gb300 {

// the text form of `fn` (rf_plan_compile's input)
std::string func_text(const reffine::Func& fn);

// the process's backend context (device 0, or RF_DEVICE), created on first use
inline rf_ctx* default_ctx()
{
    static std::once_flag once;
    static rf_ctx* ctx = nullptr;
    static int status = 0;
    std::call_once(once, [] {
        const char* d = std::getenv("RF_DEVICE");
        status = rf_gpu_init(d ? std::atoi(d) : 0, &ctx);
    });
    if (status != RF_OK || !ctx) throw std::runtime_error("reffine_gb300: no usable GPU (rf_gpu_init failed)");
    return ctx;
}

template <typename FnTy>
FnTy compile_op(std::shared_ptr<reffine::Func> op, bool vectorize = false)
{
    rf_ctx* ctx = default_ctx();
    const std::string text = func_text(*op);
    rf_plan* plan = nullptr;
    if (rf_plan_compile(ctx, text.c_str(), vectorize ? 1 : 0, &plan) != RF_OK)
        throw std::runtime_error(std::string("reffine_gb300: compile failed: ") + rf_last_error(ctx));
    void* fn = nullptr;
    if (rf_plan_thunk(plan, &fn) != RF_OK)
        throw std::runtime_error(std::string("reffine_gb300: no query function: ") + rf_last_error(ctx));
    // like the reference's ExecEngine, the compiled query lives until the process exits
    return reinterpret_cast<FnTy>(fn);
}

}  // namespace reffine_gb300
