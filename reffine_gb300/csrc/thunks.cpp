// Host function pointers with the signature of Reffine's generated query functions.
//
// compile_op<FnTy> (include/reffine/utils/utils.h:47-54) returns the address of the JIT-compiled
// `extern "C" void name(OutT* output_addr, inputs...)` (src/pass/cemitter.cpp:227-252), where
// vector inputs are `ArrowTable*` and scalars are passed by value.  rf_plan_thunk returns a
// function with that calling shape that runs the plan on the GPU: existing callers keep their
// FnTy and change only the compile call.
//
// A plain function pointer carries no state, so a fixed pool of trampolines is compiled in;
// each is bound to one plan.  A trampoline is declared with eight pointer-sized and eight
// double parameters: under both the x86-64 SysV and the AArch64 procedure-call standards the
// caller's integer/pointer arguments land in the first integer registers and its floating-point
// arguments in the first FP registers, in order, independently of how they interleave, so any
// signature with at most eight of each reaches the trampoline intact.
#include <cuda_runtime_api.h>

#include <array>
#include <cstdio>
#include <map>
#include <memory>
#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

#include "lower.h"
#include "reffine_gb300/arrow_table.h"
#include "rf_gpu.h"
#include "runtime.h"

namespace {

constexpr int kThunks = 512;
rf_plan* g_plans[kThunks];
std::mutex g_mu;

// a host table handed back through output_addr; its Arrow structs own their buffers
struct HostTable : ArrowTable {
    ArrowSchema s{};
    ArrowArray a{};
    explicit HostTable(int64_t dim) : ArrowTable(dim) {}
    ~HostTable() override
    {
        if (a.release) a.release(&a);
        if (s.release) s.release(&s);
    }
};
// like Reffine's memman (src/engine/memory.cpp:11-16) the outputs stay alive with their plan
std::map<rf_plan*, std::vector<std::unique_ptr<HostTable>>> g_outputs;

void thunk_call(int slot, void* const* a, const double* d);

template <int I>
void trampoline(void* a0, void* a1, void* a2, void* a3, void* a4, void* a5, void* a6, void* a7, double d0, double d1,
                double d2, double d3, double d4, double d5, double d6, double d7)
{
    void* a[8] = {a0, a1, a2, a3, a4, a5, a6, a7};
    double d[8] = {d0, d1, d2, d3, d4, d5, d6, d7};
    thunk_call(I, a, d);
}

using TrampolineFn = void (*)(void*, void*, void*, void*, void*, void*, void*, void*, double, double, double, double,
                              double, double, double, double);

template <int... Is>
constexpr std::array<TrampolineFn, sizeof...(Is)> make_table(std::integer_sequence<int, Is...>)
{
    return {&trampoline<Is>...};
}

}  // namespace

namespace {
const auto g_table = make_table(std::make_integer_sequence<int, kThunks>{});
}

// plan internals needed here
extern "C" int rf_plan_info(rf_plan* plan, rf_plan_info_t* info);
namespace rfrt {
const rfg::Plan& plan_of(rf_plan* p);
rf_ctx* ctx_of(rf_plan* p);
std::vector<rf_table*>& staging_of(rf_plan* p);
}  // namespace rfrt

namespace {

void thunk_call(int slot, void* const* a, const double* d)
{
    rf_plan* p;
    {
        std::lock_guard<std::mutex> g(g_mu);
        p = g_plans[slot];
    }
    if (!p) {
        fprintf(stderr, "reffine_gb300: call through a released query function\n");
        return;
    }
    const rfg::Plan& pl = rfrt::plan_of(p);
    rf_ctx* ctx = rfrt::ctx_of(p);
    void* output_addr = a[0];
    int ai = 1, di = 0;
    std::vector<rf_arg> args(pl.n_inputs);
    int rc = RF_OK;
    // a plan that reads its driving table only row by row starts on the first rows while the
    // rest are still being copied
    const bool streamed = rfrt::streamable(p);
    std::vector<rfrt::HostCopy> drive;
    for (int i = 0; i < pl.n_inputs && rc == RF_OK; i++) {
        const auto& ty = pl.input_types[i];
        rf_arg& ar = args[i];
        memset(&ar, 0, sizeof ar);
        if (ty.is_vector()) {
            if (ai >= 8) {
                rc = RF_ERR_UNSUPPORTED;
                break;
            }
            auto* t = static_cast<ArrowTable*>(a[ai++]);
            std::vector<int32_t> cols(pl.cols_read[i].begin(), pl.cols_read[i].end());
            if (pl.needs_index[i]) cols.push_back(0);
            // the plan's staging table for this input is reused call after call: only the
            // host-to-device copies of the referenced columns remain per call
            rf_table*& st = rfrt::staging_of(p)[i];
            rf_table* dt = nullptr;
            rc = rfrt::upload(ctx, t->schema, t->array, t->dim, cols.data(), (int32_t)cols.size(), nullptr, &dt, st,
                              streamed && i == pl.drive_input ? &drive : nullptr);
            if (rc == RF_OK) st = dt;
            ar.kind = RF_ARG_TABLE;
            ar.table = dt;
        } else if (ty.is_float()) {
            if (di >= 8) {
                rc = RF_ERR_UNSUPPORTED;
                break;
            }
            ar.kind = RF_ARG_F64;
            if (ty.btype == reffine::FLOAT32) {
                float f;
                memcpy(&f, &d[di++], sizeof f);  // a float argument occupies the low bits of its register
                ar.f64 = f;
            } else {
                ar.f64 = d[di++];
            }
        } else {
            if (ai >= 8) {
                rc = RF_ERR_UNSUPPORTED;
                break;
            }
            long long v = (long long)(intptr_t)a[ai++];
            switch (ty.size()) {  // narrower integers: only the low bits of the register are defined
                case 1: v = ty.is_unsigned() ? (long long)(uint8_t)v : (long long)(int8_t)v; break;
                case 2: v = ty.is_unsigned() ? (long long)(uint16_t)v : (long long)(int16_t)v; break;
                case 4: v = ty.is_unsigned() ? (long long)(uint32_t)v : (long long)(int32_t)v; break;
                default: break;
            }
            if (ty.btype == reffine::BOOL) v = (uint8_t)v != 0;
            ar.kind = RF_ARG_I64;
            ar.i64 = v;
        }
    }
    if (rc == RF_OK) {
        if (pl.out_is_table) {
            // make_vector + finalize_vector hand back an ArrowTable* (loopgen.cpp:118-135, 196-199);
            // here the device result is exported to host Arrow memory owned by the plan
            rf_table* dt = nullptr;
            rc = rf_plan_run(p, args.data(), (int32_t)args.size(), &dt, nullptr);
            if (rc == RF_OK) {
                auto* h = new HostTable(pl.out_dim);
                rc = rf_table_export(dt, &h->s, &h->a);
                rf_table_free(dt);
                if (rc == RF_OK) {
                    h->schema = &h->s;
                    h->array = &h->a;
                    *(ArrowTable**)output_addr = h;
                    std::lock_guard<std::mutex> g(g_mu);
                    g_outputs[p].emplace_back(h);
                } else {
                    delete h;
                }
            }
        } else if (streamed) {
            rc = rfrt::run_streamed(p, args.data(), (int32_t)args.size(), drive, output_addr);
        } else {
            rc = rf_plan_run(p, args.data(), (int32_t)args.size(), output_addr, nullptr);
        }
    }
    if (rc != RF_OK) fprintf(stderr, "reffine_gb300: query failed (%d): %s\n", rc, rf_last_error(ctx));
}

}  // namespace

namespace rfrt {
void thunk_release(rf_plan* p)
{
    std::lock_guard<std::mutex> g(g_mu);
    for (int i = 0; i < kThunks; i++)
        if (g_plans[i] == p) g_plans[i] = nullptr;
    g_outputs.erase(p);
}
}  // namespace rfrt

extern "C" int rf_plan_thunk(rf_plan* p, void** fn)
{
    if (!p || !fn) return RF_ERR_INVALID;
    std::lock_guard<std::mutex> g(g_mu);
    for (int i = 0; i < kThunks; i++) {
        if (g_plans[i] == p) {
            *fn = (void*)g_table[i];
            return RF_OK;
        }
    }
    for (int i = 0; i < kThunks; i++) {
        if (!g_plans[i]) {
            g_plans[i] = p;
            *fn = (void*)g_table[i];
            return RF_OK;
        }
    }
    return RF_ERR_BUSY;
}
