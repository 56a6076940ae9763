// Lowering of a Reffine Func onto the GB300 kernel templates.
//
// This is the GPU counterpart of Reffine's LoopGen + CEmitter (src/pass/loopgen.cpp,
// src/pass/cemitter.cpp): instead of a serial loop, the Func's loop nest is matched to one of
// the kernel templates of device/rf_templates.cuh and the query's own expressions (predicate,
// projection, accumulator update, epilogue) are emitted as the template's device fragment.
// Shapes that match no template are rejected (no CPU fallback).
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "reffine_gb300/ir.h"

namespace rfg {

using reffine::DataType;
using reffine::Expr;
using reffine::Func;

enum class PlanKind {
    SCAN_REDUCE = 1,   // fused scan-filter-project-reduce, accumulators in registers
    GROUP_REDUCE = 2,  // the same, with key groups privatised in shared memory
    MATERIALIZE = 3,   // Op output: selection-vector compaction into a new table
    SEG_REDUCE = 4,    // Op over a run-end encoded 2-d vector with a nested Reduce per run
    HASH_GROUP = 5,    // the same query over an unsorted flat key column: hash group-by
    MERGE_JOIN = 6,    // Op over an intersection of vectors (merge co-iteration)
    UNION_MERGE = 7,   // Op over a union of two vectors (outer merge co-iteration)
};

struct LowerError : std::runtime_error {
    bool unsupported;
    LowerError(const std::string& m, bool u = true) : std::runtime_error(m), unsupported(u) {}
};

struct ConstSlot {
    bool is_float = false;
    double f = 0;
    long long i = 0;
};

// A host-side expression the runtime evaluates before launch (loop bounds of a SubVector,
// range bounds of a Universal iteration space): constants, table lengths, scalar inputs,
// + - * max min.
struct HostExpr {
    enum Kind { NONE, CONST, LEN, SCALAR, ADD, SUB, MUL, MAX, MIN } kind = NONE;
    long long value = 0;
    int input = -1, col = -1;
    std::vector<HostExpr> args;
};

struct KernelSpec {
    std::string name;
    int threads = 256;
    size_t smem = 0;
    enum Role { MAIN, RANGE, STOP, COUNT, SCAN, SCATTER, INIT, FINAL, SEGCOUNT, SEGSCAN, SEGREDUCE, IXCOUNT, IXINIT,
                IXBUILD } role = MAIN;
};

struct Plan {
    PlanKind kind = PlanKind::SCAN_REDUCE;
    std::string source;                 // CUDA source of the query's kernels
    std::string key;                    // source hash: queries equal up to constants share it
    std::vector<KernelSpec> kernels;
    int n_inputs = 0;
    std::vector<DataType> input_types;
    std::vector<int> table_slot;        // per Func input: RfParams.t slot, or -1
    std::vector<int> scalar_slot;       // per Func input: RfParams.s slot, or -1
    std::vector<std::vector<int>> cols_read;  // per Func input: columns the query reads
    std::vector<int> needs_index;       // per Func input: 1 if the query probes its index
    std::vector<int> random_read;       // per Func input: 1 if rows are read at computed positions
                                        // (ReadData, Locate), not only at the loop's own row
    std::vector<ConstSlot> consts;
    // driving loop
    HostExpr row_lo, row_hi;            // tiling range (host-known)
    bool device_range = false;          // begin/end refined on the device (range kernels)
    int drive_input = -1;               // Func input whose rows drive the loop (-1: a range)
    long long tile_rows = 8192;
    int threads = 256;
    // results
    DataType out_type;
    size_t out_size = 0;                // bytes of the value output (C layout)
    bool out_is_table = false;
    size_t acc_bytes = 0;               // bytes of one unit's partial (scan-reduce, segmented reduce)
    int seg_chunk = 256;                // segmented reduce: rows per chunk
    int ixf_input = -1;                 // input whose index a run replaces by a filtered one (-1: none)
    int union_inputs[2] = {-1, -1};     // union merge: the two merged vectors (Func inputs)
    int hg_hot = 0;                     // hash group-by: hottest keys folded per warp (index 2x)
    int hg_warm = 0;                    // hash group-by: further hot keys in shared memory (index 2x)
    int groups = 0, aggs = 0;           // grouped plans
    std::vector<DataType> out_cols;     // table outputs: column types
    int out_dim = 0;
    bool vectorize = false;
};

// `threads`: the block size of the scan templates' kernels (128, 256 or 512; the autotuner
// chooses it per query shape)
Plan lower(const std::shared_ptr<Func>& fn, bool vectorize, int threads = 256);

// hash group-by: slots of the shared-memory hot-key table per hot key (a power of two)
constexpr int kHotSlotsPerKey = 16;

// byte size and alignment of a value type in the C layout the reference's emitted structs use
size_t c_size(const DataType& t);
size_t c_align(const DataType& t);

}  // namespace rfg
