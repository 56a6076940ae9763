// Runtime interface for the C++ that Reffine's compile path emits (oracle/ref/generated/*.cpp),
// so that code runs without a Reffine checkout.  It declares the functions that code calls, with
// the names, arguments and meanings of Reffine's include/reffine/vinstr/vinstr.h (cited per
// function); the bodies and the table type are this runtime's own.  Benchmark and test
// infrastructure only: the CPU reference arm and the oracle's tests use it.
#ifndef ORACLE_REF_RUNTIME_VINSTR_H_
#define ORACLE_REF_RUNTIME_VINSTR_H_

#include <cstdint>
#include <unordered_map>

#include "reffine_gb300/arrow_c.h"

// a table as the emitted code sees it: a struct array ("+s") of columns, and for Locate the hash
// index of column 0 (Reffine keeps a std::unordered_map there, include/reffine/arrow/table.h:13)
struct ArrowTable {
    int64_t dim;
    ArrowSchema* schema;
    ArrowArray* array;
    std::unordered_map<int64_t, int64_t>* index;
};

extern "C" {

// vinstr.h:15-23: the end of run `idx` of an int32 run-end buffer; 0 before the first run
inline int64_t read_runend_buf(void* buf, int64_t idx)
{
    return idx < 0 ? 0 : (int64_t)((const int32_t*)buf)[idx];
}

// vinstr.h:25-41: the struct array, a child, a buffer, a length
inline ArrowArray* get_vector_array(ArrowTable* tbl) { return tbl->array; }
inline ArrowArray* get_array_child(ArrowArray* arr, uint32_t col) { return arr->children[col]; }
inline void* get_array_buf(ArrowArray* arr, uint32_t buf) { return (void*)arr->buffers[buf]; }
inline int64_t get_array_len(ArrowArray* arr) { return arr->length; }

// vinstr.h:70-74: validity bit `idx` of a bitmap read as 16-bit words; no bitmap means valid
inline bool get_null_bit(uint16_t* bitmap, int64_t idx)
{
    return !bitmap || ((bitmap[idx >> 4] >> (idx & 15)) & 1u);
}

// vinstr.h:137-146: the row of key `val` in column 0's index, -1 when absent
inline int64_t vector_locate(ArrowTable* tbl, int64_t val)
{
    auto it = tbl->index->find(val);
    return it == tbl->index->end() ? -1 : it->second;
}

// vinstr.h:113-135: sets an output's length and null counts; writes the validity bitmaps from
// the per-row bytemap when any row is null, else drops them (defined in ref_runner.cpp)
void finalize_vector(ArrowTable* tbl, bool* bytemap, int64_t len, int64_t null_count);

// vinstr.h:151-153 (src/vinstr/external.cpp): a new output table of `len` rows of the column
// types registered for `mem_id`; Locate's index of column 0 (defined in ref_runner.cpp)
ArrowTable* make_vector(int64_t len, uint32_t mem_id);
ArrowTable* build_vector_index(ArrowTable* tbl);

}  // extern "C"

#endif  // ORACLE_REF_RUNTIME_VINSTR_H_
