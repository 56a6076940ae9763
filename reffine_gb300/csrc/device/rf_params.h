// Kernel parameter block shared by the host runtime and every generated kernel.
//
// One RfParams is passed by value (as a __grid_constant__ kernel parameter) to a query's
// kernels; the batched persistent kernel reads the same struct from device memory, one per
// query.  Plain C layout: the host (g++) and the device (NVRTC / nvcc) must agree on it.
#pragma once

#define RF_MAX_TABLES 4
#define RF_MAX_COLS 24
#define RF_MAX_CONSTS 128
#define RF_MAX_SCALARS 16
#define RF_MAX_GROUPS 64

#ifdef __cplusplus
extern "C" {
#endif

// One column on the device: values (run values for a run-end column), Reffine's validity
// bitmap read as uint16 words (NULL = all valid), int32 run ends (run-end columns only) and
// the number of values (runs for a run-end column: what Length() returns, readwritepass.cpp:71-79).
typedef struct RfCol {
    const void* data;
    const unsigned short* valid;
    const int* run_ends;
    long long len;
} RfCol;

// Device hash index on a table's iterator column: `cap` slots of {int64 key, int64 row}.
// An empty slot holds key RF_EMPTY_KEY; rows whose key equals RF_EMPTY_KEY are recorded in
// *special (lowest row, or INT64_MAX when none).
typedef struct RfIndex {
    const long long* slots;
    unsigned long long cap;
    const long long* special;
    long long pad_;
} RfIndex;

typedef struct RfTab {
    RfCol col[RF_MAX_COLS];
    RfIndex ix;
    long long nrows;
    long long pad_;
} RfTab;

typedef union RfK {
    double f;
    long long i;
} RfK;

typedef struct RfParams {
    RfTab t[RF_MAX_TABLES];
    RfK k[RF_MAX_CONSTS];      // hoisted constants (so one module serves every constant choice)
    long long s[RF_MAX_SCALARS];  // scalar Func inputs (doubles bit-cast)
    long long row_lo, row_hi;  // tiling range of the driving loop (host-known upper bound)
    long long tile_rows;       // rows per tile (fixed per plan: results do not depend on the grid)
    long long* range;          // device-computed loop bounds [begin, end) or NULL
    void* partials;            // per-work-unit partial results
    unsigned int* counter;     // completion ticket of the last-unit-done merge
    unsigned char* out;        // value output (device) / table output descriptor
    int* err;                  // device error flag (bounded probes and waits report here)
    void* aux0;                // kernel-specific device buffers (hash tables, offsets, output columns)
    void* aux1;
    void* aux2;
    void* aux3;
    void* aux4;
    void* aux5;
    long long aux_n0, aux_n1;  // kernel-specific sizes
    int nunits;                // work units (virtual CTAs) of the reduction
    int flags;
    int unit0;                 // first unit of this launch (a launch runs units unit0 .. unit0+grid-1)
    int rsv_;
} RfParams;

#define RF_EMPTY_KEY ((long long)0x8000000000000000ULL)

// RfParams.flags
#define RF_FLAG_VEC4 1  // every column the driving loop reads is 16-byte aligned: 4-row vector loads

// device error codes written to *err
#define RF_DEVERR_PROBE 1      // a hash probe/insert visited every slot
#define RF_DEVERR_WAIT 2       // a bounded wait ran out
#define RF_DEVERR_RANGE 3      // loop bound lookup failed (lower-bound key absent)
#define RF_DEVERR_OVERFLOW 4   // output or hash table capacity exceeded

#ifdef __cplusplus
}
#endif
