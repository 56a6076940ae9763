// Device-side building blocks of every query kernel (GB300, sm_103a).
//
// A query's kernels are compiled at plan time: the lowering pass (lower.cpp) emits a short
// source that defines the query's fragment - its row function, accumulator type, group
// function and epilogue - and then instantiates one of the templates below.  This header is
// handed to NVRTC as an in-memory header; it includes nothing from the system.
//
// Row-access helpers restate Reffine's runtime helpers (include/reffine/vinstr/vinstr.h):
//   rf_valid   get_null_bit  (vinstr.h:70-74): bitmap read as uint16 words; NULL = all valid
//   rf_runend  read_runend_buf (vinstr.h:15-23): int32 run ends, 0 for index < 0
//   rf_locate  vector_locate (vinstr.h:137-146): hash-index probe, -1 on a miss
//   rf_rd      a Load of get_array_buf(...)[idx] (readwritepass.cpp:16-30), guarded: an index
//              outside the column reads 0 (the reference reads out of bounds there)
#pragma once

#ifdef __CUDACC_RTC__
typedef signed char int8_t;
typedef short int16_t;
typedef int int32_t;
typedef long long int64_t;
typedef unsigned char uint8_t;
typedef unsigned short uint16_t;
typedef unsigned int uint32_t;
typedef unsigned long long uint64_t;
#define RF_INT64_MAX 0x7fffffffffffffffLL
#else
#include <cstdint>
#define RF_INT64_MAX 0x7fffffffffffffffLL
#endif

#include "rf_params.h"

#define RF_DEV static __device__ __forceinline__

// ---------------------------------------------------------------------------------------
// column loads.  rf_ld reads a column at the scanned row: each value is read once by a query,
// so the load is marked streaming (evict first), and a scan does not push out of L2 the data
// that is read again - index slots and columns read at a located row (rf_rd), which keep the
// normal read-only path.
// ---------------------------------------------------------------------------------------
template <class T>
struct RfLd;
template <>
struct RfLd<bool> {
    RF_DEV bool ld(const void* p, long long i) { return __ldcs((const signed char*)p + i) != 0; }
    RF_DEV bool ldg(const void* p, long long i) { return __ldg((const signed char*)p + i) != 0; }
};
template <>
struct RfLd<int8_t> {
    RF_DEV int8_t ld(const void* p, long long i) { return __ldcs((const signed char*)p + i); }
    RF_DEV int8_t ldg(const void* p, long long i) { return __ldg((const signed char*)p + i); }
};
template <>
struct RfLd<uint8_t> {
    RF_DEV uint8_t ld(const void* p, long long i) { return __ldcs((const unsigned char*)p + i); }
    RF_DEV uint8_t ldg(const void* p, long long i) { return __ldg((const unsigned char*)p + i); }
};
template <>
struct RfLd<int16_t> {
    RF_DEV int16_t ld(const void* p, long long i) { return __ldcs((const short*)p + i); }
    RF_DEV int16_t ldg(const void* p, long long i) { return __ldg((const short*)p + i); }
};
template <>
struct RfLd<uint16_t> {
    RF_DEV uint16_t ld(const void* p, long long i) { return __ldcs((const unsigned short*)p + i); }
    RF_DEV uint16_t ldg(const void* p, long long i) { return __ldg((const unsigned short*)p + i); }
};
template <>
struct RfLd<int32_t> {
    RF_DEV int32_t ld(const void* p, long long i) { return __ldcs((const int*)p + i); }
    RF_DEV int32_t ldg(const void* p, long long i) { return __ldg((const int*)p + i); }
};
template <>
struct RfLd<uint32_t> {
    RF_DEV uint32_t ld(const void* p, long long i) { return __ldcs((const unsigned int*)p + i); }
    RF_DEV uint32_t ldg(const void* p, long long i) { return __ldg((const unsigned int*)p + i); }
};
template <>
struct RfLd<int64_t> {
    RF_DEV int64_t ld(const void* p, long long i) { return __ldcs((const long long*)p + i); }
    RF_DEV int64_t ldg(const void* p, long long i) { return __ldg((const long long*)p + i); }
};
template <>
struct RfLd<uint64_t> {
    RF_DEV uint64_t ld(const void* p, long long i) { return __ldcs((const unsigned long long*)p + i); }
    RF_DEV uint64_t ldg(const void* p, long long i) { return __ldg((const unsigned long long*)p + i); }
};
template <>
struct RfLd<float> {
    RF_DEV float ld(const void* p, long long i) { return __ldcs((const float*)p + i); }
    RF_DEV float ldg(const void* p, long long i) { return __ldg((const float*)p + i); }
};
template <>
struct RfLd<double> {
    RF_DEV double ld(const void* p, long long i) { return __ldcs((const double*)p + i); }
    RF_DEV double ldg(const void* p, long long i) { return __ldg((const double*)p + i); }
};

template <class T>
RF_DEV T rf_ld(const void* p, long long i)
{
    return RfLd<T>::ld(p, i);
}

// rows r..r+3 of a column (r a multiple of 4, the column 16-byte aligned) in one or two 16-byte
// streaming loads (4- and 8-byte types; 1- and 2-byte types take one 4- or 8-byte load)
template <class T>
RF_DEV void rf_ld4(const void* p, long long r, T* v)
{
    const T* b = (const T*)p + r;
    if constexpr (sizeof(T) == 8) {
        union {
            uint4 u[2];
            T t[4];
        } x;
        x.u[0] = __ldcs((const uint4*)b);
        x.u[1] = __ldcs((const uint4*)(b + 2));
        v[0] = x.t[0], v[1] = x.t[1], v[2] = x.t[2], v[3] = x.t[3];
    } else if constexpr (sizeof(T) == 4) {
        union {
            uint4 u;
            T t[4];
        } x;
        x.u = __ldcs((const uint4*)b);
        v[0] = x.t[0], v[1] = x.t[1], v[2] = x.t[2], v[3] = x.t[3];
    } else if constexpr (sizeof(T) == 2) {
        union {
            uint2 u;
            T t[4];
        } x;
        x.u = __ldcs((const uint2*)b);
        v[0] = x.t[0], v[1] = x.t[1], v[2] = x.t[2], v[3] = x.t[3];
    } else {
        union {
            unsigned int u;
            T t[4];
        } x;
        x.u = __ldcs((const unsigned int*)b);
        v[0] = x.t[0], v[1] = x.t[1], v[2] = x.t[2], v[3] = x.t[3];
    }
}

// guarded read of column `c` at row/run `i` (a located or computed position: cached path)
template <class T>
RF_DEV T rf_rd(const RfCol& c, long long i)
{
    return (i >= 0 && i < c.len) ? RfLd<T>::ldg(c.data, i) : T(0);
}

RF_DEV bool rf_valid(const unsigned short* bm, long long i)
{
    return !bm || ((__ldg(bm + (i >> 4)) >> (i & 15)) & 1u);
}

RF_DEV long long rf_runend(const RfCol& c, long long i)
{
    return i < 0 ? 0LL : (long long)__ldg(c.run_ends + i);
}

// std::max / std::min semantics (what the reference's emitted C++ calls)
template <class T>
RF_DEV T rf_max(T a, T b)
{
    return (a < b) ? b : a;
}
template <class T>
RF_DEV T rf_min(T a, T b)
{
    return (b < a) ? b : a;
}

// ---------------------------------------------------------------------------------------
// binary64 comparisons on the integer pipe.
// IEEE 754 orders finite values and infinities of one sign by their bit patterns read as
// unsigned integers (sign-magnitude encoding), so key(x) = bits for x >= +0 and
// -(bits without sign) for negative x is monotonic, and maps -0 and +0 to the same key.  A
// comparison involving a NaN is false (== false, != true), as in IEEE and in the reference's
// C++.  GB300 executes FP64 comparisons on its narrow FP64 pipe; these run on the integer ALUs.
// ---------------------------------------------------------------------------------------
RF_DEV bool rf_dnan(double x) { return (__double_as_longlong(x) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL; }
RF_DEV long long rf_dkey(double x)
{
    long long b = __double_as_longlong(x);
    return b >= 0 ? b : -(b & 0x7fffffffffffffffLL);
}
RF_DEV bool rf_dlt(double a, double b) { return !rf_dnan(a) && !rf_dnan(b) && rf_dkey(a) < rf_dkey(b); }
RF_DEV bool rf_dle(double a, double b) { return !rf_dnan(a) && !rf_dnan(b) && rf_dkey(a) <= rf_dkey(b); }
RF_DEV bool rf_dgt(double a, double b) { return !rf_dnan(a) && !rf_dnan(b) && rf_dkey(a) > rf_dkey(b); }
RF_DEV bool rf_dge(double a, double b) { return !rf_dnan(a) && !rf_dnan(b) && rf_dkey(a) >= rf_dkey(b); }
RF_DEV bool rf_deq(double a, double b) { return !rf_dnan(a) && !rf_dnan(b) && rf_dkey(a) == rf_dkey(b); }

// ---------------------------------------------------------------------------------------
// x * (1 - y) and x * (1 + y) as one fused multiply-add, fma(-x, y, x) and fma(x, y, x): one
// binary64 rounding of the exact product instead of two (1 -/+ y rounded, then the product), so
// the two forms differ by at most the rounding of 1 -/+ y, 2^-53 relative (1 -/+ y is exact where
// it cancels, for y within a factor 2 of -/+1).  That holds where neither form can overflow or
// become subnormal: |x| in [2^-500, 2^500) and |y| < 2^500, tested with one unsigned compare on
// each high word.  Outside that band (infinities and NaN included) the product is formed as
// written, in a called function that keeps the rare path out of the caller's code.
// ---------------------------------------------------------------------------------------
RF_DEV bool rf_fma_band(double x, double y)
{
    const unsigned hx = (unsigned)__double2hiint(x) & 0x7FFFFFFFu, hy = (unsigned)__double2hiint(y) & 0x7FFFFFFFu;
    return hx - (523u << 20) < (1000u << 20) && hy < (1523u << 20);
}
__device__ __noinline__ double rf_mul_1m_plain(double x, double y) { return x * (1.0 - y); }
__device__ __noinline__ double rf_mul_1p_plain(double x, double y) { return x * (1.0 + y); }
RF_DEV double rf_mul_1m(double x, double y) { return rf_fma_band(x, y) ? __fma_rn(-x, y, x) : rf_mul_1m_plain(x, y); }
RF_DEV double rf_mul_1p(double x, double y) { return rf_fma_band(x, y) ? __fma_rn(x, y, x) : rf_mul_1p_plain(x, y); }

// ---------------------------------------------------------------------------------------
// hash index probe
// ---------------------------------------------------------------------------------------
// 64-bit finaliser of MurmurHash3 (Austin Appleby, public domain): a bijective mixer, so
// distinct keys never collide before range reduction.
RF_DEV unsigned long long rf_mix64(unsigned long long x)
{
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}

// slot of a key in a table of `cap` slots: multiply-high range reduction of the mixed key
RF_DEV unsigned long long rf_home(long long key, unsigned long long cap)
{
    return __umul64hi(rf_mix64((unsigned long long)key), cap);
}

RF_DEV long long rf_locate(const RfIndex& ix, long long key)
{
    if (ix.cap == 0) return -1;
    if (key == RF_EMPTY_KEY) {
        long long r = *ix.special;
        return r == RF_INT64_MAX ? -1 : r;
    }
    unsigned long long h = rf_home(key, ix.cap);
    const longlong2* s = (const longlong2*)ix.slots;
    for (unsigned long long n = 0; n < ix.cap; ++n) {
        longlong2 v = __ldg(s + h);
        if (v.x == key) return v.y;
        if (v.x == RF_EMPTY_KEY) return -1;
        if (++h == ix.cap) h = 0;
    }
    return -1;
}

RF_DEV void rf_set_err(const RfParams& P, int code)
{
    if (P.err) atomicCAS(P.err, 0, code);
}

// 8-byte words through L2 (coherent between the blocks of one grid)
RF_DEV void rf_st_words(void* dst, const void* src, int nbytes)
{
    unsigned long long* d = (unsigned long long*)dst;
    const unsigned long long* s = (const unsigned long long*)src;
    for (int i = 0; i < nbytes / 8; i++) __stcg(d + i, s[i]);
}
RF_DEV void rf_ld_words(void* dst, const void* src, int nbytes)
{
    unsigned long long* d = (unsigned long long*)dst;
    const unsigned long long* s = (const unsigned long long*)src;
    for (int i = 0; i < nbytes / 8; i++) d[i] = __ldcg(s + i);
}

// ---------------------------------------------------------------------------------------
// atomic accumulate of one aggregate into a 64-bit slot (shared or global memory)
// ---------------------------------------------------------------------------------------
RF_DEV void rf_atom_fsum(unsigned long long* p, double v) { atomicAdd((double*)p, v); }
RF_DEV void rf_atom_isum(unsigned long long* p, long long v) { atomicAdd(p, (unsigned long long)v); }
RF_DEV void rf_atom_imax(unsigned long long* p, long long v) { atomicMax((long long*)p, v); }
RF_DEV void rf_atom_imin(unsigned long long* p, long long v) { atomicMin((long long*)p, v); }
RF_DEV void rf_atom_umax(unsigned long long* p, unsigned long long v) { atomicMax(p, v); }
RF_DEV void rf_atom_umin(unsigned long long* p, unsigned long long v) { atomicMin(p, v); }
RF_DEV void rf_atom_or(unsigned long long* p, long long v) { if (v) atomicOr(p, 1ULL); }
RF_DEV void rf_atom_and(unsigned long long* p, long long v) { if (!v) atomicAnd(p, 0ULL); }
// binary64 max/min with std::max/std::min semantics, by compare-and-swap (bounded retries)
RF_DEV bool rf_atom_fmax(unsigned long long* p, double v)
{
    unsigned long long old = *(volatile unsigned long long*)p;
    for (int i = 0; i < (1 << 20); i++) {
        double cur = __longlong_as_double((long long)old);
        if (!(cur < v)) return true;
        unsigned long long prev = atomicCAS(p, old, (unsigned long long)__double_as_longlong(v));
        if (prev == old) return true;
        old = prev;
    }
    return false;
}
RF_DEV bool rf_atom_fmin(unsigned long long* p, double v)
{
    unsigned long long old = *(volatile unsigned long long*)p;
    for (int i = 0; i < (1 << 20); i++) {
        double cur = __longlong_as_double((long long)old);
        if (!(v < cur)) return true;
        unsigned long long prev = atomicCAS(p, old, (unsigned long long)__double_as_longlong(v));
        if (prev == old) return true;
        old = prev;
    }
    return false;
}

// 64-bit slot encodings
RF_DEV unsigned long long rf_f2u(double x) { return (unsigned long long)__double_as_longlong(x); }
RF_DEV double rf_u2f(unsigned long long x) { return __longlong_as_double((long long)x); }

// ---------------------------------------------------------------------------------------
// FP64 sums on the FP32 pipe.  GB300's FP64 pipe issues about 1/64 of its FP32 rate, and a
// grouped scan spends most of it on its sums.  A sum slot can instead hold an unevaluated pair of
// floats hi + lo (a "double-float", 48 significant bits) while its addends are non-negative: each
// addend is split into two floats with integer operations only, and added with the error-free
// two-sum of Knuth (TAOCP vol. 2, 4.2.2) and Dekker's renormalisation (as in the double-float
// additions of Hida, Li and Bailey's QD library): the pair stays within about 2^-46 of the exact
// running sum, relative to the sum.
// FP64 sums of the same rows in another order differ by the same order of rounding, far inside
// the 1e-12 relative tolerance kept against the serial reference loop.
// A slot's 64 bits hold the pair (hi in the low word, lo in the high word); +0.0 is all zeros in
// both encodings.
// ---------------------------------------------------------------------------------------

// v = hi + lo for a non-negative v, 0 <= v - (hi + lo) < 2^-46 v; false (and nothing set) unless v
// is +0 or a normal double in [2^-103, 2^91): negative values, -0, subnormals, larger values,
// infinities and NaN are left to FP64 arithmetic.  hi takes the exponent and the leading 23
// fraction bits of v (so hi is v truncated to 24 bits); lo the next 23 (the last 6 are dropped),
// built as (1.m - 1.0) x 2^k from two floats with the same exponent, which subtract exactly.  One
// unsigned compare on the high word tests sign and exponent together.  The dropped bits bias a
// sum low by at most 2^-46 of it (2^-47 on average), 4500 times inside a 1e-12 tolerance.
RF_DEV bool rf_df_split(double v, float& hi, float& lo)
{
    const unsigned h = (unsigned)__double2hiint(v), l = (unsigned)__double2loint(v);
    // computed whatever the range (no branch), kept only in range
    const bool in = h - (920u << 20) < (194u << 20);
    const unsigned hb = __funnelshift_l(l, h - (896u << 20), 3);  // exponent - 896, 23 fraction bits
    const unsigned c = (hb & 0x7F800000u) - (23u << 23);           // 2^(exponent of v - 23)
    const float lf = __uint_as_float(c + ((l & 0x1FFFFFFFu) >> 6)) - __uint_as_float(c);
    hi = in ? __uint_as_float(hb) : 0.f;
    lo = in ? lf : 0.f;
    return in || (h | l) == 0u;
}

RF_DEV void rf_two_sum(float a, float b, float& s, float& e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (ah, al) += (bh, bl) for non-negative pairs: Knuth's two-sum of the high parts, the low parts
// added to its error, one renormalisation (Dekker's fast two-sum).  Without cancellation the
// pair stays within about 2^-47 of the exact sum, relative to the sum.  (Ordering the high parts
// by size and taking Dekker's three-addition form for them too measured no faster.)
RF_DEV void rf_df_add_same_sign(float& ah, float& al, float bh, float bl)
{
    float s, e;
    rf_two_sum(ah, bh, s, e);
    e = __fadd_rn(e, __fadd_rn(al, bl));
    ah = __fadd_rn(s, e);
    al = __fsub_rn(e, __fsub_rn(ah, s));
}

// one double-float slot update, in three steps the caller interleaves over a row's slots (so
// their latencies overlap): split the addend, add it to the loaded pair, store.  rf_df_step
// returns false, with nothing to store, when the addend is not a non-negative value in the
// split's range: the caller then turns its slots into doubles and adds in FP64.  A slot so only
// ever sums non-negative values, which keeps the sum well conditioned: its relative error stays
// that of the additions (about 2^-48 times the square root of their number, typically), and it
// cannot reach the float range (addends below 2^91; a thread adds fewer than 2^36 of them to a
// slot in one work unit, far more rows than device memory holds).  Sums with negative addends,
// where cancellation can occur, are left to FP64, whose error relative to the result is 32 times
// smaller.
RF_DEV bool rf_df_step(float2 a, double v, float2& out)
{
    float bh, bl;
    const bool ok = rf_df_split(v, bh, bl);
    rf_df_add_same_sign(a.x, a.y, bh, bl);
    out = a;
    return ok;
}

// the double nearest hi + lo of a double-float slot, as slot bits
RF_DEV unsigned long long rf_df_slot_to_f64(unsigned long long w)
{
    const double hi = (double)__uint_as_float((unsigned)w), lo = (double)__uint_as_float((unsigned)(w >> 32));
    return rf_f2u(__dadd_rn(hi, lo));
}

// ---------------------------------------------------------------------------------------
// Bulk L2 prefetch (sm_90+): the copy engine pulls a contiguous byte range into L2; no
// registers, no shared memory, nothing to wait for.  rf_pf prefetches the rows [r0, r1) of a
// column of `size`-byte values, rounded inwards to whole 16-byte blocks, so it never touches
// bytes outside the rows the caller reads.
// ---------------------------------------------------------------------------------------
RF_DEV void rf_pf(const void* base, long long r0, long long r1, int size)
{
    unsigned long long a = (unsigned long long)base + (unsigned long long)(r0 * size);
    unsigned long long e = (unsigned long long)base + (unsigned long long)(r1 * size);
    a = (a + 15ULL) & ~15ULL;
    e &= ~15ULL;
    if (r1 > r0 && e > a)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"((unsigned)(e - a)) : "memory");
}
