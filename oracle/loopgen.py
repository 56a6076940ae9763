"""CPU oracle: a restatement of Reffine's CPU compile path for a Func.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (``reffine_gb300``) imports this module;
only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use it, as the
checker.

Reffine compiles a query by (1) lowering ``Op``/``Reduce`` to serial loops over an iteration
space (src/pass/loopgen.cpp, src/pass/reffinepass.cpp, src/iter/iter_space.cpp),
(2) scalarising structs (src/pass/scalarpass.cpp) and (3) emitting C++ (src/pass/cemitter.cpp)
that it compiles with ``clang++ -O3`` and JITs (src/pass/llvmgen.cpp:653-696).  This module
restates steps (1)-(3) in Python, producing the same loop structure as C++ source, which is
compiled here with ``g++ -O3 -ffp-contract=off`` and loaded with ctypes.

Parity notes (where this restatement pins the reference's exact behaviour):
  * loops are serial, in row order, so FP64 sums are sequential (loopgen.cpp:206-269);
  * a struct state is stored field by field, each field's expression reading the fields
    already stored (scalarpass.cpp:121-137);
  * FP constants are printed with ``std::to_string``, i.e. rounded to 6 decimals
    (cemitter.cpp:99-101); integer constants go through ``double`` (expr.h:76-85);
  * ``std::max``/``std::min`` keep their C++ library semantics;
  * the Z3 bound extraction (reffinepass.cpp:9-53) is restated syntactically for
    ``iter <op> affine(vars)``; a comparison that does not involve the iterator yields the
    universal space (the predicate is dropped), as the Z3 query is then unsatisfiable.
Deviations (reference behaviour is undefined or does not compile): ``abs``/``pow`` are emitted
as real function calls (the reference prints ``|x|`` and ``^``, cemitter.cpp:129-136), and a
hash probe of an absent key yields row -1, which ``readdata`` turns into a zero value instead of
reading out of bounds (as it does for a row past the column's end).  A union of two vectors
walks both from their first rows, and a side past its end takes no further part (the reference
reads past it).
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import subprocess
import threading
from typing import Dict, List, Optional

import numpy as np

from reffine_gb300 import ir
from reffine_gb300.table import Table, NP_OF

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
MAX_COLS = 64


class Unsupported(Exception):
    pass


# --------------------------------------------------------------------------------------
# C++ prelude: the runtime helpers of vinstr.h restated (table access, REE, hash locate)
# --------------------------------------------------------------------------------------
PRELUDE = r"""
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <algorithm>
struct rf_ocol { int64_t len; const void* data; const uint16_t* valid; const int32_t* run_ends; int64_t n_run_ends; };
struct rf_oindex { int64_t cap; int64_t* keys; int64_t* vals; };
struct rf_otable { int64_t dim; int64_t ncols; const rf_ocol* cols; const rf_oindex* index; };
struct rf_oout { int64_t len, cap, null_count, ncols; void* cols[64]; uint8_t* bytemap; int64_t esize[64]; };

// vinstr.h:70-74
static inline bool rf_get_null_bit(const uint16_t* bm, int64_t i) { return !bm || (bm[i >> 4] & (1u << (i & 15))); }
// vinstr.h:15-23
static inline int64_t rf_read_runend(const rf_otable* t, int64_t idx, int col) {
    if (idx < 0) return 0; return (int64_t)t->cols[col].run_ends[idx]; }
static inline uint64_t rf_hash64(uint64_t x) {
    x ^= x >> 33; x *= 0xff51afd7ed558ccdULL; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL; x ^= x >> 33; return x; }
// vinstr.h:137-146 (std::unordered_map find; -1 on miss)
static inline int64_t rf_vector_locate(const rf_otable* t, int64_t key) {
    const rf_oindex* ix = t->index; if (!ix) return -1;
    uint64_t m = (uint64_t)ix->cap - 1, h = rf_hash64((uint64_t)key) & m;
    while (ix->vals[h] >= 0) { if (ix->keys[h] == key) return ix->vals[h]; h = (h + 1) & m; }
    return -1; }
template <class T> static inline T rf_read(const rf_otable* t, int col, int64_t idx) {
    if (idx < 0 || idx >= t->cols[col].len) return T(0); return ((const T*)t->cols[col].data)[idx]; }
// a merge side past its last row takes no further part in a union's walk
#define RF_ITER_END INT64_MAX
static inline void rf_out_init(rf_oout* o, int64_t ncols, const int64_t* esize) {
    o->len = 0; o->cap = 0; o->null_count = 0; o->ncols = ncols; o->bytemap = nullptr;
    for (int64_t i = 0; i < ncols; i++) { o->cols[i] = nullptr; o->esize[i] = esize[i]; } }
static inline void rf_out_reserve(rf_oout* o, int64_t n) {
    if (n < o->cap) return; int64_t c = o->cap ? o->cap * 2 : 1024; while (c <= n) c *= 2;
    for (int64_t i = 0; i < o->ncols; i++) o->cols[i] = realloc(o->cols[i], (size_t)(c * o->esize[i]));
    o->bytemap = (uint8_t*)realloc(o->bytemap, (size_t)c); o->cap = c; }
template <class T> static inline void rf_out_write(rf_oout* o, int col, int64_t idx, T v) { ((T*)o->cols[col])[idx] = v; }

extern "C" void* rf_oracle_build_index(const rf_ocol* col0, int runend) {
    // ArrowTable2::build_index (table.h:107-138): int64 column 0 (REE: the run values),
    // valid rows only, first occurrence wins (unordered_map::emplace).
    int64_t n = col0->len; int64_t cap = 16; while (cap < 2 * n + 2) cap *= 2;
    rf_oindex* ix = (rf_oindex*)malloc(sizeof(rf_oindex));
    ix->cap = cap; ix->keys = (int64_t*)malloc(cap * 8); ix->vals = (int64_t*)malloc(cap * 8);
    for (int64_t i = 0; i < cap; i++) ix->vals[i] = -1;
    const int64_t* k = (const int64_t*)col0->data; uint64_t m = (uint64_t)cap - 1;
    for (int64_t i = 0; i < n; i++) {
        if (!rf_get_null_bit(col0->valid, i)) continue;
        uint64_t h = rf_hash64((uint64_t)k[i]) & m;
        while (ix->vals[h] >= 0 && ix->keys[h] != k[i]) h = (h + 1) & m;
        if (ix->vals[h] < 0) { ix->keys[h] = k[i]; ix->vals[h] = i; }
    }
    return ix; }
extern "C" void rf_oracle_free_index(void* p) { rf_oindex* ix = (rf_oindex*)p; if (!ix) return; free(ix->keys); free(ix->vals); free(ix); }
extern "C" void rf_oracle_free_out(rf_oout* o) { for (int64_t i = 0; i < o->ncols; i++) free(o->cols[i]); free(o->bytemap); }
#define RF_MAX(a, b) std::max(a, b)
#define RF_MIN(a, b) std::min(a, b)
"""


def cconst(c: ir.Const) -> str:
    """CEmitter::visit(Const) (cemitter.cpp:89-107)."""
    t = c.type.btype
    if t == "bool":
        return "true" if c.val else "false"
    if t in ("i8", "i16", "i32", "i64", "idx"):
        return "%s(%d)" % (c.type.ctype(), int(c.val))
    if t in ("u8", "u16", "u32", "u64"):
        return "%s(%dULL)" % (c.type.ctype(), int(c.val) & 0xFFFFFFFFFFFFFFFF)
    # std::to_string(double) == "%f"
    return "%s(%s)" % (c.type.ctype(), "%f" % c.val)


# --------------------------------------------------------------------------------------
# Values produced while emitting: a C expression string, a struct (list of values),
# or a vector reference.
# --------------------------------------------------------------------------------------

class Vec:
    """A vector value: an input table (C variable of type ``const rf_otable*``)."""

    def __init__(self, cvar: str, type: ir.DataType):
        self.cvar = cvar
        self.type = type


class SubVec:
    def __init__(self, vec: Vec, start: str, end: str):
        self.vec, self.start, self.end = vec, start, end


class OutVec:
    def __init__(self, cvar: str, type: ir.DataType):
        self.cvar, self.type = cvar, type


# --------------------------------------------------------------------------------------
# Iteration spaces (src/iter/iter_space.cpp), producing C expressions
# --------------------------------------------------------------------------------------

class Space:
    def __init__(self, it):
        self.iter = it  # the IR iterator symbol (or New of symbols for nested)

    def intersect(self, other): return None
    def is_const(self): return False
    def lower_bound(self, g): return None
    def upper_bound(self, g): return None
    def iter_cond(self, g, idx): return "true"
    def idx_to_iter(self, g, idx): return idx
    def iter_to_idx(self, g, it): return it
    def is_alive(self, g, idx): return "true"
    def next(self, g, idx): return "(%s + int64_t(1))" % idx
    def vec_iter_idxs(self, idx): return []
    def extra_syms(self): return []


class Universal(Space):
    def intersect(self, other): return other


class Constant(Space):
    """ConstantSpace: holds a C expression for the bound value."""

    def __init__(self, cexpr: str):
        super().__init__(None)
        self.cexpr = cexpr

    def is_const(self): return True
    def lower_bound(self, g): return self.cexpr
    def upper_bound(self, g): return self.cexpr
    def next(self, g, idx): return idx


class VecSpace(Space):
    def __init__(self, it, vec_sym, vec: Vec, g):
        super().__init__(it)
        self.vec_sym, self.vec = vec_sym, vec
        if vec.type.dim > 2:
            raise Unsupported("only 1d and 2d vectors")
        self.len_var = g.fresh("len")

    def lower_bound(self, g): return self.idx_to_iter(g, "int64_t(0)")
    def upper_bound(self, g): return self.idx_to_iter(g, "(%s - int64_t(1))" % self.len_var)

    def iter_cond(self, g, idx):
        valid = g.fresh("valid")
        g.emit("bool %s = %s;" % (valid, g.readbit(self.vec, idx, 0)))
        return "((%s < %s) && %s)" % (idx, self.len_var, valid)

    def idx_to_iter(self, g, idx): return g.readdata(self.vec, idx, 0)
    def iter_to_idx(self, g, it): return "rf_vector_locate(%s, %s)" % (self.vec.cvar, it)
    def is_alive(self, g, idx): return "(%s < %s)" % (idx, self.len_var)
    def next(self, g, idx): return "(%s + int64_t(1))" % idx
    def vec_iter_idxs(self, idx): return [(self.vec_sym, self.iter, idx)]
    def extra_syms(self): return [(self.len_var, lambda g: g.length(self.vec, 0))]


class SuperSpace(Space):
    def __init__(self, ispace: Space):
        super().__init__(ispace.iter)
        self.ispace = ispace

    def lower_bound(self, g): return self.ispace.lower_bound(g)
    def upper_bound(self, g): return self.ispace.upper_bound(g)
    def iter_cond(self, g, idx): return self.ispace.iter_cond(g, idx)
    def idx_to_iter(self, g, idx): return self.ispace.idx_to_iter(g, idx)
    def iter_to_idx(self, g, it): return self.ispace.iter_to_idx(g, it)
    def is_alive(self, g, idx): return self.ispace.is_alive(g, idx)
    def next(self, g, idx): return self.ispace.next(g, idx)
    def vec_iter_idxs(self, idx): return self.ispace.vec_iter_idxs(idx)
    def extra_syms(self): return self.ispace.extra_syms()


class Filtered(SuperSpace):
    def __init__(self, ispace, cond_sym):
        super().__init__(ispace)
        self.cond_sym = cond_sym

    def iter_cond(self, g, idx):
        c = g.ev(self.cond_sym)
        return "(%s && %s)" % (c, self.ispace.iter_cond(g, idx))

    def intersect(self, other):
        a = self.ispace.intersect(other)
        return Filtered(a, self.cond_sym) if a else None


class LBound(SuperSpace):
    def __init__(self, ispace, bound: Constant):
        super().__init__(ispace)
        self.bound = bound

    def lower_bound(self, g):
        lb = self.ispace.lower_bound(g)
        return "RF_MAX(%s, %s)" % (self.bound.cexpr, lb) if lb else self.bound.cexpr

    def iter_cond(self, g, idx):
        return "((%s >= %s) && %s)" % (self.idx_to_iter(g, idx), self.lower_bound(g),
                                       self.ispace.iter_cond(g, idx))

    def intersect(self, other):
        a = self.ispace.intersect(other)
        return LBound(a, self.bound) if a else None


class UBound(SuperSpace):
    def __init__(self, ispace, bound: Constant):
        super().__init__(ispace)
        self.bound = bound

    def upper_bound(self, g):
        ub = self.ispace.upper_bound(g)
        return "RF_MIN(%s, %s)" % (self.bound.cexpr, ub) if ub else self.bound.cexpr

    def iter_cond(self, g, idx):
        return "((%s <= %s) && %s)" % (self.idx_to_iter(g, idx), self.upper_bound(g),
                                       self.ispace.iter_cond(g, idx))

    def is_alive(self, g, idx):
        return "((%s <= %s) && %s)" % (self.idx_to_iter(g, idx), self.upper_bound(g),
                                       self.ispace.is_alive(g, idx))

    def intersect(self, other):
        a = self.ispace.intersect(other)
        return UBound(a, self.bound) if a else None


class Joint(Space):
    def __init__(self, left: Space, right: Space):
        super().__init__(left.iter)
        self.left, self.right = left, right

    def idx_to_iter(self, g, idx):
        return "RF_MIN(%s, %s)" % (self.left.idx_to_iter(g, idx[0]), self.right.idx_to_iter(g, idx[1]))

    def iter_to_idx(self, g, it):
        return (self.left.iter_to_idx(g, it), self.right.iter_to_idx(g, it))

    def next(self, g, idx):
        li = self.left.idx_to_iter(g, idx[0])
        ri = self.right.idx_to_iter(g, idx[1])
        lc, rc = g.fresh("lcond"), g.fresh("rcond")
        g.emit("bool %s = (%s <= %s);" % (lc, li, ri))
        g.emit("bool %s = (%s <= %s);" % (rc, ri, li))
        return (_tsel(lc, self.left.next(g, idx[0]), idx[0]),
                _tsel(rc, self.right.next(g, idx[1]), idx[1]))

    def vec_iter_idxs(self, idx):
        return self.left.vec_iter_idxs(idx[0]) + self.right.vec_iter_idxs(idx[1])

    def extra_syms(self):
        return self.left.extra_syms() + self.right.extra_syms()


def _tsel(c, a, b):
    if isinstance(a, tuple):
        return tuple(_tsel(c, x, y) for x, y in zip(a, b))
    return "(%s ? %s : %s)" % (c, a, b)


class Union(Joint):
    """UnionSpace (iter_space.cpp:278-316) over two merged vectors.  Where both sides are alive
    this is the reference's walk: the iterator is the smaller of the two current keys and the
    side(s) holding it advance; element reads use each side's current row.  The reference's walk
    is undefined at the tails (it reads an exhausted side past its end, and Locate of the lower
    bound on the side that lacks it gives row -1); here both sides start at their first row and
    a side past its end takes no further part (its key counts as larger than any)."""

    def _plain(self):
        return isinstance(self.left, VecSpace) and isinstance(self.right, VecSpace)

    def _side_iter(self, g, sp, i):
        return "(%s ? %s : RF_ITER_END)" % (sp.is_alive(g, i), sp.idx_to_iter(g, i))

    def idx_to_iter(self, g, idx):
        if not self._plain():
            return Joint.idx_to_iter(self, g, idx)
        return "RF_MIN(%s, %s)" % (self._side_iter(g, self.left, idx[0]), self._side_iter(g, self.right, idx[1]))

    def iter_to_idx(self, g, it):
        if not self._plain():
            return Joint.iter_to_idx(self, g, it)
        return ("int64_t(0)", "int64_t(0)")

    def next(self, g, idx):
        if not self._plain():
            return Joint.next(self, g, idx)
        li = self._side_iter(g, self.left, idx[0])
        ri = self._side_iter(g, self.right, idx[1])
        lc, rc = g.fresh("lcond"), g.fresh("rcond")
        g.emit("bool %s = (%s <= %s);" % (lc, li, ri))
        g.emit("bool %s = (%s <= %s);" % (rc, ri, li))
        return (_tsel(lc, self.left.next(g, idx[0]), idx[0]), _tsel(rc, self.right.next(g, idx[1]), idx[1]))

    def lower_bound(self, g):
        l, r = self.left.lower_bound(g), self.right.lower_bound(g)
        return "RF_MIN(%s, %s)" % (l, r) if (l and r) else (l or r)

    def upper_bound(self, g):
        l, r = self.left.upper_bound(g), self.right.upper_bound(g)
        return "RF_MAX(%s, %s)" % (l, r) if (l and r) else (l or r)

    def iter_cond(self, g, idx):
        return "(%s || %s)" % (self.left.iter_cond(g, idx[0]), self.right.iter_cond(g, idx[1]))

    def is_alive(self, g, idx):
        return "(%s || %s)" % (self.left.is_alive(g, idx[0]), self.right.is_alive(g, idx[1]))

    def intersect(self, other):
        a, b = self.left.intersect(other), self.right.intersect(other)
        return Union(a, b) if (a and b) else None


class Inter(Joint):
    def lower_bound(self, g):
        l, r = self.left.lower_bound(g), self.right.lower_bound(g)
        return "RF_MAX(%s, %s)" % (l, r) if (l and r) else (l or r)

    def upper_bound(self, g):
        l, r = self.left.upper_bound(g), self.right.upper_bound(g)
        return "RF_MIN(%s, %s)" % (l, r) if (l and r) else (l or r)

    def iter_cond(self, g, idx):
        li = self.left.idx_to_iter(g, idx[0])
        ri = self.right.idx_to_iter(g, idx[1])
        lc = self.left.iter_cond(g, idx[0])
        rc = self.right.iter_cond(g, idx[1])
        return "((%s && %s) && (%s == %s))" % (lc, rc, li, ri)

    def is_alive(self, g, idx):
        return "(%s && %s)" % (self.left.is_alive(g, idx[0]), self.right.is_alive(g, idx[1]))

    def intersect(self, other):
        a, b = self.left.intersect(other), self.right.intersect(other)
        return Inter(a, b) if (a and b) else None


class Nested(Space):
    def __init__(self, outer: Space, inner: Space):
        super().__init__(("nested", outer.iter, inner.iter))
        self.outer, self.inner = outer, inner

    def lower_bound(self, g):
        return (self.outer.lower_bound(g), self.inner.lower_bound(g))

    def upper_bound(self, g):
        return (self.outer.upper_bound(g), self.inner.upper_bound(g))

    def iter_cond(self, g, idx):
        return "(%s && %s)" % (self.outer.iter_cond(g, idx[0]), self.inner.iter_cond(g, idx[1]))

    def idx_to_iter(self, g, idx):
        return (self.outer.idx_to_iter(g, idx[0]), self.inner.idx_to_iter(g, idx[1]))

    def iter_to_idx(self, g, it):
        return (self.outer.iter_to_idx(g, it[0]), self.inner.iter_to_idx(g, it[1]))

    def is_alive(self, g, idx):
        return self.outer.is_alive(g, idx[0])

    def next(self, g, idx):
        o_next = self.outer.next(g, idx[0])
        i_next = self.inner.next(g, idx[1])
        i_start = self.iter_to_idx(g, self.lower_bound(g))[1]
        act = g.fresh("inner_alive")
        g.emit("bool %s = %s;" % (act, self.inner.is_alive(g, idx[1])))
        return (_tsel(act, idx[0], o_next), _tsel(act, i_next, i_start))

    def vec_iter_idxs(self, idx):
        return self.outer.vec_iter_idxs(idx[0]) + self.inner.vec_iter_idxs(idx[1])

    def extra_syms(self):
        return self.outer.extra_syms() + self.inner.extra_syms()


def space_and(l: Space, r: Space) -> Space:
    """iter_space.cpp:6-12."""
    a = l.intersect(r)
    b = r.intersect(l)
    return a or b or Inter(l, r)


# --------------------------------------------------------------------------------------
# Code generator
# --------------------------------------------------------------------------------------

def _contains(e: ir.Expr, target) -> bool:
    if e is target:
        return True
    return any(_contains(c, target) for c in e.children())


class Gen:
    def __init__(self, fn: ir.Func, vectorize: bool):
        self.fn = fn
        self.vectorize = vectorize
        self.lines: List[str] = []
        self.indent = 1
        self.counter = 0
        self.scopes: List[Dict[int, object]] = [{}]
        self.typedefs: Dict[ir.DataType, str] = {}
        self.header: List[str] = []
        self.vec_iter_idx: Dict[int, Dict[int, object]] = {}
        self.func_vars: set = set()  # ids of func inputs and symbols visible as vars (Z3 vars)

    # ---------------------------------------------------------------- utils
    def fresh(self, base: str) -> str:
        self.counter += 1
        return "%s_%d" % (base, self.counter)

    def emit(self, line: str):
        self.lines.append("    " * self.indent + line)

    def bind(self, sym, val):
        self.scopes[-1][id(sym)] = val

    def lookup(self, sym):
        for sc in reversed(self.scopes):
            if id(sym) in sc:
                return sc[id(sym)]
        return None

    def push(self):
        self.scopes.append({})
        self.indent += 1

    def pop(self):
        self.scopes.pop()
        self.indent -= 1

    def ctype(self, t: ir.DataType) -> str:
        if t.is_struct():
            if t not in self.typedefs:
                # field types first: nested structs get their typedefs (and names) before this one
                fields = " ".join("%s _%d;" % (self.ctype(d), i) for i, d in enumerate(t.dtypes))
                nm = "_%d_t" % len(self.typedefs)
                self.typedefs[t] = nm
                self.header.append("typedef struct { %s } %s;" % (fields, nm))
            return self.typedefs[t]
        return t.ctype()

    # ---------------------------------------------------------------- vector access
    def length(self, vec: Vec, col: int) -> str:
        return "%s->cols[%d].len" % (vec.cvar, col)

    def readdata(self, vec: Vec, idx: str, col: int) -> str:
        return "rf_read<%s>(%s, %d, %s)" % (vec.type.dtypes[col].ctype(), vec.cvar, col, idx)

    def readbit(self, vec: Vec, idx: str, col: int) -> str:
        return "rf_get_null_bit(%s->cols[%d].valid, %s)" % (vec.cvar, col, idx)

    # ---------------------------------------------------------------- expression evaluation
    def ev(self, e: ir.Expr):
        if isinstance(e, ir.Sym):
            v = self.lookup(e)
            if v is not None:
                return v
            if e in self.fn.tbl:
                val = self.ev(self.fn.tbl[e])
                val = self.materialise(e.name, e.type, val)
                self.bind(e, val)
                return val
            raise Unsupported("unbound symbol %s" % e.name)
        if isinstance(e, ir.Const):
            return cconst(e)
        if isinstance(e, ir.Nary):
            return self.nary(e)
        if isinstance(e, ir.Select):
            c = self.ev(e.cond)
            a, b = self.ev(e.t), self.ev(e.f)
            return _vsel(c, a, b)
        if isinstance(e, ir.Cast):
            return "((%s)%s)" % (e.type.ctype(), self.ev(e.arg))
        if isinstance(e, ir.Get):
            v = self.ev(e.val)
            if isinstance(v, list):
                return v[e.col]
            return v
        if isinstance(e, ir.New):
            return [self.ev(x) for x in e.vals]
        if isinstance(e, ir.Element):
            return self.element(e)
        if isinstance(e, ir.SubVector):
            vec = self.ev(e.vec)
            return SubVec(vec, self.ev(e.start), self.ev(e.end))
        if isinstance(e, ir.Length):
            return self.length(self.ev(e.vec), e.col)
        if isinstance(e, ir.Locate):
            return "rf_vector_locate(%s, %s)" % (self.ev(e.vec).cvar, self.ev(e.iter))
        if isinstance(e, ir.ReadData):
            return self.readdata(self.ev(e.vec), self.ev(e.idx), e.col)
        if isinstance(e, ir.Reduce):
            return self.reduce(e)
        if isinstance(e, ir.Op):
            return self.op(e)
        raise Unsupported("cannot evaluate %s" % type(e).__name__)

    def materialise(self, name, t: ir.DataType, val):
        """CEmitter::visit(Sym): a table symbol is emitted once as a typed variable."""
        if isinstance(val, (Vec, SubVec, OutVec)):
            return val
        if isinstance(val, list):
            return [self.materialise(name + "_%d" % i, t.dtypes[i], v) for i, v in enumerate(val)]
        var = self.fresh(name.replace("#", "_").replace(".", "_").replace("$", "_"))
        self.emit("%s %s = %s;" % (t.ctype(), var, val))
        return var

    def nary(self, e: ir.Nary) -> str:
        """CEmitter::visit(NaryExpr) (cemitter.cpp:112-160)."""
        a = [self.ev(x) for x in e.args]
        bin_ops = {"add": "+", "sub": "-", "mul": "*", "div": "/", "mod": "%", "eq": "==",
                   "and": "&&", "or": "||", "lt": "<", "lte": "<=", "gt": ">", "gte": ">="}
        if e.op in bin_ops:
            return "(%s %s %s)" % (a[0], bin_ops[e.op], a[1])
        if e.op == "max":
            return "RF_MAX(%s, %s)" % (a[0], a[1])
        if e.op == "min":
            return "RF_MIN(%s, %s)" % (a[0], a[1])
        if e.op == "not":
            return "(!%s)" % a[0]
        if e.op == "neg":
            return "(-%s)" % a[0]
        if e.op == "sqrt":
            return "std::sqrt(%s)" % a[0]
        if e.op == "ceil":
            return "ceil(%s)" % a[0]
        if e.op == "floor":
            return "floor(%s)" % a[0]
        if e.op == "abs":
            if e.type.is_float():
                return "std::fabs(%s)" % a[0]
            return "((%s)std::llabs((long long)%s))" % (e.type.ctype(), a[0])
        if e.op == "pow":
            return "std::pow(%s, %s)" % (a[0], a[1])
        raise Unsupported("op %s" % e.op)

    def element(self, e: ir.Element):
        """LoopGen::visit(Element) (loopgen.cpp:12-42)."""
        vec = self.ev(e.vec)
        it = self.ev(e.iter)
        m = self.vec_iter_idx.get(id(e.vec))
        if m is not None and id(e.iter) in m:
            idx = m[id(e.iter)]
        else:
            idx = "rf_vector_locate(%s, %s)" % (vec.cvar, it)
        if vec.type.dim == 1:
            return [self.readdata(vec, idx, i) for i in range(vec.type.dim, len(vec.type.dtypes))]
        if vec.type.dim == 2:
            s = "rf_read_runend(%s, (%s - int64_t(1)), 0)" % (vec.cvar, idx)
            t = "rf_read_runend(%s, %s, 0)" % (vec.cvar, idx)
            return SubVec(vec, s, t)
        raise Unsupported("Only support 1d and 2d vectors")

    # ---------------------------------------------------------------- iteration spaces
    def space_of(self, pred: ir.Expr, it: ir.Sym, vars_: List[ir.Expr]) -> Space:
        """Reffine::visit (reffinepass.cpp:55-105)."""
        if isinstance(pred, ir.Nary):
            if pred.op == "and":
                return space_and(self.space_of(pred.args[0], it, vars_), self.space_of(pred.args[1], it, vars_))
            if pred.op == "or":
                return Union(self.space_of(pred.args[0], it, vars_), self.space_of(pred.args[1], it, vars_))
            if pred.op in ("lt", "lte", "gt", "gte"):
                return self.extract_bound(pred, it, vars_)
            raise Unsupported("Operator not supported by Reffine: %s" % pred.op)
        if isinstance(pred, ir.Sym):
            uni = Universal(it)
            if pred is it:
                return uni
            if pred in self.fn.tbl:
                if pred.type == ir._bool_t:
                    return Filtered(uni, pred)
                return self.space_of(self.fn.tbl[pred], it, vars_)
            raise Unsupported("Unable to reffine symbol %s" % pred.name)
        if isinstance(pred, ir.Const):
            return Constant(cconst(pred))
        if isinstance(pred, ir.In):
            vec = self.ev(pred.vec)
            return space_and(self.space_of(pred.iter, it, vars_), VecSpace(pred.iter, pred.vec, vec, self))
        raise Unsupported("predicate node %s" % type(pred).__name__)

    def affine(self, e: ir.Expr, vars_) -> bool:
        if isinstance(e, ir.Const):
            return True
        if isinstance(e, ir.Sym):
            return any(e is v for v in vars_)
        if isinstance(e, ir.Nary) and e.op in ("add", "sub"):
            return self.affine(e.args[0], vars_) and self.affine(e.args[1], vars_)
        if isinstance(e, ir.Nary) and e.op == "mul":
            return (isinstance(e.args[0], ir.Const) and self.affine(e.args[1], vars_)) or \
                   (isinstance(e.args[1], ir.Const) and self.affine(e.args[0], vars_))
        if isinstance(e, ir.Nary) and e.op == "neg":
            return self.affine(e.args[0], vars_)
        return False

    def extract_bound(self, e: ir.Nary, it: ir.Sym, vars_) -> Space:
        """Restates reffinepass.cpp:9-53 for ``iter <op> affine`` / ``affine <op> iter``."""
        a, b = e.args
        op = e.op
        if a is it and not _contains(b, it):
            rhs = b
        elif b is it and not _contains(a, it):
            rhs = a
            op = {"lt": "gt", "lte": "gte", "gt": "lt", "gte": "lte"}[op]
        elif not _contains(e, it):
            return Universal(it)   # no bound solves the forall query
        else:
            raise Unsupported("bound form not restated: %s" % op)
        if not self.affine(rhs, vars_) or not it.type.is_int() and not it.type.is_idx():
            # Z3 over reals / non-affine terms: no solution of the bound form
            return Universal(it)
        r = self.ev(rhs)
        ct = it.type.ctype()
        if op == "gte":
            return LBound(Universal(it), Constant("((%s)(%s))" % (ct, r)))
        if op == "gt":
            return LBound(Universal(it), Constant("((%s)((%s) + 1))" % (ct, r)))
        if op == "lte":
            return UBound(Universal(it), Constant("((%s)(%s))" % (ct, r)))
        return UBound(Universal(it), Constant("((%s)((%s) - 1))" % (ct, r)))

    def op_space(self, op: ir.Op, vars_) -> Space:
        """Reffine::visit(Op) (reffinepass.cpp:107-123)."""
        it = op.iters[0]
        sp = self.space_of(op.pred, it, vars_)
        if len(op.iters) > 1:
            inner = ir.Op(op.iters[1:], op.pred, op.outputs)
            return Nested(sp, self.op_space(inner, vars_ + [it]))
        return sp

    # ---------------------------------------------------------------- loops
    def build_loop(self, op: ir.Op):
        """LoopGen::build_loop (loopgen.cpp:44-111).  Returns (idx vars, space, loop_iter fn)."""
        vars_ = [s for s in self.fn.inputs if s.type.is_val()] + self.outer_iters
        sp = self.op_space(op, vars_)
        lb = sp.lower_bound(self)
        if lb is None:
            raise Unsupported("unbounded iteration space")
        lb_var = self._assign_tuple("lb", lb)
        idx_init = sp.iter_to_idx(self, lb_var)
        idx = self._assign_tuple("idx", idx_init)
        for (name, fn) in sp.extra_syms():
            self.emit("int64_t %s = %s;" % (name, fn(self)))
        return sp, idx

    def _assign_tuple(self, base, val):
        if isinstance(val, tuple):
            return tuple(self._assign_tuple(base, v) for v in val)
        var = self.fresh(base)
        self.emit("int64_t %s = %s;" % (var, val))
        return var

    def _store_tuple(self, var, val):
        if isinstance(var, tuple):
            tmps = [self._tmp_tuple(v) for v in val]
            for v, t in zip(var, tmps):
                self._store_tuple_direct(v, t)
            return
        self.emit("%s = %s;" % (var, val))

    def _tmp_tuple(self, val):
        if isinstance(val, tuple):
            return tuple(self._tmp_tuple(v) for v in val)
        t = self.fresh("nx")
        self.emit("int64_t %s = %s;" % (t, val))
        return t

    def _store_tuple_direct(self, var, t):
        if isinstance(var, tuple):
            for v, x in zip(var, t):
                self._store_tuple_direct(v, x)
        else:
            self.emit("%s = %s;" % (var, t))

    outer_iters: List[ir.Sym] = []

    def loop_body_bind(self, op: ir.Op, sp: Space, idx):
        """Bind op iterators and vec->iter->idx map inside the loop body."""
        for (vec_sym, it_sym, ix) in sp.vec_iter_idxs(idx):
            self.vec_iter_idx.setdefault(id(vec_sym), {})[id(it_sym)] = ix
        it_val = sp.idx_to_iter(self, idx)
        if len(op.iters) == 1:
            var = self.fresh(op.iters[0].name)
            self.emit("%s %s = %s;" % (op.iters[0].type.ctype(), var, it_val))
            self.bind(op.iters[0], var)
        else:
            flat = _flatten(it_val)
            for s, v in zip(op.iters, flat):
                var = self.fresh(s.name)
                self.emit("%s %s = %s;" % (s.type.ctype(), var, v))
                self.bind(s, var)

    def reduce(self, red: ir.Reduce):
        """LoopGen::visit(Reduce) (loopgen.cpp:206-269)."""
        st_t = red.type
        init = self.ev(red.init)
        state = self.state_vars(st_t, init)
        if isinstance(red.vec, ir.Op):
            op = red.vec
            sp, idx = self.build_loop(op)
            self.emit("while (1) {")
            self.push()
            self.emit("if (!(%s)) break;" % sp.is_alive(self, idx))
            self.loop_body_bind(op, sp, idx)
            saved = self.outer_iters
            self.outer_iters = saved + list(op.iters)
            cond = sp.iter_cond(self, idx)
            outs = [self.ev(i) for i in op.iters] + [self.ev(o) for o in op.outputs]
            self.update_state(red, state, outs, cond)
            nxt = sp.next(self, idx)
            self._store_tuple(idx, nxt)
            self.outer_iters = saved
            self.pop()
            self.emit("}")
            return state
        vec = self.ev(red.vec)
        if not isinstance(vec, SubVec):
            raise Unsupported("Unsupported reduction vector")
        rvec = vec.vec
        i = self.fresh("red_idx")
        self.emit("int64_t %s = %s;" % (i, vec.start))
        end = self.fresh("red_end")
        self.emit("int64_t %s = %s;" % (end, vec.end))
        self.emit("while (1) {")
        self.push()
        self.emit("if (%s >= %s) break;" % (i, end))
        outs = [self.readdata(rvec, i, c) for c in range(1, len(rvec.type.dtypes))]
        cond = self.readbit(rvec, i, 1)
        self.update_state(red, state, outs, cond)
        self.emit("%s = %s + int64_t(1);" % (i, i))
        self.pop()
        self.emit("}")
        return state

    def state_vars(self, t: ir.DataType, init):
        if t.is_struct():
            return [self.state_vars(d, v) for d, v in zip(t.dtypes, init)]
        var = self.fresh("state")
        self.emit("%s %s = %s;" % (t.ctype(), var, init))
        return var

    def update_state(self, red: ir.Reduce, state, outs, cond):
        self.push()
        self.bind(red.state, state)
        self.bind(red.val, outs)
        if self.vectorize:
            newv = self.ev(red.acc)
            self._store_state(state, newv, cond)
        else:
            self.emit("if (%s) {" % cond)
            self.push()
            newv = self.ev(red.acc)
            self._store_state(state, newv, None)
            self.pop()
            self.emit("}")
        self.pop()

    def _store_state(self, state, newv, cond):
        """ScalarPass::visit(Store) (scalarpass.cpp:121-137): field by field, in order."""
        if isinstance(state, list):
            for s, v in zip(state, newv):
                self._store_state(s, v, cond)
            return
        if cond is None:
            self.emit("%s = %s;" % (state, newv))
        else:
            self.emit("%s = (%s ? %s : %s);" % (state, cond, newv, state))

    def op(self, op: ir.Op):
        """LoopGen::visit(Op) (loopgen.cpp:113-204) + finalize_vector (vinstr.h:113-135)."""
        out = self.fresh("out_vec")
        ncols = len(op.iters) + len(op.outputs)
        if ncols > MAX_COLS:
            raise Unsupported("too many output columns")
        types = [i.type for i in op.iters] + [o.type for o in op.outputs]
        for t in types:
            if not t.is_primitive():
                raise Unsupported("data type not supported %s" % t.str())
        es = self.fresh("esize")
        self.emit("int64_t %s[%d] = {%s};" % (es, ncols, ", ".join(str(t.size()) for t in types)))
        self.emit("rf_oout* %s = rf_out_ptr;" % out)
        self.emit("rf_out_init(%s, %d, %s);" % (out, ncols, es))
        oi = self.fresh("out_idx")
        nc = self.fresh("null_count")
        self.emit("int64_t %s = 0; int64_t %s = 0;" % (oi, nc))
        sp, idx = self.build_loop(op)
        self.emit("while (1) {")
        self.push()
        self.emit("if (!(%s)) break;" % sp.is_alive(self, idx))
        self.loop_body_bind(op, sp, idx)
        saved = self.outer_iters
        self.outer_iters = saved + list(op.iters)
        cond = sp.iter_cond(self, idx)
        cv = self.fresh("body_cond")
        self.emit("bool %s = %s;" % (cv, cond))
        if not self.vectorize:
            self.emit("if (%s) {" % cv)
            self.push()
        outs = [self.ev(i) for i in op.iters] + [self.ev(o) for o in op.outputs]
        self.emit("rf_out_reserve(%s, %s);" % (out, oi))
        for c, (t, v) in enumerate(zip(types, outs)):
            self.emit("rf_out_write<%s>(%s, %d, %s, %s);" % (t.ctype(), out, c, oi, v))
        if self.vectorize:
            self.emit("%s->bytemap[%s] = %s;" % (out, oi, cv))
            self.emit("%s += (%s ? int64_t(0) : int64_t(1));" % (nc, cv))
        self.emit("%s = %s + int64_t(1);" % (oi, oi))
        if not self.vectorize:
            self.pop()
            self.emit("}")
        nxt = sp.next(self, idx)
        self._store_tuple(idx, nxt)
        self.outer_iters = saved
        self.pop()
        self.emit("}")
        self.emit("%s->len = %s; %s->null_count = %s;" % (out, oi, out, nc))
        return OutVec(out, op.type)

    # ---------------------------------------------------------------- function
    def run(self) -> str:
        fn = self.fn
        params = []
        out_t = fn.output.type
        if out_t.is_vector():
            params.append("rf_oout* rf_out_ptr")
        else:
            params.append("void* output_addr")
        for s in fn.inputs:
            if s.type.is_vector():
                var = "in_" + self.fresh(s.name.replace("#", "_"))
                params.append("const rf_otable* %s" % var)
                self.bind(s, Vec(var, s.type))
            else:
                var = "in_" + self.fresh(s.name.replace("#", "_"))
                params.append("%s %s" % (s.type.ctype(), var))
                self.bind(s, var)
        val = self.ev(fn.output)
        if out_t.is_vector():
            if not isinstance(val, OutVec):
                raise Unsupported("vector output must be an Op")
        else:
            ctype = self.ctype(out_t)
            self.emit("%s* rf_res = (%s*)output_addr;" % (ctype, ctype))
            self._store_out("(*rf_res)", out_t, val)
        body = "\n".join(self.lines)
        return PRELUDE + "\n".join(self.header) + "\n\nextern \"C\" void rf_query(%s) {\n%s\n}\n" % (
            ", ".join(params), body)

    def _store_out(self, lhs, t, val):
        if t.is_struct():
            for i, (d, v) in enumerate(zip(t.dtypes, val)):
                self._store_out("%s._%d" % (lhs, i), d, v)
        else:
            self.emit("%s = %s;" % (lhs, val))


def _flatten(x):
    if isinstance(x, tuple):
        out = []
        for y in x:
            out.extend(_flatten(y))
        return out
    return [x]


def _vsel(c, a, b):
    if isinstance(a, list):
        return [_vsel(c, x, y) for x, y in zip(a, b)]
    return "(%s ? %s : %s)" % (c, a, b)


# --------------------------------------------------------------------------------------
# ctypes bridge
# --------------------------------------------------------------------------------------

class _OCol(ctypes.Structure):
    _fields_ = [("len", ctypes.c_int64), ("data", ctypes.c_void_p), ("valid", ctypes.c_void_p),
                ("run_ends", ctypes.c_void_p), ("n_run_ends", ctypes.c_int64)]


class _OTable(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int64), ("ncols", ctypes.c_int64),
                ("cols", ctypes.POINTER(_OCol)), ("index", ctypes.c_void_p)]


class _OOut(ctypes.Structure):
    _fields_ = [("len", ctypes.c_int64), ("cap", ctypes.c_int64), ("null_count", ctypes.c_int64),
                ("ncols", ctypes.c_int64), ("cols", ctypes.c_void_p * 64), ("bytemap", ctypes.c_void_p),
                ("esize", ctypes.c_int64 * 64)]


_CT = {"bool": ctypes.c_bool, "i8": ctypes.c_int8, "i16": ctypes.c_int16, "i32": ctypes.c_int32,
       "i64": ctypes.c_int64, "u8": ctypes.c_uint8, "u16": ctypes.c_uint16, "u32": ctypes.c_uint32,
       "u64": ctypes.c_uint64, "f32": ctypes.c_float, "f64": ctypes.c_double, "idx": ctypes.c_int64}


def ctype_of(t: ir.DataType):
    if t.is_struct():
        return type("S", (ctypes.Structure,), {"_fields_": [("_%d" % i, ctype_of(d)) for i, d in enumerate(t.dtypes)]})
    return _CT[t.btype]


def to_py(v):
    if isinstance(v, ctypes.Structure):
        return tuple(to_py(getattr(v, f[0])) for f in v._fields_)
    if hasattr(v, "value"):
        return v.value
    return v


class OracleTable:
    """A Table as the oracle's C struct, with its hash index (ArrowTable2::build_index)."""

    def __init__(self, lib, t: Table, build_index: bool = True):
        self.t = t
        n = len(t.columns)
        self.cols = (_OCol * n)()
        for i, c in enumerate(t.columns):
            oc = self.cols[i]
            oc.len = len(c.data)
            oc.data = c.data.ctypes.data
            oc.valid = None if c.valid is None else c.valid.ctypes.data
            oc.run_ends = None if c.run_ends is None else c.run_ends.ctypes.data
            oc.n_run_ends = 0 if c.run_ends is None else len(c.run_ends)
        self.s = _OTable(t.dim, n, self.cols, None)
        self.lib = lib
        self._ix = None
        if build_index and t.columns and t.columns[0].dtype == "i64":
            self._ix = lib.rf_oracle_build_index(ctypes.byref(self.cols[0]), 0)
            self.s.index = self._ix

    def __del__(self):
        if self._ix:
            try:
                self.lib.rf_oracle_free_index(ctypes.c_void_p(self._ix))
            except Exception:
                pass


_lock = threading.Lock()
_cache: Dict[str, ctypes.CDLL] = {}


def compile_source(src: str) -> ctypes.CDLL:
    h = hashlib.sha1(src.encode()).hexdigest()[:16]
    with _lock:
        if h in _cache:
            return _cache[h]
        os.makedirs(BUILD, exist_ok=True)
        so = os.path.join(BUILD, "q_%s.so" % h)
        if not os.path.exists(so):
            cpp = os.path.join(BUILD, "q_%s.cpp" % h)
            with open(cpp, "w") as f:
                f.write(src)
            tmp = so + ".%d.tmp" % os.getpid()
            # -ffp-contract=off: no FMA contraction, so rounding matches a plain mul+add
            cmd = ["g++", "-std=c++17", "-O3", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
                   "-shared", cpp, "-o", tmp]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("oracle compile failed:\n%s\n%s" % (r.stderr, src))
            os.replace(tmp, so)
        lib = ctypes.CDLL(so)
        lib.rf_oracle_build_index.restype = ctypes.c_void_p
        lib.rf_oracle_build_index.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.rf_oracle_free_index.argtypes = [ctypes.c_void_p]
        _cache[h] = lib
        return lib


class Query:
    """A compiled oracle query: ``q(*args)`` with Tables / Python scalars in Func input order."""

    def __init__(self, fn: ir.Func, vectorize: bool = False):
        self.fn = fn
        self.vectorize = vectorize
        self.src = Gen(fn, vectorize).run()
        self.lib = compile_source(self.src)
        self.entry = self.lib.rf_query
        self.entry.restype = None
        self._otables: Dict[int, OracleTable] = {}

    def table(self, t: Table) -> OracleTable:
        ot = self._otables.get(id(t))
        if ot is None or ot.t is not t:
            ot = OracleTable(self.lib, t)
            self._otables[id(t)] = ot
        return ot

    def prepare(self, *args):
        """Build the argument list once (tables' indexes included) so timing covers only the
        query loop."""
        out_t = self.fn.output.type
        cargs = []
        if out_t.is_vector():
            out = _OOut()
            cargs.append(ctypes.byref(out))
        else:
            out = ctype_of(out_t)()
            cargs.append(ctypes.byref(out))
        for s, a in zip(self.fn.inputs, args):
            if s.type.is_vector():
                cargs.append(ctypes.byref(self.table(a).s))
            elif s.type.is_float():
                cargs.append(_CT[s.type.btype](float(a)))
            else:
                cargs.append(_CT[s.type.btype](int(a)))
        return out, cargs

    def run_prepared(self, out, cargs):
        self.entry(*cargs)

    def result(self, out):
        out_t = self.fn.output.type
        if out_t.is_vector():
            res = {"len": out.len, "null_count": out.null_count, "cols": [], "valid": None}
            types = out_t.dtypes
            for c in range(out.ncols):
                npt = NP_OF[types[c].btype]
                if out.len:
                    buf = (ctypes.c_char * (out.len * np.dtype(npt).itemsize)).from_address(out.cols[c])
                    arr = np.frombuffer(bytes(buf), dtype=npt).copy()
                else:
                    arr = np.zeros(0, dtype=npt)
                res["cols"].append(arr)
            if out.null_count > 0:
                bm = (ctypes.c_uint8 * out.len).from_address(out.bytemap)
                res["valid"] = np.frombuffer(bytes(bm), dtype=np.uint8).astype(bool)
            self.lib.rf_oracle_free_out(ctypes.byref(out))
            return res
        return to_py(out)

    def __call__(self, *args):
        out, cargs = self.prepare(*args)
        self.entry(*cargs)
        return self.result(out)
