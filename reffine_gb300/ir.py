"""Reffine IR builder (Python side).

Mirrors the node set and builder DSL of Reffine's C++ IR
(include/reffine/ir/{expr,op,op_to_loop,stmt}.h, include/reffine/builder/reffiner.h:69-187)
and the construction surface of its pybind11 module (python/bindings/ir.cpp:24-217):
the same ``_op``/``_red``/``_in``/``_sym``/``_i64``/... names, the same typing rules
(type.h:132-154 ``valty``/``iterty``/``rowty``) and the same ``Func`` + symbol table.

A ``Func`` serialises to an S-expression text (``Func.text()``).  That text is what
crosses the C-ABI (``rf_plan_compile``): the GPU lowering pass parses it in C++.
The same objects feed the CPU oracle.
"""
from __future__ import annotations

import itertools
import math
from typing import Callable, Dict, List, Optional, Sequence

# --------------------------------------------------------------------------------------
# Types  (include/reffine/base/type.h:17-250)
# --------------------------------------------------------------------------------------

PRIMS = ("bool", "i8", "i16", "i32", "i64", "u8", "u16", "u32", "u64", "f32", "f64", "idx")
INT_TYPES = ("i8", "i16", "i32", "i64", "u8", "u16", "u32", "u64")
FLOAT_TYPES = ("f32", "f64")
SIGNED = ("i8", "i16", "i32", "i64", "f32", "f64")
CTYPES = {
    "bool": "bool", "i8": "int8_t", "i16": "int16_t", "i32": "int32_t", "i64": "int64_t",
    "u8": "uint8_t", "u16": "uint16_t", "u32": "uint32_t", "u64": "uint64_t",
    "f32": "float", "f64": "double", "idx": "int64_t",
}
SIZES = {"bool": 1, "i8": 1, "i16": 2, "i32": 4, "i64": 8, "u8": 1, "u16": 2, "u32": 4,
         "u64": 8, "f32": 4, "f64": 8, "idx": 8}
FLAT, RUNEND = "flat", "runend"


class DataType:
    """A Reffine data type: primitive, ``struct`` or ``vector`` (dim + per-column encodings)."""

    __slots__ = ("btype", "dtypes", "dim", "encodings")

    def __init__(self, btype: str, dtypes: Sequence["DataType"] = (), dim: int = 0,
                 encodings: Sequence[str] = ()):
        self.btype = btype
        self.dtypes = tuple(dtypes)
        self.dim = int(dim)
        self.encodings = tuple(encodings)
        if btype == "struct":
            assert dim == 0 and len(self.dtypes) > 0
        elif btype == "vector":
            assert dim > 0 and len(self.dtypes) >= dim
            if not self.encodings:
                self.encodings = tuple([FLAT] * len(self.dtypes))
            assert len(self.encodings) == len(self.dtypes)
        else:
            assert btype in PRIMS or btype == "void", btype
            assert not self.dtypes and dim == 0

    # equality ignores encodings, as DataType::operator== does (type.h:71-75)
    def __eq__(self, o):
        return (isinstance(o, DataType) and self.btype == o.btype and self.dtypes == o.dtypes
                and self.dim == o.dim)

    def __hash__(self):
        return hash((self.btype, self.dtypes, self.dim))

    def is_struct(self): return self.btype == "struct"
    def is_vector(self): return self.btype == "vector"
    def is_idx(self): return self.btype == "idx"
    def is_val(self): return not self.is_vector()
    def is_float(self): return self.btype in FLOAT_TYPES
    def is_int(self): return self.btype in INT_TYPES
    def is_signed(self): return self.btype in SIGNED
    def is_primitive(self): return self.is_int() or self.is_float() or self.is_idx() or self.btype == "bool"

    def valty(self) -> "DataType":
        assert self.is_vector()
        if self.dim == 1:
            return DataType("struct", self.dtypes[1:])
        return DataType("vector", self.dtypes[1:], self.dim - 1, self.encodings[1:])

    def iterty(self) -> "DataType":
        assert self.is_vector()
        return self.dtypes[0]

    def rowty(self) -> "DataType":
        assert self.is_vector()
        return DataType("struct", self.dtypes)

    def ctype(self) -> str:
        return CTYPES[self.btype]

    def size(self) -> int:
        return SIZES[self.btype]

    def text(self) -> str:
        if self.btype == "struct":
            return "(struct " + " ".join(d.text() for d in self.dtypes) + ")"
        if self.btype == "vector":
            return "(vector %d (%s) (%s))" % (self.dim, " ".join(d.text() for d in self.dtypes),
                                             " ".join(self.encodings))
        return self.btype

    def str(self) -> str:
        if self.btype == "struct":
            return "{" + ", ".join(d.str() for d in self.dtypes) + "}"
        if self.btype == "vector":
            return "<" + ", ".join(d.str() for d in self.dtypes[:self.dim]) + "> {" + \
                ", ".join(d.str() for d in self.dtypes[self.dim:]) + "}"
        return "x" if self.btype == "idx" else ("b" if self.btype == "bool" else self.btype)

    __repr__ = str


_bool_t = DataType("bool")
_i8_t = DataType("i8")
_i16_t = DataType("i16")
_i32_t = DataType("i32")
_i64_t = DataType("i64")
_u8_t = DataType("u8")
_u16_t = DataType("u16")
_u32_t = DataType("u32")
_u64_t = DataType("u64")
_f32_t = DataType("f32")
_f64_t = DataType("f64")
_idx_t = DataType("idx")
_ch_t = _i8_t


def _struct_t(*dtypes: DataType) -> DataType:
    return DataType("struct", dtypes)


def _vec_t(dim: int, dtypes: Sequence[DataType], encodings: Optional[Sequence[str]] = None) -> DataType:
    """types::VEC<dim, Ts...> (type.h:383-392); encodings default to FLAT."""
    return DataType("vector", dtypes, dim, encodings or [FLAT] * len(dtypes))


# --------------------------------------------------------------------------------------
# Expressions  (include/reffine/ir/expr.h, op.h, op_to_loop.h)
# --------------------------------------------------------------------------------------

class Expr:
    """Base expression; operator overloads follow reffiner.h:34-67 (``==`` is ``.eq()`` here,
    because Python uses ``__eq__`` for dictionary keys)."""

    type: DataType

    def __add__(self, o): return _add(self, o)
    def __sub__(self, o): return _sub(self, o)
    def __mul__(self, o): return _mul(self, o)
    def __truediv__(self, o): return _div(self, o)
    def __mod__(self, o): return _mod(self, o)
    def __neg__(self): return _neg(self)
    def __lt__(self, o): return _lt(self, o)
    def __le__(self, o): return _lte(self, o)
    def __gt__(self, o): return _gt(self, o)
    def __ge__(self, o): return _gte(self, o)
    def __and__(self, o): return _and(self, o)
    def __or__(self, o): return _or(self, o)
    def __invert__(self): return _not(self)
    def eq(self, o): return _eq(self, o)
    def ne(self, o): return _not(_eq(self, o))

    def __getitem__(self, key):
        if isinstance(key, Expr):
            return _elem(self, key)
        if isinstance(key, (list, tuple)):
            assert len(key) == 1
            return _elem(self, key[0])
        return _get(self, int(key))

    __hash__ = object.__hash__

    def children(self) -> List["Expr"]:
        return []


class Sym(Expr):
    def __init__(self, name: str, type_or_expr):
        self.name = name
        self.type = type_or_expr.type if isinstance(type_or_expr, Expr) else type_or_expr

    def __repr__(self):
        return "Sym(%s:%s)" % (self.name, self.type.str())


class Const(Expr):
    """Const stores a double, as Reffine's does (expr.h:76-85)."""

    def __init__(self, type: DataType, val):
        assert type.is_primitive(), type
        self.type = type
        self.val = float(val)


class Nary(Expr):
    def __init__(self, type: DataType, op: str, args: Sequence[Expr]):
        self.type = type
        self.op = op
        self.args = list(args)
        a0 = self.args[0].type
        assert not a0.is_struct(), "NaryExpr over a struct"

    def children(self):
        return self.args


class Select(Expr):
    def __init__(self, cond: Expr, t: Expr, f: Expr):
        assert cond.type == _bool_t
        assert t.type == f.type, (t.type, f.type)
        self.type = t.type
        self.cond, self.t, self.f = cond, t, f

    def children(self):
        return [self.cond, self.t, self.f]


class Cast(Expr):
    def __init__(self, type: DataType, arg: Expr):
        assert not arg.type.is_struct() and not type.is_struct()
        self.type = type
        self.arg = arg

    def children(self):
        return [self.arg]


class Get(Expr):
    def __init__(self, val: Expr, col: int):
        if val.type.is_struct():
            self.type = val.type.dtypes[col]
        else:
            assert val.type.is_primitive() and col == 0
            self.type = val.type
        self.val, self.col = val, col

    def children(self):
        return [self.val]


class New(Expr):
    def __init__(self, vals: Sequence[Expr]):
        self.vals = list(vals)
        self.type = DataType("struct", [v.type for v in self.vals])

    def children(self):
        return self.vals


class Op(Expr):
    """op.h:13-56: iterators, predicate, outputs; type is a vector of (iters, outputs)."""

    def __init__(self, iters: Sequence[Sym], pred: Expr, outputs: Sequence[Expr]):
        self.iters = list(iters)
        self.pred = pred
        self.outputs = list(outputs)
        for it in self.iters:
            assert it.type.is_primitive()
        for o in self.outputs:
            assert o.type.is_val()
        dt = [i.type for i in self.iters] + [o.type for o in self.outputs]
        self.type = DataType("vector", dt, len(self.iters), [FLAT] * len(dt))

    def children(self):
        return list(self.iters) + [self.pred] + self.outputs


class Element(Expr):
    def __init__(self, vec: Expr, it: Expr):
        assert vec.type.is_vector()
        assert it.type == vec.type.iterty(), (it.type, vec.type)
        self.vec, self.iter = vec, it
        self.type = vec.type.valty()

    def children(self):
        return [self.vec, self.iter]


class In(Expr):
    def __init__(self, it: Expr, vec: Expr):
        assert it.type == vec.type.iterty()
        self.iter, self.vec = it, vec
        self.type = _bool_t

    def children(self):
        return [self.iter, self.vec]


_red_counter = itertools.count()


class Reduce(Expr):
    """op.h:89-110.  ``init`` and ``acc`` are callables, as in Reffine; they are applied once
    to fresh state/value symbols and the resulting expressions are kept."""

    def __init__(self, vec: Expr, init: Callable[[], Expr], acc: Callable[[Expr, Expr], Expr]):
        assert vec.type.is_vector()
        self.vec = vec
        self.init_fn, self.acc_fn = init, acc
        self.init = init()
        k = next(_red_counter)
        self.state = Sym("s%d" % k, self.init.type)
        self.val = Sym("v%d" % k, vec.type.rowty())
        self.acc = acc(self.state, self.val)
        assert self.acc.type == self.init.type, (self.acc.type, self.init.type)
        self.type = self.init.type

    def children(self):
        return [self.vec, self.init, self.acc]


class SubVector(Expr):
    def __init__(self, vec: Expr, start: Expr, end: Expr):
        assert vec.type.is_vector() and start.type.is_idx() and end.type.is_idx()
        self.vec, self.start, self.end = vec, start, end
        self.type = vec.type.valty()

    def children(self):
        return [self.vec, self.start, self.end]


class Length(Expr):
    def __init__(self, vec: Expr, col: int):
        assert vec.type.is_vector() and col < len(vec.type.dtypes)
        self.vec, self.col = vec, col
        self.type = _idx_t

    def children(self):
        return [self.vec]


class Locate(Expr):
    """op_to_loop.h:106-119: hash-index probe of a vector's iterator column; -1 on miss."""

    def __init__(self, vec: Expr, it: Expr):
        assert vec.type.is_vector() and vec.type.dim <= 2
        assert vec.type.iterty() == it.type
        self.vec, self.iter = vec, it
        self.type = _idx_t

    def children(self):
        return [self.vec, self.iter]


class ReadData(Expr):
    def __init__(self, vec: Expr, idx: Expr, col: int):
        assert vec.type.is_vector() and col < len(vec.type.dtypes)
        self.vec, self.idx, self.col = vec, idx, col
        self.type = vec.type.dtypes[col]

    def children(self):
        return [self.vec, self.idx]


class Func:
    """stmt.h:8-27: name, output expression, input symbols, symbol table."""

    def __init__(self, name: str, output: Expr, inputs: Sequence[Sym], tbl: Optional[Dict[Sym, Expr]] = None,
                 is_kernel: bool = False):
        self.name = name
        self.output = output
        self.inputs = list(inputs)
        self.tbl: Dict[Sym, Expr] = dict(tbl or {})
        self.is_kernel = is_kernel

    def insert_sym(self, sym: Sym, expr: Expr):
        self.tbl[sym] = expr

    def __setitem__(self, sym, expr):
        self.tbl[sym] = expr

    def text(self) -> str:
        return _Printer(self).run()

    def str(self) -> str:
        return self.text()


# --------------------------------------------------------------------------------------
# DSL  (reffiner.h:69-187)
# --------------------------------------------------------------------------------------

def _wrap(x, like: Optional[Expr] = None) -> Expr:
    if isinstance(x, Expr):
        return x
    if like is not None and like.type.is_primitive():
        return Const(like.type, x)
    if isinstance(x, bool):
        return Const(_bool_t, 1.0 if x else 0.0)
    if isinstance(x, int):
        return Const(_i64_t, x)
    if isinstance(x, float):
        return Const(_f64_t, x)
    raise TypeError("cannot use %r as an expression" % (x,))


def _bin(op, a, b, bool_result=False):
    a = _wrap(a, b if isinstance(b, Expr) else None)
    b = _wrap(b, a)
    assert a.type == b.type, "BinaryExpr operand types differ: %s vs %s" % (a.type, b.type)
    return Nary(_bool_t if bool_result else a.type, op, [a, b])


def _add(a, b): return _bin("add", a, b)
def _sub(a, b): return _bin("sub", a, b)
def _mul(a, b): return _bin("mul", a, b)
def _div(a, b): return _bin("div", a, b)
def _max(a, b): return _bin("max", a, b)
def _min(a, b): return _bin("min", a, b)


def _mod(a, b):
    e = _bin("mod", a, b)
    assert not e.type.is_float()
    return e


def _pow(a, b):
    e = _bin("pow", a, b)
    assert e.type.is_float()
    return e


def _lt(a, b): return _bin("lt", a, b, True)
def _lte(a, b): return _bin("lte", a, b, True)
def _gt(a, b): return _bin("gt", a, b, True)
def _gte(a, b): return _bin("gte", a, b, True)
def _eq(a, b): return _bin("eq", a, b, True)


def _and(a, b):
    e = _bin("and", a, b, True)
    assert e.args[0].type == _bool_t
    return e


def _or(a, b):
    e = _bin("or", a, b, True)
    assert e.args[0].type == _bool_t
    return e


def _not(a):
    assert a.type == _bool_t
    return Nary(_bool_t, "not", [a])


def _neg(a): return Nary(a.type, "neg", [a])
def _abs(a): return Nary(a.type, "abs", [a])
def _sqrt(a): return Nary(a.type, "sqrt", [a])


def _ceil(a):
    assert a.type.is_float()
    return Nary(a.type, "ceil", [a])


def _floor(a):
    assert a.type.is_float()
    return Nary(a.type, "floor", [a])


def _sel(c, t, f):
    t = _wrap(t, f if isinstance(f, Expr) else None)
    f = _wrap(f, t)
    return Select(c, t, f)


def _cast(type, arg): return Cast(type, _wrap(arg))
def _get(val, col): return Get(val, col)
def _new(vals): return New(vals)
def _op(iters, pred, outputs): return Op(iters, pred, outputs)
def _red(vec, init, acc): return Reduce(vec, init, acc)
def _in(it, vec): return In(it, vec)
def _elem(vec, it): return Element(vec, it)
def _subvec(vec, start, end): return SubVector(vec, start, end)
def _len(vec, col): return Length(vec, col)
def _locate(vec, it): return Locate(vec, it)
def _readdata(vec, idx, col): return ReadData(vec, idx, col)


def _sym(name: str, type_or_expr) -> Sym:
    return Sym(name, type_or_expr)


def _func(name, output, inputs, tbl=None, is_kernel=False) -> Func:
    return Func(name, output, inputs, tbl, is_kernel)


def _const(type, val): return Const(type, val)
def _i8(v): return Const(_i8_t, v)
def _i16(v): return Const(_i16_t, v)
def _i32(v): return Const(_i32_t, v)
def _i64(v): return Const(_i64_t, v)
def _u8(v): return Const(_u8_t, v)
def _u16(v): return Const(_u16_t, v)
def _u32(v): return Const(_u32_t, v)
def _u64(v): return Const(_u64_t, v)
def _f32(v): return Const(_f32_t, v)
def _f64(v): return Const(_f64_t, v)
def _ch(v): return Const(_i8_t, v)
def _idx(v): return Const(_idx_t, v)
def _true(): return Const(_bool_t, 1)
def _false(): return Const(_bool_t, 0)


# --------------------------------------------------------------------------------------
# Text form (the C-ABI's query description)
# --------------------------------------------------------------------------------------

def _fmt_double(v: float) -> str:
    if math.isnan(v):
        return "nan"
    if math.isinf(v):
        return "inf" if v > 0 else "-inf"
    return repr(float(v))


class _Printer:
    """Prints a Func as S-expressions.  Symbols are printed by unique name; every symbol
    that has a table entry is emitted once in ``(tbl ...)``; op iterators and reduce
    state/value symbols are declared where they are bound."""

    def __init__(self, fn: Func):
        self.fn = fn
        self.names: Dict[int, str] = {}
        self.used = set()

    def name(self, s: Sym) -> str:
        k = id(s)
        if k not in self.names:
            base = "".join(ch if (ch.isalnum() or ch in "_.$") else "_" for ch in s.name) or "sym"
            nm, i = base, 1
            while nm in self.used:
                nm = "%s#%d" % (base, i)
                i += 1
            self.used.add(nm)
            self.names[k] = nm
        return self.names[k]

    def run(self) -> str:
        fn = self.fn
        for s in fn.inputs:
            self.name(s)
        for s in fn.tbl:
            self.name(s)
        inputs = " ".join("(%s %s)" % (self.name(s), s.type.text()) for s in fn.inputs)
        tbl = " ".join("(%s %s)" % (self.name(s), self.e(e)) for s, e in fn.tbl.items())
        return "(func %s %s (inputs %s) (tbl %s))" % (fn.name, self.e(fn.output), inputs, tbl)

    def e(self, x: Expr) -> str:
        if isinstance(x, Sym):
            return self.name(x)
        if isinstance(x, Const):
            return "(const %s %s)" % (x.type.text(), _fmt_double(x.val))
        if isinstance(x, Nary):
            return "(%s %s)" % (x.op, " ".join(self.e(a) for a in x.args))
        if isinstance(x, Select):
            return "(sel %s %s %s)" % (self.e(x.cond), self.e(x.t), self.e(x.f))
        if isinstance(x, Cast):
            return "(cast %s %s)" % (x.type.text(), self.e(x.arg))
        if isinstance(x, Get):
            return "(get %s %d)" % (self.e(x.val), x.col)
        if isinstance(x, New):
            return "(new %s)" % " ".join(self.e(v) for v in x.vals)
        if isinstance(x, Op):
            its = " ".join("(%s %s)" % (self.name(i), i.type.text()) for i in x.iters)
            return "(op (%s) %s (%s))" % (its, self.e(x.pred), " ".join(self.e(o) for o in x.outputs))
        if isinstance(x, Reduce):
            return "(reduce %s %s (%s %s) (%s %s) %s)" % (
                self.e(x.vec), self.e(x.init), self.name(x.state), x.state.type.text(),
                self.name(x.val), x.val.type.text(), self.e(x.acc))
        if isinstance(x, Element):
            return "(elem %s %s)" % (self.e(x.vec), self.e(x.iter))
        if isinstance(x, In):
            return "(in %s %s)" % (self.e(x.iter), self.e(x.vec))
        if isinstance(x, SubVector):
            return "(subvec %s %s %s)" % (self.e(x.vec), self.e(x.start), self.e(x.end))
        if isinstance(x, Length):
            return "(len %s %d)" % (self.e(x.vec), x.col)
        if isinstance(x, Locate):
            return "(locate %s %s)" % (self.e(x.vec), self.e(x.iter))
        if isinstance(x, ReadData):
            return "(readdata %s %s %d)" % (self.e(x.vec), self.e(x.idx), x.col)
        raise TypeError("cannot print %r" % (x,))
