"""Host tables in Reffine's layout (numpy-backed).

A table mirrors Reffine's ``ArrowTable2`` (include/reffine/arrow/table.h:15-151): a struct
array ("+s") whose children are the columns.  Column 0 is the iterator column; ``dim`` is
the number of iterator columns.  A run-end encoded column (Arrow format "+r",
table.h:64-105) has two children: int32 run ends and the run values.

Validity bitmaps use Arrow's LSB bit order; Reffine reads them as uint16 words
(vinstr.h:70-74), which on a little-endian host is the same bit.  A missing bitmap
means all valid.

``Table.arrow()`` exports the Arrow C Data Interface structs (``ArrowSchema`` /
``ArrowArray``) that the C-ABI's ``rf_table_upload`` consumes; the numpy buffers stay owned
by the Table.
"""
from __future__ import annotations

import ctypes
import os
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import ir

NP_OF = {"bool": np.int8, "i8": np.int8, "i16": np.int16, "i32": np.int32, "i64": np.int64,
         "u8": np.uint8, "u16": np.uint16, "u32": np.uint32, "u64": np.uint64,
         "f32": np.float32, "f64": np.float64, "idx": np.int64}
# Arrow format strings used by Reffine (table.h:82-105; bool is stored as int8 "c", table.h:33)
ARROW_FMT = {"bool": b"c", "i8": b"c", "i16": b"s", "i32": b"i", "i64": b"l",
             "u8": b"C", "u16": b"S", "u32": b"I", "u64": b"L",
             "f32": b"f", "f64": b"g", "idx": b"l"}
TYPE_OF_NP = {np.dtype(np.int8): "i8", np.dtype(np.int16): "i16", np.dtype(np.int32): "i32",
              np.dtype(np.int64): "i64", np.dtype(np.uint8): "u8", np.dtype(np.uint16): "u16",
              np.dtype(np.uint32): "u32", np.dtype(np.uint64): "u64",
              np.dtype(np.float32): "f32", np.dtype(np.float64): "f64"}


class ArrowSchema(ctypes.Structure):
    pass


ArrowSchema._fields_ = [
    ("format", ctypes.c_char_p), ("name", ctypes.c_char_p), ("metadata", ctypes.c_char_p),
    ("flags", ctypes.c_int64), ("n_children", ctypes.c_int64),
    ("children", ctypes.POINTER(ctypes.POINTER(ArrowSchema))),
    ("dictionary", ctypes.POINTER(ArrowSchema)),
    ("release", ctypes.c_void_p), ("private_data", ctypes.c_void_p)]


class ArrowArray(ctypes.Structure):
    pass


ArrowArray._fields_ = [
    ("length", ctypes.c_int64), ("null_count", ctypes.c_int64), ("offset", ctypes.c_int64),
    ("n_buffers", ctypes.c_int64), ("n_children", ctypes.c_int64),
    ("buffers", ctypes.POINTER(ctypes.c_void_p)),
    ("children", ctypes.POINTER(ctypes.POINTER(ArrowArray))),
    ("dictionary", ctypes.POINTER(ArrowArray)),
    ("release", ctypes.c_void_p), ("private_data", ctypes.c_void_p)]


def pack_validity(mask: Optional[np.ndarray]) -> Optional[np.ndarray]:
    """bool mask -> Arrow LSB bitmap, padded to whole uint16 words (Reffine reads words)."""
    if mask is None:
        return None
    mask = np.asarray(mask, dtype=bool)
    nbytes = ((len(mask) + 15) // 16) * 2
    bits = np.packbits(mask, bitorder="little")
    out = np.zeros(max(nbytes, 2), dtype=np.uint8)
    out[: len(bits)] = bits
    return out


def unpack_validity(bitmap: Optional[np.ndarray], n: int) -> np.ndarray:
    if bitmap is None:
        return np.ones(n, dtype=bool)
    return np.unpackbits(np.asarray(bitmap, dtype=np.uint8), bitorder="little")[:n].astype(bool)


class Column:
    """One column: FLAT values (+ validity) or RUNEND (int32 run ends + run values)."""

    def __init__(self, name: str, dtype: str, data: np.ndarray, valid: Optional[np.ndarray] = None,
                 run_ends: Optional[np.ndarray] = None):
        self.name = name
        self.dtype = dtype
        self.data = np.ascontiguousarray(data, dtype=NP_OF[dtype])
        self.valid = None if valid is None else np.ascontiguousarray(valid, dtype=np.uint8)
        self.run_ends = None if run_ends is None else np.ascontiguousarray(run_ends, dtype=np.int32)

    @property
    def encoding(self) -> str:
        return ir.RUNEND if self.run_ends is not None else ir.FLAT

    @property
    def length(self) -> int:
        """Logical length (rows)."""
        if self.run_ends is not None:
            return int(self.run_ends[-1]) if len(self.run_ends) else 0
        return len(self.data)

    @property
    def ir_type(self) -> ir.DataType:
        return ir.DataType(self.dtype)


class Table:
    """Owning host table; ``dim`` iterator columns first (ArrowTable2, table.h:24-60)."""

    def __init__(self, name: str, dim: int, columns: Sequence[Column]):
        self.name = name
        self.dim = dim
        self.columns: List[Column] = list(columns)
        self._keep = []

    @staticmethod
    def from_arrays(dim: int, cols: Dict[str, np.ndarray], name: str = "tbl",
                    valid: Optional[Dict[str, np.ndarray]] = None,
                    runend: Optional[Dict[str, np.ndarray]] = None,
                    types: Optional[Dict[str, str]] = None) -> "Table":
        """``cols`` maps names to values (for a run-end column: the run values);
        ``runend`` maps run-end column names to their int32 run ends; ``valid`` maps names to
        bool masks (over values for FLAT, over runs for RUNEND)."""
        out = []
        for nm, arr in cols.items():
            arr = np.asarray(arr)
            t = (types or {}).get(nm) or TYPE_OF_NP[arr.dtype]
            v = pack_validity((valid or {}).get(nm)) if valid and nm in valid else None
            re = (runend or {}).get(nm)
            out.append(Column(nm, t, arr, v, re))
        return Table(name, dim, out)

    def rows(self, lo: int, hi: int) -> "Table":
        """Rows [lo, hi) as a table of the same type (flat columns share the values; validity
        bitmaps are re-packed from bit lo).  A partition of a table for one rank of a sharded
        query; run-end columns cannot be cut by rows this way."""
        cols = []
        for c in self.columns:
            if c.run_ends is not None:
                raise ValueError("a row range of a run-end column (%s) is not taken" % c.name)
            v = None
            if c.valid is not None:
                v = pack_validity(unpack_validity(c.valid, len(c.data))[lo:hi])
            cols.append(Column(c.name, c.dtype, c.data[lo:hi], v))
        return Table(self.name, self.dim, cols)

    def get_data_type(self) -> ir.DataType:
        """ArrowTable2::get_data_type (table.h:62-80)."""
        return ir.DataType("vector", [c.ir_type for c in self.columns], self.dim,
                           [c.encoding for c in self.columns])

    def __len__(self):
        return self.columns[0].length if self.columns else 0

    @property
    def nrows(self) -> int:
        return len(self)

    def nbytes(self, cols: Optional[Sequence[int]] = None) -> int:
        idx = range(len(self.columns)) if cols is None else cols
        tot = 0
        for i in idx:
            c = self.columns[i]
            tot += c.data.nbytes + (0 if c.valid is None else c.valid.nbytes)
            tot += 0 if c.run_ends is None else c.run_ends.nbytes
        return tot

    # ---------------------------------------------------------------- Arrow C data interface
    def arrow(self):
        """Return (ArrowSchema, ArrowArray) ctypes structs describing this table.  They borrow
        this Table's buffers and have no release callback (the Table owns the memory)."""
        keep = []

        def mk_schema(fmt: bytes, name: bytes, children: List[ArrowSchema]) -> ArrowSchema:
            s = ArrowSchema()
            s.format = fmt
            s.name = name
            s.metadata = None
            s.flags = 2
            s.n_children = len(children)
            if children:
                arr = (ctypes.POINTER(ArrowSchema) * len(children))(*[ctypes.pointer(c) for c in children])
                keep.append(arr)
                s.children = arr
            keep.append(s)
            return s

        def mk_array(length: int, buffers: List[Optional[np.ndarray]], children: List[ArrowArray],
                     null_count: int = 0) -> ArrowArray:
            a = ArrowArray()
            a.length = length
            a.null_count = null_count
            a.offset = 0
            a.n_buffers = len(buffers)
            a.n_children = len(children)
            if buffers:
                bufs = (ctypes.c_void_p * len(buffers))(
                    *[None if b is None else b.ctypes.data for b in buffers])
                keep.append(bufs)
                a.buffers = bufs
            if children:
                ch = (ctypes.POINTER(ArrowArray) * len(children))(*[ctypes.pointer(c) for c in children])
                keep.append(ch)
                a.children = ch
            keep.append(a)
            return a

        sch_children, arr_children = [], []
        for c in self.columns:
            nm = c.name.encode()
            fmt = ARROW_FMT[c.dtype]
            nulls = 0 if c.valid is None else int(
                (~unpack_validity(c.valid, len(c.data))).sum())
            if c.run_ends is None:
                sch_children.append(mk_schema(fmt, nm, []))
                arr_children.append(mk_array(len(c.data), [c.valid, c.data], [], nulls))
            else:
                re_s = mk_schema(b"i", b"run_ends", [])
                va_s = mk_schema(fmt, b"values", [])
                sch_children.append(mk_schema(b"+r", nm, [re_s, va_s]))
                re_a = mk_array(len(c.run_ends), [None, c.run_ends], [])
                va_a = mk_array(len(c.data), [c.valid, c.data], [], nulls)
                arr_children.append(mk_array(c.length, [], [re_a, va_a]))
        schema = mk_schema(b"+s", self.name.encode(), sch_children)
        array = mk_array(len(self), [None], arr_children)
        self._keep = keep
        return schema, array


def ree_encode(keys: np.ndarray):
    """Run-end encode a sorted (or arbitrary) key array: (run values, int32 run ends)."""
    keys = np.asarray(keys)
    if len(keys) == 0:
        return keys[:0], np.zeros(0, dtype=np.int32)
    brk = np.flatnonzero(keys[1:] != keys[:-1]) + 1
    starts = np.concatenate([[0], brk])
    ends = np.concatenate([brk, [len(keys)]]).astype(np.int32)
    return keys[starts], ends


# ---------------------------------------------------------------------------------------------
# Arrow IPC files (load_arrow_file, src/utils/utils.cpp:11-34), read by the library's own parser
# ---------------------------------------------------------------------------------------------
DTYPE_OF_FMT = {"c": "i8", "s": "i16", "i": "i32", "l": "i64", "C": "u8", "S": "u16", "I": "u32", "L": "u64",
                "f": "f32", "g": "f64"}


def read_ipc_c(path: str):
    """Record batch 0 of an Arrow IPC file as (ArrowSchema, ArrowArray); release_c frees them."""
    from . import _capi
    s, a = ArrowSchema(), ArrowArray()
    err = ctypes.create_string_buffer(512)
    rc = _capi.load().rf_ipc_read(path.encode(), ctypes.byref(s), ctypes.byref(a), err, len(err))
    if rc:
        raise _capi.RfError(rc, err.value.decode(errors="replace"))
    return s, a


def release_c(s: "ArrowSchema", a: "ArrowArray"):
    if a.release:
        ctypes.CFUNCTYPE(None, ctypes.POINTER(ArrowArray))(a.release)(ctypes.byref(a))
    if s.release:
        ctypes.CFUNCTYPE(None, ctypes.POINTER(ArrowSchema))(s.release)(ctypes.byref(s))


def ir_type_of_c(s: "ArrowSchema", dim: int) -> ir.DataType:
    """The vector type of a "+s" table schema (ArrowTable2::get_data_type, table.h:62-80)."""
    types, encs = [], []
    for c in range(s.n_children):
        cs = s.children[c].contents
        fmt = cs.format.decode()
        if fmt == "+r":
            types.append(ir.DataType(DTYPE_OF_FMT[cs.children[1].contents.format.decode()]))
            encs.append(ir.RUNEND)
        else:
            types.append(ir.DataType(DTYPE_OF_FMT[fmt]))
            encs.append(ir.FLAT)
    return ir.DataType("vector", types, dim, encs)


def _copy(ptr, n: int, dtype) -> np.ndarray:
    out = np.zeros(n, dtype=dtype)
    if n and ptr:
        ctypes.memmove(out.ctypes.data, ptr, n * out.itemsize)
    return out


def _bitmap(ptr, n: int) -> Optional[np.ndarray]:
    if not ptr:
        return None
    out = np.zeros(max(((n + 15) // 16) * 2, 2), dtype=np.uint8)
    ctypes.memmove(out.ctypes.data, ptr, ((n + 15) // 16) * 2)
    return out


def table_from_ipc(path: str, dim: int, name: Optional[str] = None) -> Table:
    """A host Table holding record batch 0 of an Arrow IPC file (copied out of the file)."""
    s, a = read_ipc_c(path)
    try:
        cols = []
        for c in range(s.n_children):
            cs, ca = s.children[c].contents, a.children[c].contents
            nm, fmt = cs.name.decode(), cs.format.decode()
            if fmt == "+r":
                re_a = ca.children[0].contents
                vs, va = cs.children[1].contents, ca.children[1].contents
                dt = DTYPE_OF_FMT[vs.format.decode()]
                run_ends = _copy(re_a.buffers[1], re_a.length, np.int32)
                cols.append(Column(nm, dt, _copy(va.buffers[1], va.length, NP_OF[dt]), _bitmap(va.buffers[0], va.length),
                                   run_ends))
            else:
                dt = DTYPE_OF_FMT[fmt]
                cols.append(Column(nm, dt, _copy(ca.buffers[1], ca.length, NP_OF[dt]), _bitmap(ca.buffers[0], ca.length)))
        return Table(name or os.path.splitext(os.path.basename(path))[0], dim, cols)
    finally:
        release_c(s, a)
