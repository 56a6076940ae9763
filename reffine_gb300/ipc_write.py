"""Arrow IPC file writer for host tables, numpy only.

Writes the subset the backend's reader (rf_ipc_read / rf_table_load_ipc) takes: one record batch
of integer, float and run-end encoded columns, uncompressed, no dictionaries.  The encoding
follows the Arrow project's published format: the file is "ARROW1" + padding, the schema
message, the record batch message (each an encapsulated message: continuation marker, metadata
length, FlatBuffers metadata padded to 8 bytes, body), the footer (FlatBuffers), the footer
length and "ARROW1".  Body buffers are 64-byte aligned.

The reference reads such files with load_arrow_file (src/utils/utils.cpp:11-34) and has no writer
of its own; this one exists so that large inputs can be made where pyarrow is not installed.
"""
from __future__ import annotations

import struct
from typing import Callable, List, Optional, Sequence, Tuple

import numpy as np

from . import ir
from .table import Table

_V5 = 4  # MetadataVersion.V5
_INT, _FLOAT, _REE = 2, 3, 22  # Type union members
_SCHEMA, _RECORD_BATCH = 1, 3  # MessageHeader union members
_INT_BITS = {"i8": (8, 1), "u8": (8, 0), "i16": (16, 1), "u16": (16, 0), "i32": (32, 1), "u32": (32, 0),
             "i64": (64, 1), "u64": (64, 0), "bool": (8, 1), "idx": (64, 1)}
_FLOAT_PREC = {"f32": 1, "f64": 2}


class _FB:
    """FlatBuffers encoder that writes front to back: a table's vtable just before the table,
    its children after it, each child offset patched once the child is placed (offsets point
    forward, as the format's unsigned offsets must)."""

    def __init__(self):
        self.b = bytearray(4)  # root offset, patched by finish()

    def _pad(self, align: int, rem: int = 0):
        self.b += b"\0" * ((rem - len(self.b)) % align)

    def _patch_off(self, at: int, target: int):
        struct.pack_into("<I", self.b, at, target - at)

    def table(self, slots: Sequence[Optional[Tuple]]) -> int:
        """slots[i]: None (absent), (fmt, value) for a scalar ('b','B','h','i','q'), or
        ('off', writer) where writer(fb) places the child and returns its position."""
        present = [(i, s) for i, s in enumerate(slots) if s is not None]
        size = lambda s: 4 if s[0] == "off" else struct.calcsize("<" + s[0])
        order = sorted(present, key=lambda p: -size(p[1]))  # 8-byte fields first, stay aligned
        self._pad(2)
        vt = len(self.b)
        nslot = len(slots)
        self.b += b"\0" * (4 + 2 * nslot)
        self._pad(8, 4)  # the table's first field lands on an 8-byte boundary
        pos = len(self.b)
        self.b += struct.pack("<i", pos - vt)
        field_at, kids = {}, []
        for i, s in order:
            self._pad(size(s))
            field_at[i] = len(self.b)
            if s[0] == "off":
                self.b += b"\0" * 4
                kids.append((len(self.b) - 4, s[1]))
            else:
                self.b += struct.pack("<" + s[0], s[1])
        struct.pack_into("<HH", self.b, vt, 4 + 2 * nslot, len(self.b) - pos)
        for i in range(nslot):
            struct.pack_into("<H", self.b, vt + 4 + 2 * i, field_at[i] - pos if i in field_at else 0)
        for at, writer in kids:
            self._patch_off(at, writer(self))
        return pos

    def offsets(self, writers: Sequence[Callable]) -> int:
        self._pad(4)
        pos = len(self.b)
        self.b += struct.pack("<I", len(writers)) + b"\0" * (4 * len(writers))
        for k, w in enumerate(writers):
            self._patch_off(pos + 4 + 4 * k, w(self))
        return pos

    def structs(self, raw: bytes, count: int) -> int:
        self._pad(8, 4)  # elements 8-byte aligned
        pos = len(self.b)
        self.b += struct.pack("<I", count) + raw
        return pos

    def string(self, s: str) -> int:
        self._pad(4)
        pos = len(self.b)
        data = s.encode()
        self.b += struct.pack("<I", len(data)) + data + b"\0"
        return pos

    def finish(self, root: Callable) -> bytes:
        struct.pack_into("<I", self.b, 0, root(self))
        self._pad(8)
        return bytes(self.b)


def _type_slots(dtype: str):
    if dtype in _FLOAT_PREC:
        return _FLOAT, lambda fb: fb.table([("h", _FLOAT_PREC[dtype])])
    if dtype in _INT_BITS:
        bits, sgn = _INT_BITS[dtype]
        return _INT, lambda fb: fb.table([("i", bits), ("B", sgn)])
    raise ValueError("type %s has no Arrow IPC form here" % dtype)


def _field(name: str, dtype: str, nullable: bool, children: Sequence[Callable] = ()) -> Callable:
    if dtype == "ree":
        tt, tw = _REE, (lambda fb: fb.table([]))
    else:
        tt, tw = _type_slots(dtype)
    return lambda fb: fb.table([("off", lambda f: f.string(name)), ("B", int(nullable)), ("B", tt),
                                ("off", tw), None, ("off", lambda f: f.offsets(list(children)))])


def _schema_fields(t: Table) -> List[Callable]:
    out = []
    for c in t.columns:
        if c.encoding == ir.RUNEND:
            kids = [_field("run_ends", "i32", False), _field("values", c.dtype, c.valid is not None)]
            out.append(_field(c.name, "ree", False, kids))
        else:
            out.append(_field(c.name, c.dtype, c.valid is not None))
    return out


def _layout(t: Table):
    """Field nodes, buffers (offset, length) and the body pieces, in the format's depth-first
    order: a flat column has a node and two buffers (validity, values); a run-end column has a
    node of its own and none of its buffers, then its two children."""
    nodes, bufs, pieces = [], [], []
    off = 0

    def add(arr: Optional[np.ndarray], nbytes: int):
        nonlocal off
        if arr is None or nbytes == 0:
            bufs.append((off, 0))
            return
        bufs.append((off, nbytes))
        pieces.append((off, arr, nbytes))
        off += (nbytes + 63) // 64 * 64

    def flat(values: np.ndarray, valid: Optional[np.ndarray]):
        n = len(values)
        nulls = 0
        if valid is not None:
            bits = np.unpackbits(valid, bitorder="little")[:n]
            nulls = int(n - bits.sum())
        nodes.append((n, nulls))
        add(valid if nulls else None, (n + 7) // 8)
        add(values, values.nbytes)

    for c in t.columns:
        if c.encoding == ir.RUNEND:
            nodes.append((c.length, 0))
            flat(c.run_ends, None)
            flat(c.data, c.valid)
        else:
            flat(c.data, c.valid)
    return nodes, bufs, pieces, off


def _message(header_type: int, header: Callable, body_len: int) -> bytes:
    fb = _FB().finish(lambda f: f.table([("h", _V5), ("B", header_type), ("off", header), ("q", body_len)]))
    return struct.pack("<Ii", 0xFFFFFFFF, len(fb)) + fb


def write_ipc(path: str, t: Table) -> int:
    """Writes `t` as an Arrow IPC file with one record batch; returns the file's size."""
    fields = _schema_fields(t)
    schema = lambda f: f.table([("h", 0), ("off", lambda g: g.offsets(fields))])
    nodes, bufs, pieces, body_len = _layout(t)
    rows = len(t)
    rb = lambda f: f.table([("q", rows), ("off", lambda g: g.structs(b"".join(struct.pack("<qq", *x) for x in nodes),
                                                                      len(nodes))),
                            ("off", lambda g: g.structs(b"".join(struct.pack("<qq", *x) for x in bufs), len(bufs)))])
    with open(path, "wb") as fh:
        fh.write(b"ARROW1\0\0")
        fh.write(_message(_SCHEMA, schema, 0))
        batch_at = fh.tell()
        meta = _message(_RECORD_BATCH, rb, body_len)
        fh.write(meta)
        pos = 0
        for off, arr, nbytes in pieces:
            fh.write(b"\0" * (off - pos))
            fh.write(memoryview(np.ascontiguousarray(arr)).cast("B")[:nbytes])
            pos = off + nbytes
        fh.write(b"\0" * (body_len - pos))
        block = struct.pack("<qi4xq", batch_at, len(meta), body_len)
        footer = _FB().finish(lambda f: f.table([("h", _V5), ("off", schema), None,
                                                 ("off", lambda g: g.structs(block, 1))]))
        fh.write(footer)
        fh.write(struct.pack("<i", len(footer)) + b"ARROW1")
        return fh.tell()
