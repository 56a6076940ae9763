"""Python host API over the C-ABI: the GB300 counterpart of Reffine's compile-then-run path.

    eng = Engine()                       # rf_gpu_init            (ExecEngine::Get)
    dt = eng.upload(table)               # rf_table_upload        (device-resident ArrowTable)
    plan = eng.compile(func)             # rf_plan_compile        (compile_op: lower + codegen + JIT)
    out = plan.run(dt)                   # rf_plan_run            (calling the query function)
    fn = compile_op(func, engine=eng)    # rf_plan_thunk          (host ArrowTable in, same call shape)

Reduce results come back as the C struct the reference's generated function writes through
``output_addr`` (scalars, or nested tuples for struct states).
"""
from __future__ import annotations

import ctypes
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _capi, ir
from .table import NP_OF, ArrowArray, ArrowSchema, Table, unpack_validity

_CT = {"bool": ctypes.c_bool, "i8": ctypes.c_int8, "i16": ctypes.c_int16, "i32": ctypes.c_int32,
       "i64": ctypes.c_int64, "u8": ctypes.c_uint8, "u16": ctypes.c_uint16, "u32": ctypes.c_uint32,
       "u64": ctypes.c_uint64, "f32": ctypes.c_float, "f64": ctypes.c_double, "idx": ctypes.c_int64}


def ctype_of(t: ir.DataType):
    """ctypes type with the C layout of a value type (the reference's emitted struct typedefs,
    cemitter.cpp:8-31: fields _0, _1, ... in order, natural alignment)."""
    if t.is_struct():
        return type("RfStruct", (ctypes.Structure,),
                    {"_fields_": [("_%d" % i, ctype_of(d)) for i, d in enumerate(t.dtypes)]})
    return _CT[t.btype]


def from_c(v):
    if isinstance(v, ctypes.Structure):
        return tuple(from_c(getattr(v, f[0])) for f in v._fields_)
    if hasattr(v, "value"):
        return v.value
    return v


class Engine:
    """One device context (rf_ctx): stream, JIT module cache, error state."""

    def __init__(self, device: int = 0):
        self.lib = _capi.load()
        h = ctypes.c_void_p()
        _capi.check(self.lib.rf_gpu_init(device, ctypes.byref(h)), None, "rf_gpu_init failed (no usable GPU?)")
        self.h = h
        self.device = device

    def close(self):
        if self.h:
            self.lib.rf_gpu_shutdown(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, status):
        _capi.check(status, self.h)

    @property
    def stream(self) -> int:
        s = ctypes.c_void_p()
        self.check(self.lib.rf_ctx_stream(self.h, ctypes.byref(s)))
        return s.value or 0

    def sync(self):
        self.check(self.lib.rf_ctx_sync(self.h))

    def launch_count(self) -> int:
        n = ctypes.c_int64()
        self.check(self.lib.rf_ctx_launch_count(self.h, ctypes.byref(n)))
        return n.value

    def upload(self, table: Table, cols: Optional[Sequence[int]] = None, index: bool = False) -> "DeviceTable":
        schema, array = table.arrow()
        h = ctypes.c_void_p()
        if cols is None:
            self.check(self.lib.rf_table_upload(self.h, ctypes.byref(schema), ctypes.byref(array), table.dim, None,
                                                ctypes.byref(h)))
        else:
            arr = (ctypes.c_int32 * len(cols))(*cols)
            self.check(self.lib.rf_table_upload_cols(self.h, ctypes.byref(schema), ctypes.byref(array), table.dim,
                                                     arr, len(cols), None, ctypes.byref(h)))
        dt = DeviceTable(self, h, table.get_data_type(), [c.name for c in table.columns])
        if index:
            dt.build_index()
        return dt

    def load_ipc(self, path: str, dim: int) -> "DeviceTable":
        """Record batch 0 of an Arrow IPC file, streamed from the file to the device by the
        library (rf_table_load_ipc; the role of load_arrow_file, src/utils/utils.cpp:11-34)."""
        h = ctypes.c_void_p()
        self.check(self.lib.rf_table_load_ipc(self.h, path.encode(), dim, None, ctypes.byref(h)))
        names, types, encs = [], [], []
        need = ctypes.c_size_t()
        self.check(self.lib.rf_table_describe(h, None, 0, ctypes.byref(need)))
        buf = ctypes.create_string_buffer(need.value)
        self.check(self.lib.rf_table_describe(h, buf, len(buf), None))
        from .table import DTYPE_OF_FMT
        for line in buf.value.decode().splitlines():
            nm, fmt, enc = line.split("\t")
            names.append(nm)
            types.append(ir.DataType(DTYPE_OF_FMT[fmt]))
            encs.append(ir.RUNEND if enc == "runend" else ir.FLAT)
        return DeviceTable(self, h, ir.DataType("vector", types, dim, encs), names)

    def compile(self, fn: ir.Func, vectorize: bool = False) -> "Plan":
        h = ctypes.c_void_p()
        self.check(self.lib.rf_plan_compile(self.h, fn.text().encode(), int(vectorize), ctypes.byref(h)))
        return Plan(self, h, fn, vectorize)

    def tune_export(self) -> str:
        """The autotuner's choices as text lines "shape-key bucket choice" (tile rows for a Reduce
        scan, hash-table slots per 100 distinct keys for a hash group-by)."""
        need = ctypes.c_size_t()
        self.check(self.lib.rf_tune_export(self.h, None, 0, ctypes.byref(need)))
        buf = ctypes.create_string_buffer(need.value)
        self.check(self.lib.rf_tune_export(self.h, buf, need.value, None))
        return buf.value.decode()

    def tune_import(self, text: str):
        self.check(self.lib.rf_tune_import(self.h, text.encode()))

    def tune_save(self, path: str):
        """Persists the autotuner's choices as JSON (entries keyed by query shape and size bucket)."""
        import json
        entries = [{"shape": k, "bucket": int(b), "choice": int(t)}
                   for k, b, t in (l.split() for l in self.tune_export().splitlines() if l.strip())]
        with open(path, "w") as f:
            json.dump({"version": 2, "entries": entries}, f, indent=1)

    def tune_load(self, path: str):
        import json
        with open(path) as f:
            d = json.load(f)
        # version 1 files name the choice "tile_rows" (they held scan tilings only)
        self.tune_import("".join("%s %d %d\n" % (e["shape"], e["bucket"], e.get("choice", e.get("tile_rows")))
                                 for e in d["entries"]))

    def host_alloc(self, nbytes: int) -> "PinnedBuffer":
        return PinnedBuffer(self, nbytes)


class PinnedBuffer:
    """Page-locked host memory (rf_host_alloc), exposed as a numpy byte array."""

    def __init__(self, eng: Engine, nbytes: int):
        self.eng = eng
        p = ctypes.c_void_p()
        eng.check(eng.lib.rf_host_alloc(eng.h, nbytes, ctypes.byref(p)))
        self.ptr = p.value
        self.nbytes = nbytes
        self.array = np.ctypeslib.as_array((ctypes.c_uint8 * max(nbytes, 1)).from_address(self.ptr))[:nbytes]

    def view(self, dtype, count: int, offset: int = 0) -> np.ndarray:
        return self.array[offset: offset + count * np.dtype(dtype).itemsize].view(dtype)

    def free(self):
        if self.ptr:
            self.eng.lib.rf_host_free(self.eng.h, ctypes.c_void_p(self.ptr))
            self.ptr = None


class DeviceTable:
    def __init__(self, eng: Engine, h, type: ir.DataType, names: List[str]):
        self.eng, self.h, self.type, self.names = eng, h, type, names

    def free(self):
        if self.h:
            self.eng.lib.rf_table_free(self.h)
            self.h = None

    def __del__(self):
        try:
            if self.eng.h:
                self.free()
        except Exception:
            pass

    def build_index(self):
        self.eng.check(self.eng.lib.rf_table_build_index(self.h, None))
        return self

    @property
    def nrows(self) -> int:
        n = ctypes.c_int64()
        self.eng.check(self.eng.lib.rf_table_num_rows(self.h, ctypes.byref(n)))
        return n.value

    @property
    def null_count(self) -> int:
        n = ctypes.c_int64()
        self.eng.check(self.eng.lib.rf_table_null_count(self.h, ctypes.byref(n)))
        return n.value

    def export(self) -> Dict:
        """Copies the table back; returns {"cols": [numpy...], "valid": [bool mask or None...], "len"}."""
        s, a = ArrowSchema(), ArrowArray()
        self.eng.check(self.eng.lib.rf_table_export(self.h, ctypes.byref(s), ctypes.byref(a)))
        try:
            return arrow_to_dict(s, a)
        finally:
            rel_a = ctypes.CFUNCTYPE(None, ctypes.POINTER(ArrowArray))(a.release) if a.release else None
            rel_s = ctypes.CFUNCTYPE(None, ctypes.POINTER(ArrowSchema))(s.release) if s.release else None
            if rel_a:
                rel_a(ctypes.byref(a))
            if rel_s:
                rel_s(ctypes.byref(s))


def arrow_to_dict(s: ArrowSchema, a: ArrowArray) -> Dict:
    """Copies an Arrow struct batch (a table's columns as children) into numpy arrays:
    {"cols": [numpy...], "valid": [bool mask or None...], "len"}."""
    cols, valids = [], []
    for c in range(a.n_children):
        cs, ca = s.children[c].contents, a.children[c].contents
        fmt = cs.format.decode()
        arr = ca
        if fmt == "+r":
            arr = ca.children[1].contents
            fmt = cs.children[1].contents.format.decode()
        dt = {"c": np.int8, "C": np.uint8, "s": np.int16, "S": np.uint16, "i": np.int32, "I": np.uint32,
              "l": np.int64, "L": np.uint64, "f": np.float32, "g": np.float64}[fmt]
        n = arr.length
        vals = np.zeros(n, dtype=dt)
        if n and arr.buffers[1]:
            ctypes.memmove(vals.ctypes.data, arr.buffers[1], n * vals.itemsize)
        cols.append(vals)
        if arr.buffers[0]:
            nb = (n + 15) // 16 * 2
            bm = np.zeros(nb, dtype=np.uint8)
            ctypes.memmove(bm.ctypes.data, arr.buffers[0], nb)
            valids.append(unpack_validity(bm, n))
        else:
            valids.append(None)
    return {"cols": cols, "valid": valids, "len": a.length}


class Plan:
    """A compiled query (rf_plan)."""

    def __init__(self, eng: Engine, h, fn: ir.Func, vectorize: bool):
        self.eng, self.h, self.fn, self.vectorize = eng, h, fn, vectorize
        info = _capi.RfPlanInfo()
        eng.check(eng.lib.rf_plan_info(h, ctypes.byref(info)))
        self.info = info
        self.out_type = fn.output.type
        self._out_ct = None if info.output_is_table else ctype_of(self.out_type)

    def free(self):
        if self.h:
            self.eng.lib.rf_plan_free(self.h)
            self.h = None

    def __del__(self):
        try:
            if self.eng.h:
                self.free()
        except Exception:
            pass

    @property
    def source(self) -> str:
        return self.eng.lib.rf_plan_source(self.h).decode()

    @property
    def kind(self) -> int:
        return self.info.kind

    def args(self, *inputs) -> ctypes.Array:
        if len(inputs) != len(self.fn.inputs):
            raise ValueError("query takes %d inputs, got %d" % (len(self.fn.inputs), len(inputs)))
        arr = (_capi.RfArg * max(len(inputs), 1))()
        for i, (s, v) in enumerate(zip(self.fn.inputs, inputs)):
            if s.type.is_vector():
                if not isinstance(v, DeviceTable):
                    raise TypeError("input %d (%s) must be a DeviceTable" % (i, s.name))
                arr[i].kind, arr[i].table = _capi.RF_ARG_TABLE, v.h
            elif s.type.is_float():
                arr[i].kind, arr[i].f64 = _capi.RF_ARG_F64, float(v)
            else:
                arr[i].kind, arr[i].i64 = _capi.RF_ARG_I64, int(v)
        arr._inputs = inputs  # the device tables must outlive the argument array
        return arr

    def run(self, *inputs):
        """Runs on device tables and returns the value result (Python scalar / nested tuple)."""
        args = self.args(*inputs)
        out = self._out_ct()
        self.eng.check(self.eng.lib.rf_plan_run(self.h, args, len(inputs), ctypes.byref(out), None))
        return from_c(out)

    def run_args(self, args: ctypes.Array, n: int, out: ctypes.Structure):
        self.eng.check(self.eng.lib.rf_plan_run(self.h, args, n, ctypes.byref(out), None))

    def launch(self, args: ctypes.Array, n: int, dev_out=None):
        """Enqueues without waiting (value outputs only)."""
        self.eng.check(self.eng.lib.rf_plan_launch(self.h, args, n, dev_out, None))

    def new_out(self):
        return self._out_ct()

    def tune(self, *inputs, reps: int = 3):
        """Autotunes this query shape for these inputs' size bucket (rf_plan_tune): the tiling of
        a Reduce scan, the table sizing of a hash group-by; returns (choice, ms of the fastest) -
        tile rows, or hash-table slots per 100 distinct keys."""
        args = self.args(*inputs)
        t, ms = ctypes.c_int64(), ctypes.c_double()
        self.eng.check(self.eng.lib.rf_plan_tune(self.h, args, len(inputs), reps, ctypes.byref(t), ctypes.byref(ms)))
        return t.value, ms.value

    def thunk(self):
        """The host query function (reference calling shape) as a ctypes function pointer."""
        p = ctypes.c_void_p()
        self.eng.check(self.eng.lib.rf_plan_thunk(self.h, ctypes.byref(p)))
        return p.value


class Batch:
    """Many Reduce queries in one launch per query shape (rf_batch_*).  add() returns the ctypes
    struct that receives the query's result after wait()/poll()."""

    def __init__(self, eng: Engine, capacity: int = 1024):
        self.eng = eng
        h = ctypes.c_void_p()
        eng.check(eng.lib.rf_batch_create(eng.h, capacity, ctypes.byref(h)))
        self.h = h
        self.capacity = capacity
        self._keep = []

    def add(self, plan: "Plan", *inputs):
        args = plan.args(*inputs)
        out = plan.new_out()
        self.eng.check(self.eng.lib.rf_batch_add(self.h, plan.h, args, len(inputs), ctypes.byref(out)))
        self._keep.append((args, out))
        return out

    def __len__(self):
        return len(self._keep)

    def launch(self):
        self.eng.check(self.eng.lib.rf_batch_launch(self.h, None))

    def wait(self):
        self.eng.check(self.eng.lib.rf_batch_wait(self.h))
        return [from_c(o) for _, o in self._keep]

    def poll(self) -> bool:
        d = ctypes.c_int32()
        self.eng.check(self.eng.lib.rf_batch_poll(self.h, ctypes.byref(d)))
        return bool(d.value)

    def reset(self):
        self.eng.check(self.eng.lib.rf_batch_reset(self.h))
        self._keep = []

    def free(self):
        if self.h:
            self.eng.lib.rf_batch_free(self.h)
            self.h = None

    def __del__(self):
        try:
            if self.eng.h:
                self.free()
        except Exception:
            pass


def check(fn: ir.Func, vectorize: bool = False) -> str:
    """Lowers and compiles a query for sm_103a without a device; returns the generated source."""
    lib = _capi.load()
    buf = ctypes.create_string_buffer(1 << 20)
    st = lib.rf_plan_check(fn.text().encode(), int(vectorize), buf, len(buf))
    if st != _capi.RF_OK:
        raise _capi.RfError(st, buf.value.decode(errors="replace"))
    return buf.value.decode()


def compile_op(fn: ir.Func, vectorize: bool = False, engine: Optional[Engine] = None):
    """compile_op (utils.h:47-54): returns a callable taking host Tables / scalars in the Func's
    input order.  Each call goes through the reference-shaped host function (rf_plan_thunk):
    host tables are copied to the device, the plan runs, the result is copied back."""
    eng = engine or Engine()
    plan = eng.compile(fn, vectorize)
    addr = plan.thunk()
    argtypes = [ctypes.c_void_p]
    for s in fn.inputs:
        if s.type.is_vector():
            argtypes.append(ctypes.c_void_p)
        elif s.type.is_float():
            argtypes.append(_CT[s.type.btype])
        else:
            argtypes.append(_CT[s.type.btype])
    cfn = ctypes.CFUNCTYPE(None, *argtypes)(addr)

    table_out = bool(plan.info.output_is_table)

    def call(*inputs):
        # a table result comes back as an ArrowTable* that the plan keeps (as the reference's
        # memman keeps its outputs, src/engine/memory.cpp:11-16)
        out = ctypes.c_void_p() if table_out else plan.new_out()
        cargs = [ctypes.cast(ctypes.byref(out), ctypes.c_void_p)]
        keep = []
        for s, v in zip(fn.inputs, inputs):
            if s.type.is_vector():
                ref = _RefTable.of(v)
                keep.append(ref)
                cargs.append(ctypes.cast(ctypes.byref(ref), ctypes.c_void_p))
            else:
                cargs.append(v)
        cfn(*cargs)
        if table_out:
            if not out.value:
                raise _capi.RfError(_capi.RF_ERR_DEVICE, "the query function returned no table: " +
                                    eng.lib.rf_last_error(eng.h).decode(errors="replace"))
            return HostArrowTable(out.value)
        return from_c(out)

    call.plan = plan
    call.engine = eng
    return call


class _RefTable(ctypes.Structure):
    """The memory layout of Reffine's ArrowTable (abi.h:56-69): a vtable pointer, then
    {dim, schema, array, index}.  Built here so that Python can call the reference-shaped
    query function; the vtable slot is never used by the backend."""

    _fields_ = [("vptr", ctypes.c_void_p), ("dim", ctypes.c_int64), ("schema", ctypes.POINTER(ArrowSchema)),
                ("array", ctypes.POINTER(ArrowArray)), ("index", ctypes.c_void_p)]

    @staticmethod
    def of(t: Table) -> "_RefTable":
        s, a = t.arrow()
        r = _RefTable(None, t.dim, ctypes.pointer(s), ctypes.pointer(a), None)
        r._keep = (s, a)
        return r


class HostArrowTable:
    """A table result of a query function: the host ArrowTable at `addr` (Reffine's layout,
    abi.h:56-69), owned by the plan that made it."""

    def __init__(self, addr: int):
        self.ref = _RefTable.from_address(addr)

    @property
    def num_rows(self) -> int:
        return int(self.ref.array.contents.length)

    def to_dict(self) -> Dict:
        return arrow_to_dict(self.ref.schema.contents, self.ref.array.contents)
