"""Runs the C++ that Reffine's own compile path emitted for the four benchmark query shapes
(oracle/ref/generated/*.cpp, written by oracle/ref/emit_generated.py from a Reffine checkout),
without the checkout: compiled with g++ together with oracle/ref/runtime (the vinstr.h interface
that code calls, and a host runner).

BENCHMARK AND TEST INFRASTRUCTURE ONLY.  Nothing in the product (``reffine_gb300``) imports this
module.  ``bench.py --impl reference`` times Reffine's generated code with it on the host cores;
the tests check that the code gives the oracle's bits.

``contract``: None leaves floating-point contraction to the compiler's default (g++ fuses a*b + c
where the target has FMA, as clang's default does in Reffine's JIT), False compiles with
``-ffp-contract=off`` (every product rounded before it is added, as the oracle does).
"""
from __future__ import annotations

import ctypes
import os
import re
import subprocess
import threading
from typing import List, Optional

import numpy as np

from reffine_gb300 import ir
from reffine_gb300.table import NP_OF, ArrowArray, ArrowSchema, Table

from . import loopgen

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GEN = os.path.join(HERE, "ref", "generated")
RUNTIME = os.path.join(HERE, "ref", "runtime")
BUILD = os.path.join(HERE, "_build")

_lock = threading.Lock()
_libs = {}


def _source(name: str) -> str:
    with open(os.path.join(GEN, name + ".cpp")) as f:
        return f.read()


def _build(name: str, contract: Optional[bool]) -> ctypes.CDLL:
    tag = {None: "default", False: "exact", True: "fma"}[contract]
    with _lock:
        key = (name, tag)
        if key in _libs:
            return _libs[key]
        os.makedirs(BUILD, exist_ok=True)
        so = os.path.join(BUILD, "refgen_%s_%s.so" % (name, tag))
        srcs = [os.path.join(GEN, name + ".cpp"), os.path.join(RUNTIME, "ref_runner.cpp"),
                os.path.join(RUNTIME, "reffine", "vinstr", "vinstr.h")]
        if not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(s) for s in srcs):
            flags = {None: [], False: ["-ffp-contract=off"], True: ["-ffp-contract=fast"]}[contract]
            tmp = so + ".%d.tmp" % os.getpid()
            cmd = ["g++", "-std=c++17", "-O3", "-fPIC", "-shared", "-w"] + flags + \
                  ["-I", RUNTIME, "-I", os.path.join(ROOT, "include"), srcs[0], srcs[1], "-o", tmp, "-lpthread",
                   # the query's calls of make_vector etc. bind to this library's own runtime, even
                   # where Reffine's (oracle/_ref, same names) is loaded in the process
                   "-Wl,-Bsymbolic"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("compiling Reffine's generated %s failed:\n%s" % (name, r.stderr[-4000:]))
            os.replace(tmp, so)
        L = ctypes.CDLL(so)
        L.rr_table.restype = ctypes.c_void_p
        L.rr_table.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.rr_table_free.argtypes = [ctypes.c_void_p]
        L.rr_output_free.argtypes = [ctypes.c_void_p]
        L.rr_set_output.argtypes = [ctypes.c_uint32, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        L.rr_run.restype = ctypes.c_double
        L.rr_run.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                             ctypes.c_void_p, ctypes.c_int64]
        _libs[key] = L
        return L


class GeneratedQuery:
    """Reffine's emitted code for benchmark query ``name``, on the tables given to ``prepare``.

    ``fn`` is the same query built with the Python builder; its output type says how to read the
    result.  ``run(nthreads)`` runs the query once on each of ``nthreads`` threads at the same
    time and returns (wall seconds, the results of all threads)."""

    def __init__(self, name: str, fn: ir.Func, contract: Optional[bool] = None):
        src = _source(name)
        self.entry_name = re.search(r"^// entry: (\w+)", src, re.M).group(1)
        self.lib = _build(name, contract)
        self.fn = fn
        self.entry = ctypes.cast(getattr(self.lib, self.entry_name), ctypes.c_void_p).value
        out_t = fn.output.type
        self.table_out = out_t.is_vector()
        if self.table_out:
            m = re.search(r"make_vector\(int64_t\(\d+\), uint32_t\((\d+)\)\)", src)
            esize = [np.dtype(NP_OF[t.btype]).itemsize for t in out_t.dtypes]
            arr = (ctypes.c_int * len(esize))(*esize)
            self.lib.rr_set_output(int(m.group(1)), len(esize), arr)
            self.out_bytes = 8
        else:
            self.out_type = loopgen.ctype_of(out_t)
            self.out_bytes = ctypes.sizeof(self.out_type)
        self.handles: List[int] = []
        self._keep = []

    def prepare(self, *tables: Table):
        """Borrows the tables' buffers (Arrow C structs) and builds Locate's indexes."""
        self.release()
        for s, t in zip(self.fn.inputs, tables):
            if not s.type.is_vector():
                raise ValueError("emitted benchmark queries take tables only")
            sch, arr = t.arrow()
            self._keep.append((t, sch, arr, t._keep))
            self.handles.append(self.lib.rr_table(t.dim, ctypes.addressof(sch), ctypes.addressof(arr), 1))

    def run(self, nthreads: int = 1):
        n = len(self.handles)
        tabs = (ctypes.c_void_p * n)(*self.handles)
        out = ctypes.create_string_buffer(self.out_bytes * nthreads)
        sec = self.lib.rr_run(self.entry, nthreads, n, tabs, out, self.out_bytes)
        if sec < 0:
            raise RuntimeError("could not start %d query threads" % nthreads)
        results = []
        for i in range(nthreads):
            if self.table_out:
                h = ctypes.c_void_p.from_buffer(out, i * 8).value
                results.append(self._table(h))
                self.lib.rr_output_free(h)
            else:
                results.append(loopgen.to_py(self.out_type.from_buffer(out, i * self.out_bytes)))
        return sec, results

    def _table(self, h):
        out_t = self.fn.output.type
        top = ctypes.cast(h, ctypes.POINTER(_RrTable)).contents.array.contents
        n = top.length
        res = {"len": n, "null_count": 0, "cols": [], "valid": None}
        for c in range(top.n_children):
            col = top.children[c].contents
            npt = NP_OF[out_t.dtypes[c].btype]
            size = n * np.dtype(npt).itemsize
            res["cols"].append(np.frombuffer(bytes((ctypes.c_char * size).from_address(col.buffers[1])),
                                             dtype=npt).copy() if n else np.zeros(0, dtype=npt))
            if c == 0:
                res["null_count"] = col.null_count
        return res

    def release(self):
        for h in self.handles:
            self.lib.rr_table_free(h)
        self.handles = []
        self._keep = []

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class _RrTable(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int64), ("schema", ctypes.POINTER(ArrowSchema)),
                ("array", ctypes.POINTER(ArrowArray)), ("index", ctypes.c_void_p)]
