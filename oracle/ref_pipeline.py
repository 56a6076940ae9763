"""Reffine's own compile path run on the CPU, as a check of the oracle.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (``reffine_gb300``) imports this module; the
tests use it to check the oracle (``oracle/loopgen.py``) against Reffine itself, and the golden
generator ``tests/golden/make_ref_pipeline_golden.py`` records its answers.

``oracle/ref/build_ref.py`` builds ``oracle/_ref/libref_pipeline.so`` from a Reffine checkout:
Reffine's builder, IR, iteration spaces and passes (LoopGen, CanonPass, ReadWritePass,
ScalarPass, CEmitter; include/reffine/utils/utils.h:20-54) with two header stand-ins (no LLVM
printer; a Z3 stand-in for the linear bound queries).  ``RefQuery`` takes the C++ text CEmitter
prints for one of the queries of ``oracle/ref/ref_queries.h``, compiles it with g++ against the
checkout's ``reffine/vinstr/vinstr.h`` (Reffine compiles it with ``clang++ -O3`` and JITs it,
src/pass/llvmgen.cpp:653-696), and calls it on ``Table``s copied into Reffine's own ArrowTable2.

``contract``: False compiles with ``-ffp-contract=off`` (every product rounded before it is
added, as the oracle and the GPU kernels do); True lets the compiler fuse ``a*b + c`` into one
FMA, as clang's default ``-ffp-contract=on`` with Reffine's host-targeted JIT does on a CPU with
FMA (src/engine/engine.cpp:32, ``JITTargetMachineBuilder::detectHost``).
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import platform
import subprocess
import threading
from typing import Optional

import numpy as np

from reffine_gb300 import ir
from reffine_gb300.table import NP_OF, Table

from . import loopgen

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "_ref")
LIB = os.path.join(REF, "libref_pipeline.so")

_lock = threading.Lock()
_lib: Optional[ctypes.CDLL] = None
_so_cache = {}


def available() -> bool:
    """The library is built and the checkout it was built from is still there."""
    src = _ref_src()
    return os.path.exists(LIB) and src is not None and os.path.isdir(os.path.join(src, "include"))


def _ref_src() -> Optional[str]:
    p = os.path.join(REF, "ref_src.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        return f.read().strip()


def lib() -> ctypes.CDLL:
    global _lib
    with _lock:
        if _lib is None:
            # RTLD_GLOBAL: the generated code's make_vector / build_vector_index resolve to it
            L = ctypes.CDLL(LIB, mode=ctypes.RTLD_GLOBAL)
            L.refp_emit.restype = ctypes.c_char_p
            L.refp_emit.argtypes = [ctypes.c_char_p, ctypes.c_int]
            L.refp_error.restype = ctypes.c_char_p
            L.refp_func_name.restype = ctypes.c_char_p
            L.refp_table_import.restype = ctypes.c_void_p
            L.refp_table_import.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
            L.refp_table_build_index.argtypes = [ctypes.c_void_p]
            L.refp_table_free.argtypes = [ctypes.c_void_p]
            for f in ("refp_table_len", "refp_table_ncols"):
                getattr(L, f).restype = ctypes.c_int64
                getattr(L, f).argtypes = [ctypes.c_void_p]
            for f in ("refp_col_data", "refp_col_validity"):
                getattr(L, f).restype = ctypes.c_void_p
                getattr(L, f).argtypes = [ctypes.c_void_p, ctypes.c_int64]
            L.refp_col_null_count.restype = ctypes.c_int64
            L.refp_col_null_count.argtypes = [ctypes.c_void_p, ctypes.c_int64]
            _lib = L
        return _lib


def emit(name: str, vectorize: bool) -> tuple:
    """(C++ text, function symbol) of Reffine's pipeline for query ``name``."""
    L = lib()
    with _lock:
        code = L.refp_emit(name.encode(), int(vectorize))
        if code is None:
            raise RuntimeError("Reffine's pipeline failed on %s: %s" % (name, L.refp_error().decode()))
        return code.decode(), L.refp_func_name().decode()


def _compile(code: str, contract: bool) -> ctypes.CDLL:
    flags = ["-ffp-contract=fast"] if contract else ["-ffp-contract=off"]
    if contract and platform.machine() == "x86_64":
        flags.append("-mfma")  # FMA is part of the aarch64 base ISA; on x86-64 it must be enabled
    key = hashlib.sha1((code + " ".join(flags)).encode()).hexdigest()[:16]
    with _lock:
        if key in _so_cache:
            return _so_cache[key]
        so = os.path.join(REF, "q_%s.so" % key)
        if not os.path.exists(so):
            cpp = os.path.join(REF, "q_%s.cpp" % key)
            with open(cpp, "w") as f:
                f.write(code)
            tmp = so + ".%d.tmp" % os.getpid()
            cmd = ["g++", "-std=c++20", "-O3", "-fno-fast-math", "-fPIC", "-shared", "-w"] + flags + \
                  ["-I", os.path.join(_ref_src(), "include"), cpp, "-o", tmp]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("compiling Reffine's generated code failed:\n%s" % r.stderr[-4000:])
            os.replace(tmp, so)
        so_lib = ctypes.CDLL(so)
        _so_cache[key] = so_lib
        return so_lib


# Reffine's generated code keeps an Op's validity bytemap on the stack, sized by the output cap of
# 1e8 rows (loopgen.cpp:150-160): 100 MB, more than a default thread stack
_STACK = 1 << 30


def _on_big_stack(f, args):
    err = []

    def run():
        try:
            f(*args)
        except BaseException as e:  # ctypes errors are re-raised on the caller's thread
            err.append(e)

    with _lock:
        old = threading.stack_size(_STACK)
        try:
            th = threading.Thread(target=run)
            th.start()
        finally:
            threading.stack_size(old)
    th.join()
    if err:
        raise err[0]


class RefTable:
    """A copy of a ``Table`` in Reffine's ArrowTable2 (freed with the object)."""

    def __init__(self, t: Table, index: bool = False):
        s, a = t.arrow()
        self.h = lib().refp_table_import(t.dim, ctypes.addressof(s), ctypes.addressof(a))
        if not self.h:
            raise RuntimeError(lib().refp_error().decode())
        if index and lib().refp_table_build_index(self.h) != 0:
            raise RuntimeError(lib().refp_error().decode())

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.refp_table_free(self.h)
            self.h = None


class RefQuery:
    """Query ``name`` of oracle/ref/ref_queries.h compiled by Reffine's own pipeline.

    ``fn`` is the same query built with the Python builder: its output type says how to read the
    result (tests/test_ref_binding.py checks that both builders make the same graph).  Results
    have the oracle's form (``loopgen.Query``): a nested tuple for a value, a dict with ``len``,
    ``null_count``, ``cols`` and ``valid`` for a table."""

    def __init__(self, name: str, fn: ir.Func, vectorize: bool = False, contract: bool = False):
        self.name = name
        self.fn = fn
        self.code, sym = emit(name, vectorize)
        self.entry = getattr(_compile(self.code, contract), sym)
        self.entry.restype = None

    def __call__(self, *args):
        out_t = self.fn.output.type
        keep = []
        cargs = []
        if out_t.is_vector():
            out = ctypes.c_void_p()
        else:
            out = loopgen.ctype_of(out_t)()
        cargs.append(ctypes.byref(out))
        for s, a in zip(self.fn.inputs, args):
            if s.type.is_vector():
                rt = RefTable(a, index=True)
                keep.append(rt)
                cargs.append(ctypes.c_void_p(rt.h))
            elif s.type.is_float():
                cargs.append(loopgen._CT[s.type.btype](float(a)))
            else:
                cargs.append(loopgen._CT[s.type.btype](int(a)))
        _on_big_stack(self.entry, cargs)
        if not out_t.is_vector():
            return loopgen.to_py(out)
        return self._table(out.value, out_t)

    @staticmethod
    def _table(h, out_t):
        L = lib()
        n = L.refp_table_len(h)
        res = {"len": n, "null_count": 0, "cols": [], "valid": None}
        for c in range(L.refp_table_ncols(h)):
            npt = NP_OF[out_t.dtypes[c].btype]
            size = n * np.dtype(npt).itemsize
            ptr = L.refp_col_data(h, c)
            arr = np.frombuffer(bytes((ctypes.c_char * size).from_address(ptr)), dtype=npt).copy() \
                if n else np.zeros(0, dtype=npt)
            res["cols"].append(arr)
            if c == 0:
                res["null_count"] = L.refp_col_null_count(h, c)
                vb = L.refp_col_validity(h, c)
                if res["null_count"] > 0 and vb:
                    words = np.frombuffer(bytes((ctypes.c_char * (((n + 15) // 16) * 2)).from_address(vb)),
                                          dtype=np.uint8)
                    res["valid"] = np.unpackbits(words, bitorder="little")[:n].astype(bool)
        return res
