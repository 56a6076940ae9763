#!/usr/bin/env python3
"""Builds oracle/_ref/libref_pipeline.so: Reffine's own CPU compile path, from a Reffine checkout,
for the oracle's tests.  Test infrastructure: nothing in the product loads it.

    python oracle/ref/build_ref.py [REFFINE_SRC]      (default: /root/reference)

Compiled with g++ directly from the checkout's own sources (no CMake, nothing copied):
  src/base/type.cpp, src/builder/reffiner.cpp, src/ir/ir.cpp, src/iter/iter_space.cpp,
  src/arrow/base.cpp, src/pass/{irclone,canonpass,readwritepass,scalarpass,cemitter,loopgen,
  reffinepass}.cpp, src/vinstr/external.cpp, src/engine/memory.cpp
and oracle/ref/ref_pipeline.cpp (the C-ABI), with oracle/ref/shim ahead on the include path for
the two headers that need libraries absent here: printer2.h (LLVM; only ir.cpp's printing uses it)
and z3solver.h (Z3; a stand-in that decides the linear bound queries of reffinepass.cpp:9-53).
The checkout's path is written to oracle/_ref/ref_src.txt: the C++ text the pipeline emits
includes the checkout's reffine/vinstr/vinstr.h.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
SOURCES = ["src/base/type.cpp", "src/builder/reffiner.cpp", "src/ir/ir.cpp",
           "src/iter/iter_space.cpp", "src/arrow/base.cpp", "src/pass/irclone.cpp",
           "src/pass/canonpass.cpp", "src/pass/readwritepass.cpp", "src/pass/scalarpass.cpp",
           "src/pass/cemitter.cpp", "src/pass/loopgen.cpp", "src/pass/reffinepass.cpp",
           "src/vinstr/external.cpp", "src/engine/memory.cpp"]
LIB = os.path.join(OUT, "libref_pipeline.so")


def build(src: str = "/root/reference", quiet: bool = False) -> str:
    src = os.path.abspath(src)
    if not os.path.isdir(os.path.join(src, "include", "reffine")):
        raise FileNotFoundError("not a Reffine checkout: %s" % src)
    os.makedirs(OUT, exist_ok=True)
    flags = ["g++", "-std=c++20", "-O1", "-fPIC", "-w",
             "-I", os.path.join(HERE, "shim"), "-I", HERE, "-I", os.path.join(src, "include")]
    units = [os.path.join(src, s) for s in SOURCES] + [os.path.join(HERE, "ref_pipeline.cpp")]
    objs = [os.path.join(OUT, os.path.basename(u).replace(".cpp", ".o")) for u in units]

    def compile_one(pair):
        unit, obj = pair
        if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(unit), _newest_header()):
            return
        r = subprocess.run(flags + ["-c", unit, "-o", obj], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compiling %s failed:\n%s" % (unit, r.stderr[-4000:]))

    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        list(ex.map(compile_one, zip(units, objs)))
    tmp = LIB + ".%d.tmp" % os.getpid()
    r = subprocess.run(["g++", "-shared", "-o", tmp] + objs, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("linking failed:\n%s" % r.stderr[-4000:])
    os.replace(tmp, LIB)
    with open(os.path.join(OUT, "ref_src.txt"), "w") as f:
        f.write(src)
    if not quiet:
        print("built %s" % LIB)
    return LIB


def _newest_header() -> float:
    t = 0.0
    for d, _, fs in os.walk(HERE):
        for f in fs:
            if f.endswith(".h"):
                t = max(t, os.path.getmtime(os.path.join(d, f)))
    return t


if __name__ == "__main__":
    build(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
