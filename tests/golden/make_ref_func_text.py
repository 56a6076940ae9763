#!/usr/bin/env python3
"""Writes tests/golden/ref_func_text.tsv: the benchmark and golden queries built with Reffine's own
IR builder and printed by the GPU backend's binding (reffine_gb300::func_text), one NAME<TAB>TEXT
line each.

    python tests/golden/make_ref_func_text.py REFFINE_SRC [OUT]

REFFINE_SRC is a checkout of Reffine.  The test program (tests/ref_binding/ref_queries.cpp) is
compiled with g++ together with the binding (reffine_gb300/binding/ref_binding.cpp) and the
reference's LLVM-free IR sources: src/builder/reffiner.cpp, src/base/type.cpp and src/ir/ir.cpp,
the last with oracle/ref/shim ahead on the include path (its printer2.h needs LLVM).  The queries
themselves are in oracle/ref/ref_queries.h, shared with the reference-pipeline oracle.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
FIXTURE = os.path.join(HERE, "ref_func_text.tsv")


def build_and_run(src: str) -> str:
    out_dir = os.path.join(ROOT, "tests", "cpp", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "ref_queries")
    cmd = ["g++", "-std=c++20", "-O1",
           "-I", os.path.join(ROOT, "oracle", "ref", "shim"),
           "-I", os.path.join(ROOT, "oracle", "ref"),
           "-I", os.path.join(src, "include"),
           "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "ref_binding", "ref_queries.cpp"),
           os.path.join(ROOT, "reffine_gb300", "binding", "ref_binding.cpp"),
           os.path.join(src, "src", "builder", "reffiner.cpp"),
           os.path.join(src, "src", "base", "type.cpp"),
           os.path.join(src, "src", "ir", "ir.cpp"),
           "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return subprocess.run([exe], check=True, capture_output=True, text=True).stdout


def main():
    if len(sys.argv) < 2:
        raise SystemExit(__doc__)
    out = sys.argv[2] if len(sys.argv) > 2 else FIXTURE
    text = build_and_run(sys.argv[1])
    with open(out, "w") as f:
        f.write(text)
    print("wrote %s (%d queries)" % (out, len(text.splitlines())))


if __name__ == "__main__":
    main()
