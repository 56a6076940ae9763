"""The C++ drop-in: a program written like the reference's gtest sources (same builder calls,
compile_op<FnTy>, ArrowTable* arguments) compiles against include/ and links the C-ABI library;
on a GPU it reproduces the reference's known answers."""
import os
import subprocess

import numpy as np
import pytest

import refqueries as rq

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dropin_test.cpp")
OUT = os.path.join(ROOT, "tests", "cpp", "_build")


def build_program():
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "dropin_test")
    lib = os.path.join(ROOT, "reffine_gb300", "_lib")
    cmd = ["g++", "-std=c++17", "-O1", SRC, "-I" + os.path.join(ROOT, "include"), "-L" + lib, "-lrf_gpu",
           "-Wl,-rpath," + lib, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_reference_style_program_compiles_and_links():
    assert os.path.exists(build_program())


@pytest.mark.gpu
def test_reference_style_program_runs_on_gpu(tmp_path):
    exe = build_program()
    st = rq.students_table()
    f = tmp_path / "students.bin"
    with open(f, "wb") as h:
        h.write(np.int64(len(st)).tobytes())
        for c in st.columns:
            h.write(np.ascontiguousarray(c.data, dtype=np.int64).tobytes())
    r = subprocess.run([exe, str(f)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "reduce_op 696" in r.stdout
    assert "mismatches 0" in r.stdout
