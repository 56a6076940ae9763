"""load_arrow_file from C++ (include/reffine_gb300/utils.h): a program compiled against the
drop-in header reads the pyarrow-written fixtures (no GPU needed for the read) and, on a GPU,
runs the filter+sum query on the loaded table with compile_op."""
import os
import subprocess

import numpy as np
import pytest

from oracle import loopgen
from parity import assert_same
from reffine_gb300 import workloads as W
from reffine_gb300.table import table_from_ipc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "ipc_load_test.cpp")
OUT = os.path.join(ROOT, "tests", "cpp", "_build")
GOLDEN = os.path.join(ROOT, "tests", "golden")


def build_program():
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "ipc_load_test")
    lib = os.path.join(ROOT, "reffine_gb300", "_lib")
    cmd = ["g++", "-std=c++17", "-O1", SRC, "-I" + os.path.join(ROOT, "include"), "-L" + lib, "-lrf_gpu",
           "-Wl,-rpath," + lib, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def run(*args):
    r = subprocess.run([build_program(), *args], capture_output=True, text=True, timeout=600)
    return r.returncode, r.stdout


def test_read_filter_sum_file():
    rc, out = run("read", os.path.join(GOLDEN, "ipc_filter_sum.arrow"), "2")
    assert rc == 0, out
    lines = out.splitlines()
    assert lines[0] == "type (vector 2 (i64 i32 f64 f64 f64) (flat flat flat flat flat))"
    assert lines[1] == "rows 5003"
    ref = np.load(os.path.join(GOLDEN, "ipc_filter_sum.npz"))
    sums = {l.split()[1]: float(l.split()[2]) for l in lines[2:]}
    assert list(sums) == list(ref.files)
    for k in ref.files:
        assert sums[k] == pytest.approx(float(ref[k].astype(np.float64).sum()), rel=1e-12), k


def test_read_nulls_and_run_ends():
    rc, out = run("read", os.path.join(GOLDEN, "ipc_types.arrow"), "1")
    assert rc == 0, out
    ref = np.load(os.path.join(GOLDEN, "ipc_types.npz"))
    for l in out.splitlines()[2:]:
        _, name, v = l.split()
        m = ref["valid_" + name]
        assert float(v) == pytest.approx(float(ref[name][m].astype(np.float64).sum()), rel=1e-9), name
    rc, out = run("read", os.path.join(GOLDEN, "ipc_runend.arrow"), "2")
    assert rc == 0, out
    assert out.splitlines()[0] == "type (vector 2 (i64 f64) (runend flat))"


def test_refused_file_throws():
    rc, out = run("read", os.path.join(GOLDEN, "ipc_lz4.arrow"), "1")
    assert rc == 1 and out.startswith("error load_arrow_file:") and "compressed" in out


@pytest.mark.gpu
def test_query_on_loaded_file():
    path = os.path.join(GOLDEN, "ipc_filter_sum.arrow")
    rc, out = run("run", path)
    assert rc == 0, out
    _, s, c = out.split()
    host = table_from_ipc(path, 2)
    ref = loopgen.Query(W.filter_sum_query(host.get_data_type(), 100, 2000))(host)
    assert_same((float(s), int(c)), tuple(ref))
    assert ref[1] > 0
