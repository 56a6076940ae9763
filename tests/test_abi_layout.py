"""The Python mirrors of the C-ABI structs (reffine_gb300/_capi.py) have the layout the header
declares: a C program built against include/rf_gpu.h prints sizeof and offsetof of every field,
and ctypes must agree.  No GPU needed."""
import ctypes
import os
import shutil
import subprocess

import pytest

from reffine_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# ctypes mirror -> C type name in include/rf_gpu.h
STRUCTS = {
    "RfArg": "rf_arg",
    "RfPlanInfo": "rf_plan_info_t",
    "RfServerConfig": "rf_server_config",
    "RfCompletion": "rf_completion",
    "RfServerStats": "rf_server_stats",
}


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_ctypes_mirrors_match_the_header(tmp_path):
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "rf_gpu.h"', "int main(void) {"]
    for py, c in STRUCTS.items():
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (py, c))
        for name, _ in getattr(_capi, py)._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (py, name, c, name))
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for py in STRUCTS:
        cls = getattr(_capi, py)
        assert got[(py, "size")] == ctypes.sizeof(cls), py
        for name, _ in cls._fields_:
            assert got[(py, name)] == getattr(cls, name).offset, (py, name)
