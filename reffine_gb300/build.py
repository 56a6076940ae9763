"""Builds the backend's shared library in-tree: reffine_gb300/_lib/librf_gpu.so.

Host sources (lowering pass, runtime, thunks) are compiled with g++; the ahead-of-time kernels
with nvcc for sm_103a.  The device headers that NVRTC needs at query-compile time are embedded
into the library as string literals.  Incremental: a unit is recompiled only when a source or
header is newer than its object.  No cmake; runs on x86_64 and aarch64 alike.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
DEVICE = os.path.join(CSRC, "device")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
GEN = os.path.join(BUILD, "gen")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "librf_gpu.so")

CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

HOST_SRCS = ["lower.cpp", "runtime.cpp", "thunks.cpp", "batch.cpp", "server.cpp", "ipc.cpp"]
CUDA_SRCS = ["kernels.cu"]
EMBED = ["rf_device.cuh", "rf_templates.cuh", "rf_params.h"]


def _headers():
    hs = []
    for d in (CSRC, DEVICE, os.path.join(INCLUDE), os.path.join(INCLUDE, "reffine_gb300")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                hs.append(os.path.join(d, f))
    return hs


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths if os.path.exists(p)), default=0.0)


def _embed():
    os.makedirs(GEN, exist_ok=True)
    for name in EMBED:
        src = os.path.join(DEVICE, name)
        dst = os.path.join(GEN, name + ".inc")
        if os.path.exists(dst) and os.path.getmtime(dst) >= os.path.getmtime(src):
            continue
        text = open(src).read()
        assert ')RFSRC"' not in text
        # raw string literals are limited in length by some compilers: split in chunks
        chunks = [text[i:i + 12000] for i in range(0, len(text), 12000)] or [""]
        with open(dst + ".tmp", "w") as f:
            for c in chunks:
                f.write('R"RFSRC(' + c + ')RFSRC"\n')
        os.replace(dst + ".tmp", dst)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def build(verbose: bool = False, force: bool = False) -> str:
    """Compiles and links the library if needed; returns its path."""
    if not os.path.exists(os.path.join(CUDA, "bin", "nvcc")):
        raise RuntimeError("nvcc not found under %s" % CUDA)
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    _embed()
    hdr_time = max(_newest(_headers()), _newest([os.path.join(GEN, n + ".inc") for n in EMBED]))
    incs = ["-I" + INCLUDE, "-I" + CSRC, "-I" + DEVICE, "-I" + GEN, "-I" + os.path.join(CUDA, "include")]
    jobs = []
    objs = []
    for s in HOST_SRCS:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_time):
            jobs.append(["g++", "-std=c++17", "-O2", "-g", "-fPIC", "-Wall", "-Wno-unused-function", *incs,
                         "-c", src, "-o", obj])
    for s in CUDA_SRCS:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_time):
            jobs.append([os.path.join(CUDA, "bin", "nvcc"), "-std=c++17", "-O3", ARCH, "-lineinfo",
                         "-Xcompiler", "-fPIC", "-Xptxas", "-v" if verbose else "-O3", *incs, "-c", src, "-o", obj])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for r in ex.map(_run, jobs):
                if verbose and (r.stdout or r.stderr):
                    print(r.stdout + r.stderr, file=sys.stderr)
    if force or jobs or not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest(objs):
        cudalib = os.path.join(CUDA, "lib64")
        tmp = LIB + ".%d.tmp" % os.getpid()
        _run(["g++", "-shared", "-o", tmp, *objs, "-L" + cudalib, "-Wl,--no-as-needed", "-lcudart", "-lnvrtc",
              "-lnvrtc-builtins", "-Wl,--as-needed", "-Wl,-rpath," + cudalib, "-lpthread", "-ldl"])
        os.replace(tmp, LIB)
    return LIB


def clean():
    shutil.rmtree(BUILD, ignore_errors=True)
    shutil.rmtree(LIBDIR, ignore_errors=True)


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
