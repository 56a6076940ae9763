"""Minimal CUDA runtime access for timing (events on a given stream) through ctypes."""
from __future__ import annotations

import ctypes
import os

_rt = None


def rt():
    global _rt
    if _rt is None:
        for name in ("libcudart.so.13", os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64",
                                                     "libcudart.so.13"), "libcudart.so"):
            try:
                _rt = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if _rt is None:
            raise RuntimeError("libcudart not found")
        _rt.cudaEventCreate.argtypes = [ctypes.POINTER(ctypes.c_void_p)]
        _rt.cudaEventRecord.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        _rt.cudaEventSynchronize.argtypes = [ctypes.c_void_p]
        _rt.cudaEventElapsedTime.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.c_void_p, ctypes.c_void_p]
        _rt.cudaEventDestroy.argtypes = [ctypes.c_void_p]
        _rt.cudaStreamSynchronize.argtypes = [ctypes.c_void_p]
        _rt.cudaMemsetAsync.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p]
        _rt.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
        _rt.cudaFree.argtypes = [ctypes.c_void_p]
    return _rt


def _ok(e, what):
    if e != 0:
        raise RuntimeError("%s failed: cuda error %d" % (what, e))


class Event:
    def __init__(self):
        self.h = ctypes.c_void_p()
        _ok(rt().cudaEventCreate(ctypes.byref(self.h)), "cudaEventCreate")

    def record(self, stream):
        _ok(rt().cudaEventRecord(self.h, ctypes.c_void_p(stream)), "cudaEventRecord")

    def synchronize(self):
        _ok(rt().cudaEventSynchronize(self.h), "cudaEventSynchronize")

    def elapsed_ms(self, end: "Event") -> float:
        f = ctypes.c_float()
        _ok(rt().cudaEventElapsedTime(ctypes.byref(f), self.h, end.h), "cudaEventElapsedTime")
        return f.value

    def __del__(self):
        try:
            rt().cudaEventDestroy(self.h)
        except Exception:
            pass


def stream_sync(stream):
    _ok(rt().cudaStreamSynchronize(ctypes.c_void_p(stream)), "cudaStreamSynchronize")


class DeviceBuffer:
    """Scratch device memory (used to flush L2 between timed steps when inputs fit in L2)."""

    def __init__(self, nbytes: int):
        self.ptr = ctypes.c_void_p()
        _ok(rt().cudaMalloc(ctypes.byref(self.ptr), nbytes), "cudaMalloc")
        self.nbytes = nbytes

    def memset(self, stream, value: int = 0):
        _ok(rt().cudaMemsetAsync(self.ptr, value, self.nbytes, ctypes.c_void_p(stream)), "cudaMemsetAsync")

    def __del__(self):
        try:
            rt().cudaFree(self.ptr)
        except Exception:
            pass
