"""The library's crash report (RF_CRASH_TRACE=1): a fatal signal in the process prints the native
frames of the faulting thread, then the handler installed before it runs.  Host only: the child
installs the report through rf_gpu_init with a device index that does not exist (the call fails
before any CUDA context is created) and then reads address 0 on the host."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import ctypes, sys
sys.path.insert(0, %r)
from reffine_gb300 import _capi
lib = _capi.load()
h = ctypes.c_void_p()
assert lib.rf_gpu_init(9999, ctypes.byref(h)) != 0
print("installed", flush=True)
ctypes.string_at(0)
""" % ROOT


def test_fatal_signal_prints_native_frames():
    from reffine_gb300 import build
    build.build()
    env = dict(os.environ, RF_CRASH_TRACE="1", CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "-c", CHILD], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode != 0
    assert "installed" in r.stdout
    assert "reffine_gb300: fatal signal" in r.stderr
    assert "native frames of the faulting thread" in r.stderr
    assert "librf_gpu.so +0x" in r.stderr or "libc" in r.stderr


def test_report_is_off_unless_asked():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    env.pop("RF_CRASH_TRACE", None)
    r = subprocess.run([sys.executable, "-c", CHILD], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode != 0
    assert "reffine_gb300: fatal signal" not in r.stderr
