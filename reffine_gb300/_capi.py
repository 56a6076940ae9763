"""ctypes binding of the C-ABI (include/rf_gpu.h).

The library is built in-tree by ``reffine_gb300.build``; loading fails loudly if it is missing:
there is no CPU fallback behind this module.
"""
from __future__ import annotations

import ctypes
import os

from .table import ArrowArray, ArrowSchema

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "librf_gpu.so")

(RF_OK, RF_ERR_INVALID, RF_ERR_UNSUPPORTED, RF_ERR_CUDA, RF_ERR_JIT, RF_ERR_OOM, RF_ERR_DEVICE, RF_ERR_BUSY,
 RF_ERR_CANCELLED) = range(9)
STATUS_NAMES = {0: "RF_OK", 1: "RF_ERR_INVALID", 2: "RF_ERR_UNSUPPORTED", 3: "RF_ERR_CUDA", 4: "RF_ERR_JIT",
                5: "RF_ERR_OOM", 6: "RF_ERR_DEVICE", 7: "RF_ERR_BUSY", 8: "RF_ERR_CANCELLED"}
RF_SERVE_BATCHED, RF_SERVE_PER_QUERY = 0, 1
RF_ARG_TABLE, RF_ARG_I64, RF_ARG_F64 = 0, 1, 2


class RfArg(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("pad_", ctypes.c_int32), ("table", ctypes.c_void_p),
                ("i64", ctypes.c_int64), ("f64", ctypes.c_double)]


class RfPlanInfo(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("n_inputs", ctypes.c_int32), ("output_is_table", ctypes.c_int32),
                ("n_groups", ctypes.c_int32), ("output_size", ctypes.c_int64),
                ("bytes_per_row", ctypes.c_int64 * 8), ("n_kernels", ctypes.c_int32), ("vectorize", ctypes.c_int32)]


class RfServerConfig(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int32), ("max_batch", ctypes.c_int32), ("lanes", ctypes.c_int32),
                ("queue_capacity", ctypes.c_int32), ("hbm_budget_bytes", ctypes.c_int64),
                ("lane_share_pct", ctypes.c_int32), ("table_lanes", ctypes.c_int32),
                ("table_priority", ctypes.c_int32), ("table_share_pct", ctypes.c_int32)]


class RfCompletion(ctypes.Structure):
    _fields_ = [("tag", ctypes.c_uint64), ("status", ctypes.c_int32), ("batch_queries", ctypes.c_int32),
                ("t_submit_ns", ctypes.c_int64), ("t_launch_ns", ctypes.c_int64), ("t_done_ns", ctypes.c_int64)]


class RfServerStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in (
        "submitted", "completed", "failed", "cancelled", "rejected", "batches", "batched_queries",
        "queue_depth", "max_queue_depth", "inflight_bytes", "peak_inflight_bytes", "inflight_queries")]


# every entry point of include/rf_gpu.h: name -> (restype, argtypes)
P = ctypes.c_void_p
PP = ctypes.POINTER(ctypes.c_void_p)
I = ctypes.c_int
I32 = ctypes.c_int32
I64 = ctypes.c_int64
SIGNATURES = {
    "rf_gpu_init": (I, [I, PP]),
    "rf_gpu_shutdown": (I, [P]),
    "rf_last_error": (ctypes.c_char_p, [P]),
    "rf_ctx_stream": (I, [P, PP]),
    "rf_ctx_sync": (I, [P]),
    "rf_ctx_launch_count": (I, [P, ctypes.POINTER(I64)]),
    "rf_host_alloc": (I, [P, ctypes.c_size_t, PP]),
    "rf_host_free": (I, [P, P]),
    "rf_table_upload": (I, [P, ctypes.POINTER(ArrowSchema), ctypes.POINTER(ArrowArray), I64, P, PP]),
    "rf_table_upload_cols": (I, [P, ctypes.POINTER(ArrowSchema), ctypes.POINTER(ArrowArray), I64,
                                 ctypes.POINTER(I32), I32, P, PP]),
    "rf_table_free": (I, [P]),
    "rf_table_build_index": (I, [P, P]),
    "rf_table_num_rows": (I, [P, ctypes.POINTER(I64)]),
    "rf_table_num_cols": (I, [P, ctypes.POINTER(I32)]),
    "rf_table_column": (I, [P, I32, I32, PP, ctypes.POINTER(I64)]),
    "rf_table_export": (I, [P, ctypes.POINTER(ArrowSchema), ctypes.POINTER(ArrowArray)]),
    "rf_table_null_count": (I, [P, ctypes.POINTER(I64)]),
    "rf_table_describe": (I, [P, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
    "rf_ipc_read": (I, [ctypes.c_char_p, ctypes.POINTER(ArrowSchema), ctypes.POINTER(ArrowArray), ctypes.c_char_p,
                        ctypes.c_size_t]),
    "rf_table_load_ipc": (I, [P, ctypes.c_char_p, I64, P, PP]),
    "rf_plan_compile": (I, [P, ctypes.c_char_p, I, PP]),
    "rf_plan_free": (I, [P]),
    "rf_plan_check": (I, [ctypes.c_char_p, I, ctypes.c_char_p, ctypes.c_size_t]),
    "rf_plan_info": (I, [P, ctypes.POINTER(RfPlanInfo)]),
    "rf_plan_source": (ctypes.c_char_p, [P]),
    "rf_plan_run": (I, [P, ctypes.POINTER(RfArg), I32, P, P]),
    "rf_plan_launch": (I, [P, ctypes.POINTER(RfArg), I32, P, P]),
    "rf_plan_run_noalloc": (I, [P, ctypes.POINTER(RfArg), I32, P, P]),
    "rf_plan_thunk": (I, [P, PP]),
    "rf_batch_create": (I, [P, I32, PP]),
    "rf_batch_free": (I, [P]),
    "rf_batch_add": (I, [P, P, ctypes.POINTER(RfArg), I32, P]),
    "rf_batch_launch": (I, [P, P]),
    "rf_batch_wait": (I, [P]),
    "rf_batch_reset": (I, [P]),
    "rf_batch_poll": (I, [P, ctypes.POINTER(I32)]),
    "rf_clock_ns": (I64, []),
    "rf_plan_tune": (I, [P, ctypes.POINTER(RfArg), I32, I32, ctypes.POINTER(I64), ctypes.POINTER(ctypes.c_double)]),
    "rf_tune_export": (I, [P, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
    "rf_tune_import": (I, [P, ctypes.c_char_p]),
    "rf_server_create": (I, [P, ctypes.POINTER(RfServerConfig), PP]),
    "rf_server_submit": (I, [P, P, ctypes.POINTER(RfArg), I32, P, ctypes.c_uint64]),
    "rf_server_cancel": (I, [P, ctypes.c_uint64]),
    "rf_server_pause": (I, [P, I32]),
    "rf_server_poll": (I, [P, ctypes.POINTER(RfCompletion), I32, ctypes.POINTER(I32), I32]),
    "rf_server_get_stats": (I, [P, ctypes.POINTER(RfServerStats)]),
    "rf_server_free": (I, [P]),
    "rf_server_replay": (I, [P, I32, PP, ctypes.POINTER(ctypes.POINTER(RfArg)), ctypes.POINTER(I32), PP,
                             ctypes.POINTER(I64), ctypes.POINTER(RfCompletion)]),
}

_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("reffine_gb300: %s is not built (run `python -m reffine_gb300.build`); "
                           "the GPU backend has no fallback" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class RfError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), msg))
        self.status = status


def check(status: int, ctx=None, what: str = ""):
    if status != RF_OK:
        msg = load().rf_last_error(ctx).decode(errors="replace") if ctx else what
        raise RfError(status, msg)
