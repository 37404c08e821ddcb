"""ctypes binding of libfastc_bc7.so (the C ABI declared in include/fastc_bc7.h).

The library is built in-tree by ``fastc_gb300.build``. Loading fails loudly
when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

u8p = C.POINTER(C.c_uint8)

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_UNSUPPORTED = 2
ERR_OUT_OF_MEMORY = 3
ERR_CUDA = 4
ERR_BUDGET = 5
ERR_TIMEOUT = 6
ERR_NOT_FOUND = 7
ERR_CANCELLED = 8
ERR_NO_DEVICE = 9
ERR_INTERNAL = 10


class Settings(C.Structure):
    _fields_ = [
        ("shape_selection_fn", C.c_void_p),
        ("shape_selection_user_data", C.c_void_p),
        ("block_modes", C.c_uint32),
        ("error_metric", C.c_uint32),
        ("steps", C.c_uint32),
        ("seed", C.c_uint32),
        ("watermark_start", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


class Job(C.Structure):
    _fields_ = [
        ("in_", C.c_void_p),
        ("out", C.c_void_p),
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("x_start", C.c_uint32),
        ("y_start", C.c_uint32),
        ("x_end", C.c_uint32),
        ("y_end", C.c_uint32),
    ]


class LogicalBlock(C.Structure):
    _fields_ = [
        ("mode", C.c_uint32), ("shape", C.c_uint32), ("subsets", C.c_uint32),
        ("rotation", C.c_uint32), ("index_mode", C.c_uint32), ("depth", C.c_uint8 * 4),
        ("endpoints", ((C.c_uint8 * 4) * 2) * 3), ("indices", C.c_uint8 * 16),
        ("alpha_indices", C.c_uint8 * 16),
    ]


class BlockStats(C.Structure):
    """fastc_bc7_block_stats: what CompressWithStats logs for one block."""
    _fields_ = [("path", C.c_int32), ("mode", C.c_int32), ("estimate", C.c_double * 8),
                ("error", C.c_double * 8), ("n_two", C.c_int32), ("n_three", C.c_int32),
                ("two_shape", C.c_double * 64), ("three_shape", C.c_double * 64)]


class PlanTuning(C.Structure):
    """fastc_bc7_plan_tuning_info."""
    _fields_ = [("engine", C.c_int32), ("warps_per_cta", C.c_int32), ("anneal_ctas_per_sm", C.c_int32),
                ("yield_lanes", C.c_int32), ("select_ctas_per_sm", C.c_int32),
                ("setup_ctas_per_sm", C.c_int32), ("chunk_blocks", C.c_uint64)]


class ServerConfig(C.Structure):
    _fields_ = [("memory_budget", C.c_size_t), ("max_inflight", C.c_uint32),
                ("max_batch_blocks", C.c_uint32), ("max_batch_jobs", C.c_uint32), ("reserved", C.c_uint32)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("cancelled", C.c_uint64), ("rejected", C.c_uint64), ("batches", C.c_uint64),
                ("pixels_completed", C.c_uint64), ("bytes_in_use", C.c_size_t), ("peak_bytes", C.c_size_t),
                ("p50_latency_ms", C.c_double), ("p99_latency_ms", C.c_double),
                ("mean_latency_ms", C.c_double), ("max_latency_ms", C.c_double), ("mpix_per_s", C.c_double),
                ("psnr_db", C.c_double)]


# Every function include/fastc_bc7.h declares, with its ctypes signature.
SIGNATURES = {
    "fastc_bc7_settings_default": (None, [C.POINTER(Settings)]),
    "fastc_bc7_status_string": (C.c_char_p, [C.c_int]),
    "fastc_bc7_last_error": (C.c_char_p, []),
    "fastc_bc7_abi_version": (C.c_uint32, []),
    "fastc_bc7_job_blocks": (C.c_uint64, [C.POINTER(Job)]),
    "fastc_bc7_compress": (C.c_int, [C.POINTER(Job), C.POINTER(Settings)]),
    "fastc_bc7_compress_batch": (C.c_int, [C.POINTER(Job), C.c_uint32, C.POINTER(Settings), C.c_int]),
    "fastc_bc7_compress_image": (C.c_int, [u8p, C.c_uint32, C.c_uint32, u8p, C.c_size_t,
                                           C.POINTER(Settings)]),
    "fastc_bc7_decompress": (C.c_int, [u8p, u8p, C.c_uint32, C.c_uint32, C.c_int]),
    "fastc_bc7_decode_logical": (C.c_int, [u8p, C.c_size_t, C.POINTER(LogicalBlock)]),
    "fastc_bc7_compress_device": (C.c_int, [C.POINTER(Job), C.c_uint32, C.POINTER(Settings), C.c_int,
                                            C.c_void_p]),
    "fastc_bc7_decompress_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_int,
                                              C.c_void_p]),
    "fastc_bc7_compress_device_noalloc": (C.c_int, [C.POINTER(Job), C.c_uint32, C.POINTER(Settings),
                                                  C.c_int, C.c_void_p]),
    "fastc_bc7_plan_create": (C.c_int, [C.POINTER(Job), C.c_uint32, C.POINTER(Settings), C.c_int,
                                        C.POINTER(C.c_void_p)]),
    "fastc_bc7_plan_launch": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fastc_bc7_plan_flags": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32)]),
    "fastc_bc7_plan_blocks": (C.c_uint64, [C.c_void_p]),
    "fastc_bc7_plan_kernels": (C.c_uint64, [C.c_void_p]),
    "fastc_bc7_plan_autotune": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "fastc_bc7_plan_tuning": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "fastc_bc7_plan_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(PlanTuning)]),
    "fastc_bc7_plan_destroy": (C.c_int, [C.c_void_p]),
    "fastc_bc7_set_watermark_counter": (None, [C.c_uint32]),
    "fastc_bc7_get_watermark_counter": (C.c_uint32, []),
    "fastc_bc7_server_config_default": (None, [C.POINTER(ServerConfig)]),
    "fastc_bc7_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(C.c_void_p)]),
    "fastc_bc7_server_submit": (C.c_int, [C.c_void_p, C.POINTER(Job), C.POINTER(Settings),
                                          C.POINTER(C.c_uint64)]),
    "fastc_dxt_server_submit": (C.c_int, [C.c_void_p, C.POINTER(Job), C.c_int, C.POINTER(C.c_uint64)]),
    "fastc_bc7_server_poll": (C.c_int, [C.c_void_p, C.c_uint64]),
    "fastc_bc7_server_wait": (C.c_int, [C.c_void_p, C.c_uint64, C.c_int64]),
    "fastc_bc7_server_request_psnr": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_double)]),
    "fastc_bc7_server_cancel": (C.c_int, [C.c_void_p, C.c_uint64]),
    "fastc_bc7_server_release": (C.c_int, [C.c_void_p, C.c_uint64]),
    "fastc_bc7_server_get_stats": (C.c_int, [C.c_void_p, C.POINTER(ServerStats)]),
    "fastc_bc7_server_destroy": (C.c_int, [C.c_void_p]),
    "fastc_bc7_compress_stats": (C.c_int, [C.POINTER(Job), C.POINTER(Settings), C.c_void_p]),
    "fastc_bc7_stats_log": (C.c_int, [C.POINTER(Job), C.c_void_p, C.c_char_p, C.c_size_t,
                                      C.POINTER(C.c_size_t)]),
    "fastc_bc7_psnr": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                 C.POINTER(C.c_double), C.c_void_p]),
    "fastc_bc7_block_error_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                               C.c_void_p, C.c_void_p, C.c_void_p]),
    "fastc_dxt_compress": (C.c_int, [C.POINTER(Job), C.c_int]),
    "fastc_dxt_compress_batch": (C.c_int, [C.POINTER(Job), C.c_uint32, C.c_int]),
    "fastc_dxt_compress_device": (C.c_int, [C.POINTER(Job), C.c_uint32, C.c_int, C.c_void_p]),
    "fastc_dxt_decompress": (C.c_int, [u8p, u8p, C.c_uint32, C.c_uint32, C.c_int]),
    "fastc_dxt_decompress_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_int,
                                              C.c_void_p]),
    "fastc_dxt_psnr": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_int,
                                 C.POINTER(C.c_double), C.c_void_p]),
    "fastc_dxt_block_error_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_int,
                                               C.c_void_p, C.c_void_p, C.c_void_p]),
    "fastc_bc7_set_engine": (C.c_int, [C.c_int]),
    "fastc_bc7_get_engine": (C.c_int, []),
    "fastc_bc7_set_launch_shape": (C.c_int, [C.c_int, C.c_int]),
    "fastc_bc7_get_launch_shape": (C.c_int, [C.POINTER(C.c_int), C.POINTER(C.c_int)]),
}

_lock = threading.Lock()
_lib = None


class BC7Error(RuntimeError):
    """A non-OK status from the C ABI."""

    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        msg = f"{where}: {status_string(status)}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (and if needed build) the library; raises if that is impossible."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = lib_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise FileNotFoundError(f"{path} is missing; run python -m fastc_gb300.build")
            _build.build()
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def status_string(st: int) -> str:
    try:
        return load().fastc_bc7_status_string(st).decode()
    except Exception:  # pragma: no cover - only when the library cannot load
        return f"status {st}"


def check(st: int, where: str) -> None:
    if st != OK:
        detail = ""
        if st in (ERR_CUDA, ERR_OUT_OF_MEMORY, ERR_NO_DEVICE):
            detail = load().fastc_bc7_last_error().decode()
        raise BC7Error(st, where, detail)
