"""ctypes binding of libhd_gb300.so (the C ABI declared in include/hd/hd.h).

The library is built in-tree by ``housdorffhdf5cmake_gb300.build``.  Loading
fails loudly when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

HD_OK = 0
HD_EMPTY_MASK = 1
HD_ERR_BAD_ARG = 2
HD_ERR_OOM = 3
HD_ERR_CUDA = 4
HD_ERR_TIMEOUT = 5
HD_ERR_CANCELLED = 6
HD_ERR_ITER_LIMIT = 7
HD_ERR_NOT_READY = 8
HD_ERR_UNSUPPORTED = 9
HD_ERR_BUSY = 10

HD_SE6 = 0
HD_SE18_FORBENCH = 1

# Every entry point of include/hd/hd.h.
EXPORTS = (
    "hd_options_init", "hd_status_string", "hd_version", "hd_context_create", "hd_context_destroy",
    "hd_context_last_error", "hd_context_last_timings", "hd_compute_u8", "hd_compute_u8_device",
    "hd_compute_u8_device_async", "hd_compute_u8_async", "hd_compute_u8_device_pipelined", "hd_pipeline_flush",
    "hd_batch_compute",
    "hd_profile_u8_device", "hd_distance_map_device", "hd_autotune", "hd_server_options_init",
    "hd_server_create", "hd_server_submit", "hd_server_poll", "hd_server_wait", "hd_server_wait_any",
    "hd_server_cancel",
    "hd_server_get_stats", "hd_server_destroy", "hd_compute_u8_device_noalloc", "hd_load_hdf5_bool", "hd_compute_hdf5",
    "hd_free",
)


class HdResult(ctypes.Structure):
    _fields_ = [
        ("hd", ctypes.c_int32),
        ("iterations", ctypes.c_int32),
        ("sum_ab", ctypes.c_uint64),
        ("sum_ba", ctypes.c_uint64),
        ("n_a", ctypes.c_uint64),
        ("n_b", ctypes.c_uint64),
        ("n_a_not_b", ctypes.c_uint64),
        ("n_b_not_a", ctypes.c_uint64),
        ("avg_hd", ctypes.c_double),
        ("status", ctypes.c_int32),
        ("hd_ab", ctypes.c_int32),
        ("hd_ba", ctypes.c_int32),
        ("hd_robust", ctypes.c_int32),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class HdOptions(ctypes.Structure):
    _fields_ = [
        ("brick_x_words", ctypes.c_int32),
        ("brick_z", ctypes.c_int32),
        ("ctas_per_sm", ctypes.c_int32),
        ("max_iterations", ctypes.c_int32),
        ("barrier_timeout_ns", ctypes.c_int64),
        ("percentile", ctypes.c_float),
        ("zero_copy", ctypes.c_int32),
        ("tuning_table", ctypes.c_char_p),
        ("record_timings", ctypes.c_int32),
        ("kernel", ctypes.c_int32),
        ("steps_per_barrier", ctypes.c_int32),
        ("label", ctypes.c_int32),
    ]


class HdTimings(ctypes.Structure):
    _fields_ = [
        ("pack_ms", ctypes.c_float),
        ("setup_ms", ctypes.c_float),
        ("solve_ms", ctypes.c_float),
        ("total_ms", ctypes.c_float),
        ("iterations", ctypes.c_int32),
        ("grid_ctas", ctypes.c_int32),
        ("brick_x_words", ctypes.c_int32),
        ("brick_z", ctypes.c_int32),
        ("kernel", ctypes.c_int32),
        ("steps_per_barrier", ctypes.c_int32),
        ("brick_rows", ctypes.c_int32),
        ("dilation_partitions", ctypes.c_int32),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class HdPairDesc(ctypes.Structure):
    _fields_ = [
        ("a", ctypes.c_void_p),
        ("b", ctypes.c_void_p),
        ("W", ctypes.c_int32),
        ("H", ctypes.c_int32),
        ("D", ctypes.c_int32),
        ("metric", ctypes.c_int32),
        ("on_device", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


class HdServerOptions(ctypes.Structure):
    _fields_ = [
        ("hbm_budget_bytes", ctypes.c_uint64),
        ("max_inflight", ctypes.c_int32),
        ("max_queue", ctypes.c_int32),
        ("tick_iterations", ctypes.c_int32),
        ("metric", ctypes.c_int32),
    ]


class HdServerStats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_uint64),
        ("completed", ctypes.c_uint64),
        ("cancelled", ctypes.c_uint64),
        ("ticks", ctypes.c_uint64),
        ("resident_pairs", ctypes.c_uint64),
        ("waiting_pairs", ctypes.c_uint64),
        ("bytes_in_use", ctypes.c_uint64),
        ("bytes_peak", ctypes.c_uint64),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


_lock = threading.Lock()
_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libhd_gb300.so (building it first if it is absent and nvcc exists)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError(f"{path} is missing: run housdorffhdf5cmake_gb300.build.build()")
            _build.build()
        L = ctypes.CDLL(path)
        vp, i32, u64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint64
        st = ctypes.c_int
        res_p = ctypes.POINTER(HdResult)
        u64p = ctypes.POINTER(ctypes.c_uint64)
        sig = {
            "hd_options_init": (None, [ctypes.POINTER(HdOptions)]),
            "hd_status_string": (ctypes.c_char_p, [st]),
            "hd_version": (ctypes.c_char_p, []),
            "hd_context_create": (st, [ctypes.c_int, ctypes.POINTER(HdOptions), ctypes.POINTER(vp)]),
            "hd_context_destroy": (st, [vp]),
            "hd_context_last_error": (ctypes.c_char_p, [vp]),
            "hd_context_last_timings": (st, [vp, ctypes.POINTER(HdTimings)]),
            "hd_compute_u8": (st, [vp, vp, vp, i32, i32, i32, st, res_p]),
            "hd_compute_u8_device": (st, [vp, vp, vp, i32, i32, i32, st, vp, res_p]),
            "hd_compute_u8_device_async": (st, [vp, vp, vp, i32, i32, i32, st, vp, vp]),
            "hd_compute_u8_async": (st, [vp, vp, vp, i32, i32, i32, st, vp, vp]),
            "hd_compute_u8_device_pipelined": (st, [vp, vp, vp, i32, i32, i32, st, vp, vp]),
            "hd_pipeline_flush": (st, [vp, vp]),
            "hd_batch_compute": (st, [vp, ctypes.POINTER(HdPairDesc), i32, res_p]),
            "hd_profile_u8_device": (st, [vp, vp, vp, i32, i32, i32, st, res_p, u64p, u64p, i32, u64p]),
            "hd_distance_map_device": (st, [vp, vp, vp, i32, i32, i32, st, vp, vp, res_p]),
            "hd_autotune": (st, [vp, ctypes.POINTER(HdPairDesc), i32, i32, ctypes.c_char_p, ctypes.c_size_t]),
            "hd_server_options_init": (None, [ctypes.POINTER(HdServerOptions)]),
            "hd_server_create": (st, [vp, ctypes.POINTER(HdServerOptions), ctypes.POINTER(vp)]),
            "hd_server_submit": (st, [vp, ctypes.POINTER(HdPairDesc), u64p]),
            "hd_server_poll": (st, [vp, u64, res_p]),
            "hd_server_wait": (st, [vp, u64, ctypes.c_int64, res_p]),
            "hd_server_wait_any": (st, [vp, ctypes.c_int64, u64p, res_p]),
            "hd_server_cancel": (st, [vp, u64]),
            "hd_server_get_stats": (st, [vp, ctypes.POINTER(HdServerStats)]),
            "hd_server_destroy": (st, [vp]),
            "hd_compute_u8_device_noalloc": (st, [vp, vp, i32, i32, i32, st, vp, vp]),
            "hd_load_hdf5_bool": (st, [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(vp),
                                       ctypes.POINTER(ctypes.c_size_t)]),
            "hd_compute_hdf5": (st, [vp, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
                                     ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int, res_p]),
            "hd_free": (None, [vp]),
        }
        for name, (restype, argtypes) in sig.items():
            f = getattr(L, name)
            f.restype = restype
            f.argtypes = argtypes
        _lib = L
        return _lib


def status_string(code: int) -> str:
    return load().hd_status_string(int(code)).decode()
