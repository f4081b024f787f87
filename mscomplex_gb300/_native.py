"""ctypes binding of libdmsc.so (include/dmsc.h).

The library is the only implementation of the hot path: if it is missing or
fails to load, every call raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

DMSC_OK = 0
ERRORS = {
    1: "BAD_ARG", 2: "OOM", 3: "CUDA", 4: "INT16_OVERFLOW", 5: "DEVICE_TIMEOUT",
    6: "INVARIANT", 7: "INPUT", 8: "STATE", 9: "PARTIAL",
}
DMSC_ERR_PARTIAL = 9

# Every extern "C" entry point declared in include/dmsc.h, with its argument types.
_vp, _i64, _i32, _f64 = C.c_void_p, C.c_int64, C.c_int, C.c_double
SIGNATURES = {
    "dmsc_last_error": ([], C.c_char_p),
    "dmsc_init": ([_i32, _vp], _i32),
    "dmsc_shutdown": ([_vp], _i32),
    "dmsc_dataset_create": ([_vp, _vp, _vp, _vp], _i32),
    "dmsc_dataset_destroy": ([_vp], _i32),
    "dmsc_dataset_init": ([_vp, _vp, _i64, _i32, _vp], _i32),
    "dmsc_dataset_work": ([_vp, _vp], _i32),
    "dmsc_dataset_work_ocl": ([_vp, _vp], _i32),
    "dmsc_dataset_num_critical": ([_vp, _vp], _i32),
    "dmsc_dataset_export_cells": ([_vp, _vp, _vp, _vp, _vp], _i32),
    "dmsc_dataset_export_critical": ([_vp, _vp, _vp], _i32),
    "dmsc_dataset_writeout_connectivity": ([_vp, _vp, _vp], _i32),
    "dmsc_dataset_writeout_connectivity_ocl": ([_vp, _vp, _vp], _i32),
    "dmsc_msc_destroy": ([_vp], _i32),
    "dmsc_msc_sizes": ([_vp, _vp], _i32),
    "dmsc_msc_export": ([_vp] * 15, _i32),
    "dmsc_msc_export_async": ([_vp] * 15, _i32),
    "dmsc_set_timing": ([_vp, _i32], _i32),
    "dmsc_dataset_stage_times": ([_vp, _vp, _i32], _i32),
    "dmsc_kernel_launches": ([_vp], _i32),
    "dmsc_msc_simplify_un_simplify": ([_vp, _f64, _i64, _vp], _i32),
    "dmsc_msc_simplify_stats": ([_vp, _vp], _i32),
    "dmsc_dataset_fill_discs": ([_vp, _vp, _vp], _i32),
    "dmsc_msc_write_discs": ([_vp, C.c_char_p], _i32),
    "dmsc_pipeline_run": ([_vp, _vp, _i64, _i32, _i32, _i32, _i32, C.c_double, _i32, _vp, _vp], _i32),
    "dmsc_pipeline_destroy": ([_vp], _i32),
    "dmsc_pipeline_num_pieces": ([_vp, _vp], _i32),
    "dmsc_pipeline_piece": ([_vp, _i64, _vp, _vp], _i32),
    "dmsc_pipeline_write_discs": ([_vp, C.c_char_p], _i32),
    "dmsc_pipeline_stage_times": ([_vp, _vp], _i32),
    "dmsc_batch_run": ([_vp, _i32, _vp, _vp, _i32, _vp, _i64, _vp, _vp], _i32),
    "dmsc_batch_destroy": ([_vp], _i32),
    "dmsc_batch_num_grids": ([_vp, _vp], _i32),
    "dmsc_batch_sizes": ([_vp, _i64, _vp], _i32),
    "dmsc_batch_simplify_stats": ([_vp, _i64, _vp], _i32),
    "dmsc_batch_export": ([_vp, _i64] + [_vp] * 9 + [_vp], _i32),
    "dmsc_batch_totals": ([_vp, _vp], _i32),
    "dmsc_set_merge_parallel_min": ([_vp, _i64], _i32),
    "dmsc_set_merge_rounds": ([_vp, _i64, _i64], _i32),
    "dmsc_set_use_ocl": ([_vp, _i32], _i32),
    "dmsc_set_out_of_core": ([_vp, C.c_char_p], _i32),
    "dmsc_msc_save": ([_vp, C.c_char_p], _i32),
    "dmsc_msc_load": ([_vp, C.c_char_p, _vp], _i32),
    "dmsc_pipeline_merge_times": ([_vp, _vp], _i32),
    "dmsc_pool_stats": ([_vp, _vp], _i32),
    "dmsc_batch_grid_status": ([_vp, _i64, _vp, C.c_char_p, _i32], _i32),
    "dmsc_batch_export_all": ([_vp] + [_vp] * 11 + [_vp], _i32),
    "dmsc_batch_tile_times": ([_vp, _vp], _i32),
    "dmsc_batch_autotune": ([_vp, _i32, _vp, _vp, _i32, _i32, _vp], _i32),
    "dmsc_batch_autotune_reset": ([_vp], _i32),
    "dmsc_batch_set_launch": ([_vp, _i32, _i32, _i32], _i32),
    "dmsc_server_create": ([_vp, _i64, _i32, _i32, _i64, _vp], _i32),
    "dmsc_server_submit": ([_vp, _vp, _i32, _i32, C.c_double, _vp], _i32),
    "dmsc_server_wait": ([_vp, _i64, _i32, _vp, _vp], _i32),
    "dmsc_server_result": ([_vp, _i64, _vp, _vp, C.c_char_p, _i32], _i32),
    "dmsc_server_export": ([_vp, _i64] + [_vp] * 8, _i32),
    "dmsc_server_release": ([_vp, _i64], _i32),
    "dmsc_server_stats": ([_vp, _vp], _i32),
    "dmsc_server_destroy": ([_vp], _i32),
    "dmsc_prefix_scan": ([_vp, _vp, _vp, _i64, _vp, _vp], _i32),
    "dmsc_prefix_scan_noalloc": ([_vp, _vp, _vp, _i64, _vp, _vp], _i32),
    "dmsc_sort_pairs": ([_vp, _vp, _vp, _vp, _vp, C.c_uint32, C.c_uint32, C.c_uint32, _vp], _i32),
}


class DmscError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"dmsc error {ERRORS.get(code, code)}: {msg}")
        self.code = code


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libdmsc.so, building it first when it is missing (needs nvcc)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing:
            path = _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f"libdmsc.so not found at {path}; run mscomplex_gb300.build.build()")
        L = C.CDLL(path)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.argtypes = args
            fn.restype = res
        _lib = L
        return L


def check(rc: int):
    if rc != DMSC_OK:
        raise DmscError(rc, load().dmsc_last_error().decode())


def kernel_launches() -> int:
    n = C.c_uint64()
    check(load().dmsc_kernel_launches(C.byref(n)))
    return n.value
