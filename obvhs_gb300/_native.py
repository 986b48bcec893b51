"""ctypes binding of libobvhs_gb300.so (declared in include/obvhs_gb300.h).

Loading fails loudly: there is no CPU fallback.  If the shared library is
missing it is compiled with nvcc (obvhs_gb300/build.py).
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

P = ctypes.c_void_p
U32 = ctypes.c_uint32
U64 = ctypes.c_uint64
I32 = ctypes.c_int32
F32 = ctypes.c_float

OBVHS_OK = 0
ERRORS = {
    -1: "invalid argument",
    -2: "CUDA error",
    -3: "out of device memory",
    -4: "bad input",
    -5: "device limit reached",
    -6: "device status set",
    -7: "input larger than the entry point's fixed capacity",
}


class ObvhsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"obvhs error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


class BuildParams(ctypes.Structure):
    _fields_ = [
        ("pre_split", I32),
        ("ploc_search_distance", U32),
        ("search_depth_threshold", U32),
        ("reinsertion_batch_ratio", F32),
        ("post_collapse_reinsertion_batch_ratio_multiplier", F32),
        ("sort_precision", U32),
        ("max_prims_per_leaf", U32),
        ("collapse_traversal_cost", F32),
    ]


class BuildStats(ctypes.Structure):
    _fields_ = [
        ("core_build_ms", ctypes.c_double),
        ("leaf_count", U32),
        ("ploc_passes", U32),
        ("ploc_sum_counts", U64),
        ("reinsertions", U64),
        ("kernel_launches", U64),
        ("stage_ms", ctypes.c_double * 4),
    ]


#: every symbol include/obvhs_gb300.h declares, with (restype, argtypes)
SIGNATURES = {
    "obvhs_ctx_create": (I32, [I32, U64, ctypes.POINTER(P)]),
    "obvhs_ctx_destroy": (I32, [P]),
    "obvhs_ctx_last_error": (ctypes.c_char_p, [P]),
    "obvhs_ctx_stream": (P, [P]),
    "obvhs_ctx_synchronize": (I32, [P]),
    "obvhs_ctx_kernel_launches": (U64, [P]),
    "obvhs_ctx_set_profiling": (I32, [P, I32]),
    "obvhs_ctx_set_shared_gpu": (I32, [P, I32]),
    "obvhs_ctx_set_wait_limit": (I32, [P, U32]),
    "obvhs_ctx_set_output_reserve": (I32, [P, U64]),
    "obvhs_ctx_set_traversal_config": (I32, [P, U32, I32]),
    "obvhs_ctx_profile_report": (I32, [P, P, U64]),
    "obvhs_ploc_build": (I32, [P, P, P, U32, U32, U32, U32, I32, ctypes.POINTER(P), ctypes.POINTER(BuildStats)]),
    "obvhs_bvh2_info": (I32, [P, ctypes.POINTER(U32), ctypes.POINTER(U32), ctypes.POINTER(U32)]),
    "obvhs_bvh2_download": (I32, [P, P, P, P]),
    "obvhs_bvh2_upload": (I32, [P, P, U32, P, U32, U32, ctypes.POINTER(P)]),
    "obvhs_bvh2_free": (I32, [P]),
    "obvhs_reinsertion_run": (I32, [P, P, F32, P, U32, ctypes.POINTER(U64)]),
    "obvhs_split_aabbs_preset": (I32, [P, P, U32, P, P, U32, ctypes.POINTER(U32)]),
    "obvhs_split_thresholds": (I32, [P, P, U32, P]),
    "obvhs_bvh2_collapse": (I32, [P, P, U32, F32]),
    "obvhs_build_bvh2_from_tris": (I32, [P, P, U32, ctypes.POINTER(BuildParams), I32, ctypes.POINTER(P),
                                         ctypes.POINTER(BuildStats)]),
    "obvhs_build_bvh2": (I32, [P, P, U32, ctypes.POINTER(BuildParams), I32, ctypes.POINTER(P),
                               ctypes.POINTER(BuildStats)]),
    "obvhs_bvh2_set_triangles": (I32, [P, P, P, U32, I32]),
    "obvhs_bvh2_ray_traverse": (I32, [P, P, P, U32, P, I32]),
    "obvhs_bvh2_ray_traverse_miss": (I32, [P, P, P, U32, P, I32]),
    "obvhs_bvh2_set_node_aabbs": (I32, [P, P, P, P, U32, I32]),
    "obvhs_bvh2_refit_all": (I32, [P, P]),
    "obvhs_bvh2_full_rebuild": (I32, [P, P, U32, U32, U32]),
    "obvhs_bvh2_partial_rebuild": (I32, [P, P, P, U32, U32, U32, U32, I32]),
    "obvhs_bvh2_query": (I32, [P, P, I32, P, U32, P, U32, P, P, U64, I32]),
    "obvhs_cwbvh_query": (I32, [P, P, I32, P, U32, P, U32, P, P, P, U64, I32]),
    "obvhs_bvh2_to_cwbvh": (I32, [P, P, U32, I32, ctypes.POINTER(P)]),
    "obvhs_bvh2_to_cwbvh_ex": (I32, [P, P, U32, I32, I32, ctypes.POINTER(P)]),
    "obvhs_cwbvh_exact_node_aabbs": (I32, [P, P, P]),
    "obvhs_cwbvh_order_children": (I32, [P, P, P, U32, I32, I32]),
    "obvhs_cwbvh_order_node_children": (I32, [P, P, P, U32, U32, I32, I32]),
    "obvhs_build_cwbvh_from_tris": (I32, [P, P, U32, ctypes.POINTER(BuildParams), I32, ctypes.POINTER(P),
                                          ctypes.POINTER(BuildStats)]),
    "obvhs_build_cwbvh": (I32, [P, P, U32, ctypes.POINTER(BuildParams), I32, ctypes.POINTER(P),
                                ctypes.POINTER(BuildStats)]),
    "obvhs_cwbvh_info": (I32, [P, ctypes.POINTER(U32), ctypes.POINTER(U32), P]),
    "obvhs_cwbvh_download": (I32, [P, P, P, P]),
    "obvhs_cwbvh_upload": (I32, [P, P, U32, P, U32, ctypes.POINTER(P)]),
    "obvhs_cwbvh_set_triangles": (I32, [P, P, P, U32, I32]),
    "obvhs_cwbvh_free": (I32, [P]),
    "obvhs_ray_traverse": (I32, [P, P, P, U32, P, I32]),
    "obvhs_ray_traverse_miss": (I32, [P, P, P, U32, P, I32]),
    "obvhs_ray_traverse_tlas_blas": (I32, [P, P, P, U32, P, U32, P, I32]),
    "obvhs_build_cwbvh_from_tris_batch": (I32, [P, U32, P, P, U32, ctypes.POINTER(BuildParams), I32, P, P]),
    "obvhs_build_cwbvh_from_tris_segmented": (I32, [P, P, P, U32, ctypes.POINTER(BuildParams), I32, P, P]),
    "obvhs_ray_traverse_multi": (I32, [P, P, U32, P, P, U32, P, I32]),
    "obvhs_ray_traverse_batches": (I32, [P, P, U32, U32, P, P, P, P]),
    "obvhs_cwbvh_set_triangles_compressed": (I32, [P, P, P, U32, I32]),
    "obvhs_cwbvh_download_compressed": (I32, [P, P, P]),
    "obvhs_ray_traverse_compressed": (I32, [P, P, P, U32, P, I32]),
    "obvhs_ray_traverse_miss_compressed": (I32, [P, P, P, U32, P, I32]),
    "obvhs_morton_sort": (I32, [P, P, U32, U32, P, P]),
    "obvhs_morton_sort_noalloc": (I32, [P, U32, U32, P, P, P]),
}

_lib = None
_lock = threading.Lock()


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Loads (building if needed) the CUDA library and declares its symbols."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise OSError(f"{path} is not built")
            _build.build()
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib
