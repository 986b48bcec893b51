"""GB300-native (sm_103a) BVH hot path of obvhs: PLOC BVH2 build, reinsertion,
spatial pre-splits, BVH2 -> CWBVH8 conversion and CWBVH closest-hit /
occlusion traversal, behind the reference's builder and traversal API.

`params` and `test_util` are plain Python; everything in `bvh` runs on the
GPU through libobvhs_gb300.so (loaded on first use, no CPU fallback).
"""
from .params import PRESETS, BvhBuildParams, PlocSearchDistance, SortPrecision

__all__ = [
    "BvhBuildParams", "PlocSearchDistance", "SortPrecision", "PRESETS", "Context", "Bvh2", "CwBvh", "PlocBuilder",
    "ReinsertionOptimizer", "bvh2_to_cwbvh", "build_cwbvh_from_tris", "build_cwbvh", "split_aabbs_preset",
    "morton_sort", "split_thresholds", "ObvhsError", "build_cwbvh_from_tris_batch", "build_cwbvh_from_tris_segmented",
    "ray_traverse_multi", "ray_traverse_batches", "build_bvh2_from_tris", "build_bvh2",
]


def __getattr__(name):
    if name in ("Context", "Bvh2", "CwBvh", "PlocBuilder", "ReinsertionOptimizer", "bvh2_to_cwbvh",
                "build_cwbvh_from_tris", "build_cwbvh", "split_aabbs_preset", "morton_sort", "BuildStats",
                "split_thresholds", "build_cwbvh_from_tris_batch", "build_cwbvh_from_tris_segmented",
                "ray_traverse_multi", "ray_traverse_batches", "build_bvh2_from_tris", "build_bvh2"):
        from . import bvh

        return getattr(bvh, name)
    if name == "ObvhsError":
        from ._native import ObvhsError

        return ObvhsError
    raise AttributeError(name)
