"""Autotuner for batched builds and traversal.

The reference fixes its PLOC search radius per preset (PlocSearchDistance,
src/ploc/mod.rs:534-561) and has no batched form.  For a batch of many
scenes, the radius trades build time against tree quality (traversal time),
so it is chosen here by measurement: a sample of the batch is built with the
segmented builder and its rays traced in one multi-BVH launch for every
candidate radius, and the radius with the lowest build + trace time wins.
The choice changes the trees (a different radius is a different build), so
a caller compares batched and one-scene-per-call results under the tuned
parameters; both forms then give identical hits.
"""
from __future__ import annotations

import dataclasses
import time

import numpy as np

from .params import BvhBuildParams

RADII = (8, 14, 24)


def _sync():
    import torch

    torch.cuda.synchronize()


def tune_segmented(scenes, rays, ray_owner, base: BvhBuildParams, ctx=None, radii=RADII, reps: int = 2):
    """Times build_cwbvh_from_tris_segmented(scenes) + ray_traverse_multi(rays)
    per candidate radius (device tensors: scenes, rays (n, 8) f32 and
    ray_owner (n,) int32 indexing `scenes`).  Returns (params, seconds per
    radius)."""
    from . import bvh

    table = {}
    for r in radii:
        p = dataclasses.replace(base, ploc_search_distance=int(r))
        best = float("inf")
        for _ in range(reps + 1):  # the first round warms up
            _sync()
            t0 = time.perf_counter()
            out = bvh.build_cwbvh_from_tris_segmented(scenes, p, ctx=ctx)
            bvh.ray_traverse_multi(out, ray_owner, rays, ctx=ctx)
            _sync()
            best = min(best, time.perf_counter() - t0)
            for b in out:
                b.free()
        table[int(r)] = best
    choice = min(table, key=table.get)
    return dataclasses.replace(base, ploc_search_distance=int(choice)), table


def sample_indices(sizes, k: int, seed: int = 0) -> np.ndarray:
    """k scenes spread over the size range (every size quantile represented)."""
    order = np.argsort(np.asarray(sizes), kind="stable")
    if k >= len(order):
        return order
    pick = np.linspace(0, len(order) - 1, k).round().astype(int)
    return np.sort(order[pick])
