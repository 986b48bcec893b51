"""Autotuner for batched builds and traversal.

The reference fixes its PLOC search radius per preset (PlocSearchDistance,
src/ploc/mod.rs:534-561), its traversal stack at 32 entries
(src/cwbvh/mod.rs:60-64), and has no batched form.  For a batch of many
scenes, the radius trades build time against tree quality (traversal time),
so it is chosen here by measurement: a sample of the batch is built with the
segmented builder and its rays traced in one multi-BVH launch for every
candidate radius, and the radius with the lowest build + trace time wins.
The choice changes the trees (a different radius is a different build), so
a caller compares batched and one-scene-per-call results under the tuned
parameters; both forms then give identical hits.

Then, on the trees of the chosen radius, the traversal's launch form: block
size and where each ray's 32-entry group stack lives (local or shared
memory).  Every form gives the same hits, so only time decides; the stack
keeps the reference's 32 entries and clamping in every form.
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
    ray_owner (n,) int32 indexing `scenes`), then the traversal launch forms
    on the chosen radius's trees.  Returns (params, {"radius_s": seconds per
    radius, "traversal": tune_traversal's result}).""" 
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
    params = dataclasses.replace(base, ploc_search_distance=int(choice))
    out = {"radius_s": table}
    ctx_ = ctx or bvh.Context.default()
    built = bvh.build_cwbvh_from_tris_segmented(scenes, params, ctx=ctx_)
    try:
        out["traversal"] = tune_traversal(lambda: bvh.ray_traverse_multi(built, ray_owner, rays, ctx=ctx_), ctx_,
                                          reps=reps)
    finally:
        for b in built:
            b.free()
    return params, out


def tune_traversal(trace, ctx, reps: int = 3, forms=None):
    """Times `trace()` (one traversal call on `ctx`, device work synchronised
    after it) in every traversal launch form; leaves ctx in the default form.
    Returns {"block", "smem_stack", "ms": {"<block><L|S>": best ms}}."""
    from . import bvh

    forms = forms or bvh.Context.TRAVERSAL_CONFIGS
    ms = {}
    try:
        for block, smem in forms:
            ctx.set_traversal_config(block, smem)
            best = float("inf")
            for _ in range(reps + 1):  # the first round warms up
                _sync()
                t0 = time.perf_counter()
                trace()
                _sync()
                best = min(best, time.perf_counter() - t0)
            ms[f"{block}{'S' if smem else 'L'}"] = round(best * 1e3, 4)
    finally:
        ctx.set_traversal_config(0, False)
    key = min(ms, key=ms.get)
    return {"block": int(key[:-1]), "smem_stack": key[-1] == "S", "ms": ms}


def sample_indices(sizes, k: int, seed: int = 0) -> np.ndarray:
    """k scenes spread over the size range (every size quantile represented)."""
    order = np.argsort(np.asarray(sizes), kind="stable")
    if k >= len(order):
        return order
    pick = np.linspace(0, len(order) - 1, k).round().astype(int)
    return np.sort(order[pick])
