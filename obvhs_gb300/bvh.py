"""Host-side mirror of obvhs's builder and traversal API over the CUDA library.

Names, argument meaning and error behaviour follow the Rust crate:
  PlocBuilder.build / build_ploc            src/ploc/mod.rs:95-251
  ReinsertionOptimizer.run                  src/bvh2/reinsertion.rs:40-57
  split_aabbs_preset                        src/splits.rs:16-34
  bvh2_to_cwbvh                             src/cwbvh/bvh2_to_cwbvh.rs:490-510
  build_cwbvh_from_tris / build_cwbvh       src/cwbvh/builder.rs:20-123
  CwBvh.ray_traverse / ray_traverse_miss    src/cwbvh/mod.rs:169-225
Every call runs on the GPU through libobvhs_gb300.so; there is no CPU path.
Where the reference panics (PlocSearchDistance::from, a leaf with several
primitives, a NaN box) these raise ObvhsError / ValueError.

Arrays are numpy (host) or torch CUDA tensors (device, zero-copy):
  triangles float32 (n, 9); aabbs float32 (n, 6); rays float32 (n, 8) =
  origin xyz, tmin, direction xyz, tmax.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .params import BvhBuildParams, PlocSearchDistance, SortPrecision

INVALID = 0xFFFFFFFF


def _is_cuda_tensor(x) -> bool:
    return hasattr(x, "is_cuda") and hasattr(x, "data_ptr") and bool(x.is_cuda)


def _prep(x, dtype, cols):
    """Returns (pointer, n_rows, device_flag, keepalive)."""
    if _is_cuda_tensor(x):
        import torch

        want = {np.float32: torch.float32, np.uint32: torch.int32}[dtype]
        if x.dtype != want and not (dtype is np.uint32 and x.dtype == torch.int32):
            raise TypeError(f"expected a {want} tensor")
        x = x.contiguous()
        # the tensor's producer ran on torch's current stream; the library's
        # work goes on its own stream
        torch.cuda.current_stream(x.device).synchronize()
        n = x.numel() // cols if cols else x.numel()
        return ctypes.c_void_p(x.data_ptr()), n, 1, x
    a = np.ascontiguousarray(x, dtype=dtype)
    if cols:
        a = a.reshape(-1, cols)
    return a.ctypes.data_as(ctypes.c_void_p), (len(a) if cols else a.size), 0, a


class Context:
    """A CUDA stream plus grow-only scratch buffers on one device (one thread
    at a time), standing in for the reference builders' reusable Vecs."""

    _default = None

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        self.lib = N.load()
        h = ctypes.c_void_p()
        r = self.lib.obvhs_ctx_create(device, hbm_budget_bytes, ctypes.byref(h))
        if r != 0:
            raise N.ObvhsError(r, f"cannot create a context on device {device}")
        self.h = h
        self.device = device

    def close(self):
        """Destroys the context (its stream and scratch buffers)."""
        if getattr(self, "h", None):
            self.lib.obvhs_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @classmethod
    def default(cls) -> "Context":
        if cls._default is None:
            cls._default = Context(0)
        return cls._default

    def check(self, r: int):
        if r != 0:
            msg = self.lib.obvhs_ctx_last_error(self.h)
            raise N.ObvhsError(r, msg.decode() if msg else "")

    def synchronize(self):
        self.check(self.lib.obvhs_ctx_synchronize(self.h))

    @property
    def stream(self) -> int:
        return self.lib.obvhs_ctx_stream(self.h) or 0

    @property
    def kernel_launches(self) -> int:
        return int(self.lib.obvhs_ctx_kernel_launches(self.h))

    def set_profiling(self, enable: bool):
        """Brackets every kernel launch with CUDA events on the context's stream."""
        self.check(self.lib.obvhs_ctx_set_profiling(self.h, int(enable)))

    def set_shared_gpu(self, shared: bool = True):
        """Builds on this context leave most of the GPU to other work (one-block
        PLOC and conflict resolution); results are identical."""
        self.check(self.lib.obvhs_ctx_set_shared_gpu(self.h, int(bool(shared))))

    #: (threads per block, group stack in shared memory) forms of the traversal
    TRAVERSAL_CONFIGS = ((128, False), (64, False), (256, False), (64, True), (128, True))

    def set_traversal_config(self, block: int = 0, smem_stack: bool = False):
        """Launch form of this context's CWBVH traversals: block size and
        where each ray's 32-entry group stack lives (identical results in
        every form; (0, False) is the default (128, local memory))."""
        self.check(self.lib.obvhs_ctx_set_traversal_config(self.h, int(block), int(bool(smem_stack))))

    #: OBVHS_DEFAULT_WAIT_LIMIT in include/obvhs_gb300.h
    DEFAULT_WAIT_LIMIT = 16777216

    def set_wait_limit(self, spins: int = DEFAULT_WAIT_LIMIT):
        """Empty look-back rounds a radix-sort tile waits for earlier tiles
        before it gives up (the build then raises ObvhsError with
        OBVHS_ERR_LIMIT); small values exercise that failure path."""
        self.check(self.lib.obvhs_ctx_set_wait_limit(self.h, int(spins)))

    #: OBVHS_DEFAULT_OUTPUT_RESERVE in include/obvhs_gb300.h
    DEFAULT_OUTPUT_RESERVE = 4 << 30

    def set_output_reserve(self, nbytes: int = DEFAULT_OUTPUT_RESERVE):
        """Bytes of freed BVH output memory (nodes, primitive indices,
        triangles) the device's output pool keeps mapped for later builds;
        memory above it goes back to the device now (0: all that is free)."""
        self.check(self.lib.obvhs_ctx_set_output_reserve(self.h, int(nbytes)))

    def profile_report(self) -> dict:
        """Per-kernel {launches, total_ms, max_ms} since the last report."""
        import json

        buf = ctypes.create_string_buffer(1 << 16)
        self.check(self.lib.obvhs_ctx_profile_report(self.h, buf, len(buf)))
        return json.loads(buf.value.decode())

    def close(self):
        if self.h:
            self.lib.obvhs_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _ctx(ctx):
    return ctx or Context.default()


@dataclass
class BuildStats:
    core_build_ms: float
    leaf_count: int
    ploc_passes: int
    ploc_sum_counts: int
    reinsertions: int
    kernel_launches: int
    stage_ms: tuple = (0.0, 0.0, 0.0, 0.0)  # pre-split, PLOC, reinsertion, conversion

    @staticmethod
    def from_c(s: N.BuildStats) -> "BuildStats":
        return BuildStats(s.core_build_ms, s.leaf_count, s.ploc_passes, s.ploc_sum_counts, s.reinsertions,
                          s.kernel_launches, tuple(s.stage_ms))


class Bvh2:
    """A device-resident binary BVH (src/bvh2/mod.rs:31-85): 32-byte nodes
    (min, prim_count, max, first_index) and primitive_indices."""

    def __init__(self, ctx: Context, handle: ctypes.c_void_p, stats: BuildStats | None = None):
        self.ctx = ctx
        self.h = handle
        self.stats = stats

    def info(self):
        a, b, c = N.U32(), N.U32(), N.U32()
        self.ctx.check(self.ctx.lib.obvhs_bvh2_info(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    @property
    def max_depth(self) -> int:
        return self.info()[2]

    def download(self):
        nn, npr, _ = self.info()
        nodes = np.zeros((nn, 32), np.uint8)
        pidx = np.zeros(npr, np.uint32)
        self.ctx.check(self.ctx.lib.obvhs_bvh2_download(self.ctx.h, self.h, nodes.ctypes.data_as(ctypes.c_void_p),
                                                        pidx.ctypes.data_as(ctypes.c_void_p)))
        return nodes, pidx

    @property
    def nodes(self) -> np.ndarray:
        return self.download()[0]

    @property
    def primitive_indices(self) -> np.ndarray:
        return self.download()[1]

    @staticmethod
    def upload(nodes, primitive_indices, max_depth=96, ctx: Context | None = None) -> "Bvh2":
        ctx = _ctx(ctx)
        nodes = np.ascontiguousarray(nodes, dtype=np.uint8).reshape(-1, 32)
        pidx = np.ascontiguousarray(primitive_indices, dtype=np.uint32)
        h = ctypes.c_void_p()
        ctx.check(ctx.lib.obvhs_bvh2_upload(ctx.h, nodes.ctypes.data_as(ctypes.c_void_p), len(nodes),
                                            pidx.ctypes.data_as(ctypes.c_void_p), len(pidx), max_depth,
                                            ctypes.byref(h)))
        return Bvh2(ctx, h)

    def collapse(self, max_prims: int, traversal_cost: float):
        """collapse (src/bvh2/leaf_collapser.rs:20-199), in place."""
        self.ctx.check(self.ctx.lib.obvhs_bvh2_collapse(self.ctx.h, self.h, int(max_prims), float(traversal_cost)))

    def set_triangles(self, triangles):
        """Attach float (n, 9) triangles (original order) for traversal."""
        p, n, dev, keep = _prep(triangles, np.float32, 9)
        self.ctx.check(self.ctx.lib.obvhs_bvh2_set_triangles(self.ctx.h, self.h, p, n, dev))
        del keep

    def set_node_aabbs(self, node_ids, aabbs):
        """Bvh2Node::set_aabb for the given nodes (e.g. moved leaves)."""
        pi, n, dev, ki = _prep(node_ids, np.uint32, 0)
        pa, na, deva, ka = _prep(aabbs, np.float32, 6)
        if na != n or deva != dev:
            raise ValueError("one box per node id, same memory space")
        self.ctx.check(self.ctx.lib.obvhs_bvh2_set_node_aabbs(self.ctx.h, self.h, pi, pa, n, dev))
        del ki, ka

    def aabb_query(self, boxes, prim_aabbs=None):
        """Bvh2::aabb_traverse for (n, 6) query boxes: per box the original ids
        of the reached leaves' primitives in traversal order (only those whose
        box intersects, when prim_aabbs is given)."""
        return _query(self, self.ctx.lib.obvhs_bvh2_query, "aabb", boxes, prim_aabbs, [])

    def point_query(self, points, prim_aabbs=None):
        """Bvh2::point_traverse for (n, 3) points."""
        return _query(self, self.ctx.lib.obvhs_bvh2_query, "point", points, prim_aabbs, [])

    def refit_all(self):
        """Bvh2::refit_all (src/bvh2/mod.rs:527-570)."""
        self.ctx.check(self.ctx.lib.obvhs_bvh2_refit_all(self.ctx.h, self.h))

    def full_rebuild(self, search_distance, sort_precision=0, search_depth_threshold=0):
        """PlocBuilder::full_rebuild (src/ploc/rebuild.rs:53-81)."""
        self.ctx.check(self.ctx.lib.obvhs_bvh2_full_rebuild(self.ctx.h, self.h, int(search_distance),
                                                            int(sort_precision), int(search_depth_threshold)))

    def partial_rebuild(self, leaves, search_distance, sort_precision=0, search_depth_threshold=0):
        """compute_rebuild_path_flags(leaves) + PlocBuilder::partial_rebuild
        (src/ploc/rebuild.rs:12-134); `leaves` are leaf node ids."""
        pl, n, dev, keep = _prep(leaves, np.uint32, 0)
        self.ctx.check(self.ctx.lib.obvhs_bvh2_partial_rebuild(self.ctx.h, self.h, pl, n, int(search_distance),
                                                               int(sort_precision), int(search_depth_threshold),
                                                               dev))
        del keep

    def ray_traverse(self, rays, out=None):
        """Closest hit per ray (Bvh2::ray_traverse with Triangle::intersect):
        (original ids, 0xffffffff = miss; t, +inf = miss), or an int32 (n, 2)
        tensor for device rays."""
        out = CwBvh._trav(self, rays, out, self.ctx.lib.obvhs_bvh2_ray_traverse, 8)
        if _is_cuda_tensor(out):
            return out.view(-1, 2)
        o = out.reshape(-1, 2)
        return o[:, 0].copy(), o[:, 1].copy().view(np.float32)

    def ray_traverse_miss(self, rays, out=None):
        """True where the ray hits nothing (Bvh2::ray_traverse_miss)."""
        out = CwBvh._trav(self, rays, out, self.ctx.lib.obvhs_bvh2_ray_traverse_miss, 1)
        if _is_cuda_tensor(out):
            return out
        return out.astype(bool)

    def free(self):
        if self.h:
            self.ctx.lib.obvhs_bvh2_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class PlocBuilder:
    """PLOC BVH2 builder (src/ploc/mod.rs:34-251).  Scratch lives in the context."""

    def __init__(self, ctx: Context | None = None):
        self.ctx = _ctx(ctx)

    @staticmethod
    def with_capacity(prim_count: int, ctx: Context | None = None) -> "PlocBuilder":
        return PlocBuilder(ctx)

    def build(self, search_distance, aabbs, indices=None, sort_precision=SortPrecision.U64,
              search_depth_threshold: int = 0) -> Bvh2:
        """`search_distance` is a PlocSearchDistance (radius 1, 2, 6, 14, 24, 32)."""
        sd = PlocSearchDistance(int(search_distance))
        return self.build_ploc(int(sd), aabbs, indices, sort_precision, search_depth_threshold)

    def build_ploc(self, search_distance: int, aabbs, indices=None, sort_precision=SortPrecision.U64,
                   search_depth_threshold: int = 0) -> Bvh2:
        """build_ploc::<SEARCH_DISTANCE>: any radius 1..=32."""
        if not 1 <= int(search_distance) <= 32:
            raise ValueError("SEARCH_DISTANCE should be <= 32")
        ctx = self.ctx
        pa, n, dev, keep_a = _prep(aabbs, np.float32, 6)
        if indices is not None:
            pi, ni, devi, keep_i = _prep(indices, np.uint32, 0)
            if ni != n or devi != dev:
                raise ValueError("indices must match aabbs in length and memory space")
        else:
            pi, keep_i = None, None
        h = ctypes.c_void_p()
        st = N.BuildStats()
        ctx.check(ctx.lib.obvhs_ploc_build(ctx.h, pa, pi, n, int(search_distance), int(sort_precision),
                                           int(search_depth_threshold), dev, ctypes.byref(h), ctypes.byref(st)))
        del keep_a, keep_i
        return Bvh2(ctx, h, BuildStats.from_c(st))


class ReinsertionOptimizer:
    """Parallel reinsertion (src/bvh2/reinsertion.rs:24-57)."""

    def run(self, bvh: Bvh2, batch_size_ratio: float, ratio_sequence=None) -> int:
        ctx = bvh.ctx
        applied = N.U64()
        if ratio_sequence is None:
            ctx.check(ctx.lib.obvhs_reinsertion_run(ctx.h, bvh.h, float(batch_size_ratio), None, 0,
                                                    ctypes.byref(applied)))
        else:
            seq = np.ascontiguousarray(ratio_sequence, dtype=np.float32)
            ctx.check(ctx.lib.obvhs_reinsertion_run(ctx.h, bvh.h, float(batch_size_ratio),
                                                    seq.ctypes.data_as(ctypes.c_void_p), len(seq),
                                                    ctypes.byref(applied)))
        return int(applied.value)


def split_aabbs_preset(triangles, ctx: Context | None = None):
    """Triangle AABBs with large triangles split (src/splits.rs:16-34): returns
    (aabbs (m, 6), indices (m,))."""
    ctx = _ctx(ctx)
    t = np.ascontiguousarray(triangles, dtype=np.float32).reshape(-1, 9)
    m = N.U32()
    cap = max(len(t) * 2, 16)
    while True:
        a = np.zeros((cap, 6), np.float32)
        ix = np.zeros(cap, np.uint32)
        r = ctx.lib.obvhs_split_aabbs_preset(ctx.h, t.ctypes.data_as(ctypes.c_void_p), len(t),
                                             a.ctypes.data_as(ctypes.c_void_p), ix.ctypes.data_as(ctypes.c_void_p),
                                             cap, ctypes.byref(m))
        if r == -1 and m.value > cap:
            cap = m.value
            continue
        ctx.check(r)
        return a[: m.value].copy(), ix[: m.value].copy()


def split_thresholds(triangles, ctx: Context | None = None):
    """(area_thresh_low, area_thresh_high, avg_half_area, largest_half_area,
    sequential f32 sum, blocks summed element by element) as
    build_cwbvh_from_tris computes them (src/cwbvh/builder.rs:31-43)."""
    ctx = _ctx(ctx)
    t = np.ascontiguousarray(triangles, dtype=np.float32).reshape(-1, 9)
    out = np.zeros(6, np.float32)
    ctx.check(ctx.lib.obvhs_split_thresholds(ctx.h, t.ctypes.data_as(ctypes.c_void_p), len(t),
                                             out.ctypes.data_as(ctypes.c_void_p)))
    return out


class CwBvh:
    """A device-resident compressed wide BVH8 (src/cwbvh/mod.rs:43-55):
    80-byte nodes and primitive_indices, plus the triangles used by the
    traversal calls (Triangle::intersect is the fixed intersection closure)."""

    def __init__(self, ctx: Context, handle: ctypes.c_void_p, stats: BuildStats | None = None):
        self.ctx = ctx
        self.h = handle
        self.stats = stats

    def info(self):
        a, b = N.U32(), N.U32()
        box = np.zeros(6, np.float32)
        self.ctx.check(self.ctx.lib.obvhs_cwbvh_info(self.h, ctypes.byref(a), ctypes.byref(b),
                                                     box.ctypes.data_as(ctypes.c_void_p)))
        return a.value, b.value, box

    @property
    def total_aabb(self) -> np.ndarray:
        return self.info()[2]

    def download(self):
        nn, npr, _ = self.info()
        nodes = np.zeros((nn, 80), np.uint8)
        pidx = np.zeros(npr, np.uint32)
        self.ctx.check(self.ctx.lib.obvhs_cwbvh_download(self.ctx.h, self.h, nodes.ctypes.data_as(ctypes.c_void_p),
                                                         pidx.ctypes.data_as(ctypes.c_void_p)))
        return nodes, pidx

    @property
    def nodes(self) -> np.ndarray:
        return self.download()[0]

    @property
    def primitive_indices(self) -> np.ndarray:
        return self.download()[1]

    @staticmethod
    def upload(nodes, primitive_indices, ctx: Context | None = None) -> "CwBvh":
        ctx = _ctx(ctx)
        nodes = np.ascontiguousarray(nodes, dtype=np.uint8).reshape(-1, 80)
        pidx = np.ascontiguousarray(primitive_indices, dtype=np.uint32)
        h = ctypes.c_void_p()
        ctx.check(ctx.lib.obvhs_cwbvh_upload(ctx.h, nodes.ctypes.data_as(ctypes.c_void_p), len(nodes),
                                             pidx.ctypes.data_as(ctypes.c_void_p), len(pidx), ctypes.byref(h)))
        return CwBvh(ctx, h)

    def aabb_query(self, boxes, prim_aabbs=None, direction=None):
        """The traverse! loop with CwBvhNode::intersect_aabb for (n, 6) query
        boxes: per box the original ids of the reached primitives in traversal
        order (filtered by their boxes when prim_aabbs is given)."""
        d = None if direction is None else np.ascontiguousarray(direction, dtype=np.float32)
        keep = d
        return _query(self, self.ctx.lib.obvhs_cwbvh_query, "aabb", boxes, prim_aabbs,
                      [None if keep is None else keep.ctypes.data_as(ctypes.c_void_p)])

    def point_query(self, points, prim_aabbs=None, direction=None):
        """The traverse! loop with CwBvhNode::contains_point for (n, 3) points."""
        d = None if direction is None else np.ascontiguousarray(direction, dtype=np.float32)
        keep = d
        return _query(self, self.ctx.lib.obvhs_cwbvh_query, "point", points, prim_aabbs,
                      [None if keep is None else keep.ctypes.data_as(ctypes.c_void_p)])

    def exact_node_aabbs(self):
        """CwBvh::exact_node_aabbs: (n_nodes, 6) float32 (min xyz, max xyz), or
        None when the CWBVH was built without them."""
        nn, _, _ = self.info()
        out = np.zeros((nn, 6), np.float32)
        r = self.ctx.lib.obvhs_cwbvh_exact_node_aabbs(self.ctx.h, self.h, out.ctypes.data_as(ctypes.c_void_p))
        if r == -1 and nn:  # invalid argument: built without exact boxes
            return None
        self.ctx.check(r)
        return out

    def order_children(self, prim_aabbs, direct_layout: bool = False):
        """CwBvh::order_children (src/cwbvh/mod.rs:520-524): prim_aabbs are the
        primitives' boxes (n, 6), in primitive_indices order if direct_layout."""
        pa, n, dev, keep = _prep(prim_aabbs, np.float32, 6)
        self.ctx.check(self.ctx.lib.obvhs_cwbvh_order_children(self.ctx.h, self.h, pa, n, int(direct_layout), dev))
        del keep

    def order_node_children(self, prim_aabbs, node_index: int, direct_layout: bool = False):
        """CwBvh::order_node_children (src/cwbvh/mod.rs:537-735) for one node."""
        pa, n, dev, keep = _prep(prim_aabbs, np.float32, 6)
        self.ctx.check(self.ctx.lib.obvhs_cwbvh_order_node_children(self.ctx.h, self.h, pa, n, int(node_index),
                                                                    int(direct_layout), dev))
        del keep

    def set_triangles(self, triangles):
        p, n, dev, keep = _prep(triangles, np.float32, 9)
        self.ctx.check(self.ctx.lib.obvhs_cwbvh_set_triangles(self.ctx.h, self.h, p, n, dev))
        if dev:
            self.ctx.synchronize()
        del keep
        return self

    def _trav(self, rays, out, fn, width):
        pr, n, dev, keep = _prep(rays, np.float32, 8)
        ctx = self.ctx
        if out is None:
            if dev:
                import torch

                out = torch.empty(n * width // 4 if width >= 4 else n, dtype=torch.int32 if width >= 4 else torch.uint8,
                                  device=rays.device)
            else:
                out = np.zeros(n * width // 4 if width >= 4 else n, np.uint32 if width >= 4 else np.uint8)
        po = ctypes.c_void_p(out.data_ptr()) if dev else out.ctypes.data_as(ctypes.c_void_p)
        ctx.check(fn(ctx.h, self.h, pr, n, po, dev))
        if dev:
            ctx.synchronize()
        del keep
        return out

    def ray_traverse(self, rays, out=None):
        """Closest hit per ray (CwBvh::ray_traverse with Triangle::intersect).

        Host rays: returns (primitive_id uint32 (original ids, 0xffffffff =
        miss), t float32 (+inf = miss)).  Device rays: returns an int32 tensor
        of shape (n, 2) holding (id, t bits)."""
        out = self._trav(rays, out, self.ctx.lib.obvhs_ray_traverse, 8)
        if _is_cuda_tensor(out):
            return out.view(-1, 2)
        o = out.reshape(-1, 2)
        return o[:, 0].copy(), o[:, 1].copy().view(np.float32)

    def ray_traverse_miss(self, rays, out=None):
        """True where the ray hits nothing in [tmin, tmax] (CwBvh::ray_traverse_miss)."""
        out = self._trav(rays, out, self.ctx.lib.obvhs_ray_traverse_miss, 1)
        if _is_cuda_tensor(out):
            return out
        return out.astype(bool)

    def set_triangles_compressed(self, triangles):
        """Attach RtCompressedTriangle records (src/rt_triangle.rs:13-47) built
        from float (n, 9) triangles in original order."""
        p, n, dev, keep = _prep(triangles, np.float32, 9)
        self.ctx.check(self.ctx.lib.obvhs_cwbvh_set_triangles_compressed(self.ctx.h, self.h, p, n, dev))
        del keep

    def download_compressed(self) -> np.ndarray:
        """The attached RtCompressedTriangle records, (n_prims, 24) bytes."""
        _, npr, _ = self.info()
        out = np.zeros((npr, 24), np.uint8)
        self.ctx.check(self.ctx.lib.obvhs_cwbvh_download_compressed(self.ctx.h, self.h,
                                                                    out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def ray_traverse_compressed(self, rays, out=None):
        """ray_traverse with RtCompressedTriangle::intersect (see ray_traverse)."""
        out = self._trav(rays, out, self.ctx.lib.obvhs_ray_traverse_compressed, 8)
        if _is_cuda_tensor(out):
            return out.view(-1, 2)
        o = out.reshape(-1, 2)
        return o[:, 0].copy(), o[:, 1].copy().view(np.float32)

    def ray_traverse_miss_compressed(self, rays, out=None):
        """ray_traverse_miss with RtCompressedTriangle::intersect."""
        out = self._trav(rays, out, self.ctx.lib.obvhs_ray_traverse_miss_compressed, 1)
        if _is_cuda_tensor(out):
            return out
        return out.astype(bool)

    def ray_traverse_tlas_blas(self, blas, rays, out=None):
        """CwBvh::ray_traverse_tlas_blas (src/cwbvh/mod.rs:342-491): this CWBVH
        is the TLAS over instance boxes, its primitive_indices index `blas`
        (a sequence of CwBvh with triangles).  Host rays: returns
        (geometry_id, primitive_id (BVH order in that BLAS), original_id, t);
        device rays: an int32 tensor of shape (n, 4) with t as bits."""
        pr, n, dev, keep = _prep(rays, np.float32, 8)
        ctx = self.ctx
        arr = (ctypes.c_void_p * max(len(blas), 1))(*[b.h for b in blas])
        if out is None:
            if dev:
                import torch

                out = torch.empty((n, 4), dtype=torch.int32, device=rays.device)
            else:
                out = np.zeros((n, 4), np.uint32)
        po = ctypes.c_void_p(out.data_ptr()) if dev else out.ctypes.data_as(ctypes.c_void_p)
        ctx.check(ctx.lib.obvhs_ray_traverse_tlas_blas(ctx.h, self.h, ctypes.cast(arr, ctypes.c_void_p), len(blas), pr,
                                                       n, po, dev))
        if dev:
            ctx.synchronize()
            return out
        del keep
        return out[:, 0].copy(), out[:, 1].copy(), out[:, 2].copy(), out[:, 3].copy().view(np.float32)

    def free(self):
        if self.h:
            self.ctx.lib.obvhs_cwbvh_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def bvh2_to_cwbvh(bvh2: Bvh2, max_prims_per_leaf: int, order_children: bool,
                  include_exact_node_aabbs: bool = False) -> CwBvh:
    """bvh2_to_cwbvh (src/cwbvh/bvh2_to_cwbvh.rs:490-510); with
    include_exact_node_aabbs the result keeps each node's exact BVH2 box
    (CwBvh.exact_node_aabbs)."""
    if not 1 <= max_prims_per_leaf <= 3:
        raise ValueError("max_prims_per_leaf must be 1..=3")
    ctx = bvh2.ctx
    h = ctypes.c_void_p()
    ctx.check(ctx.lib.obvhs_bvh2_to_cwbvh_ex(ctx.h, bvh2.h, max_prims_per_leaf, int(order_children),
                                             int(bool(include_exact_node_aabbs)), ctypes.byref(h)))
    return CwBvh(ctx, h)


def build_cwbvh_from_tris_segmented(scenes, config: BvhBuildParams, ctx: Context | None = None) -> list:
    """Many scenes built together: every stage of the build runs once for all
    of them (segmented sorts, one cooperative PLOC launch, reinsertion and
    CWBVH launches that cover every scene).  Each result is byte-identical to
    building that scene alone; the results share one device allocation."""
    ctx = _ctx(ctx)
    preps = [_prep(t, np.float32, 9) for t in scenes]
    devs = {p[2] for p in preps}
    if len(devs) > 1:
        raise ValueError("scenes must all be host arrays or all device tensors")
    dev = devs.pop() if devs else 0
    n = len(preps)
    ptrs = (ctypes.c_void_p * max(n, 1))(*[p[0].value if isinstance(p[0], ctypes.c_void_p) else p[0] for p in preps])
    counts = (ctypes.c_uint32 * max(n, 1))(*[p[1] for p in preps])
    outs = (ctypes.c_void_p * max(n, 1))()
    stats = (N.BuildStats * max(n, 1))()
    prm = _params(config)
    ctx.check(ctx.lib.obvhs_build_cwbvh_from_tris_segmented(ctx.h, ctypes.cast(ptrs, ctypes.c_void_p),
                                                            ctypes.cast(counts, ctypes.c_void_p), n,
                                                            ctypes.byref(prm), dev, ctypes.cast(outs, ctypes.c_void_p),
                                                            ctypes.cast(stats, ctypes.c_void_p)))
    del preps
    return [CwBvh(ctx, ctypes.c_void_p(outs[i]), BuildStats.from_c(stats[i])) for i in range(n)]


def build_cwbvh_from_tris_batch(scenes, config: BvhBuildParams, contexts=None) -> list:
    """Many independent build_cwbvh_from_tris calls at once.  Without
    `contexts`: the segmented build (build_cwbvh_from_tris_segmented).  With
    `contexts`: they work concurrently (one host thread and CUDA stream each),
    largest scenes first.  Each result is byte-identical to building that
    scene alone."""
    if contexts is None:
        return build_cwbvh_from_tris_segmented(scenes, config)
    contexts = list(contexts)
    if not contexts:
        raise ValueError("at least one context")
    ctx = contexts[0]
    preps = [_prep(t, np.float32, 9) for t in scenes]
    devs = {p[2] for p in preps}
    if len(devs) > 1:
        raise ValueError("scenes must all be host arrays or all device tensors")
    dev = devs.pop() if devs else 0
    n = len(preps)
    ptrs = (ctypes.c_void_p * max(n, 1))(*[p[0].value if isinstance(p[0], ctypes.c_void_p) else p[0] for p in preps])
    counts = (ctypes.c_uint32 * max(n, 1))(*[p[1] for p in preps])
    outs = (ctypes.c_void_p * max(n, 1))()
    stats = (N.BuildStats * max(n, 1))()
    ctxs = (ctypes.c_void_p * len(contexts))(*[c.h.value for c in contexts])
    prm = _params(config)
    ctx.check(ctx.lib.obvhs_build_cwbvh_from_tris_batch(ctypes.cast(ctxs, ctypes.c_void_p), len(contexts),
                                                        ctypes.cast(ptrs, ctypes.c_void_p),
                                                        ctypes.cast(counts, ctypes.c_void_p), n, ctypes.byref(prm),
                                                        dev, ctypes.cast(outs, ctypes.c_void_p),
                                                        ctypes.cast(stats, ctypes.c_void_p)))
    if dev:
        for c in contexts:
            c.synchronize()
    del preps
    return [CwBvh(ctx, ctypes.c_void_p(outs[i]), BuildStats.from_c(stats[i])) for i in range(n)]


def ray_traverse_multi(bvhs, ray_bvh, rays, ctx: Context | None = None, out=None):
    """Closest hits of rays against several CWBVHs in one launch: ray i is
    traced in bvhs[ray_bvh[i]].  Host rays: (primitive_id, t) as
    CwBvh.ray_traverse; device rays: an int32 (n, 2) tensor."""
    ctx = _ctx(ctx)
    pr, n, dev, keep = _prep(rays, np.float32, 8)
    pb, nb, devb, keepb = _prep(ray_bvh, np.uint32, 0)
    if nb != n or devb != dev:
        raise ValueError("ray_bvh must match rays in length and memory space")
    arr = (ctypes.c_void_p * max(len(bvhs), 1))(*[b.h.value if isinstance(b.h, ctypes.c_void_p) else b.h for b in bvhs])
    if out is None:
        if dev:
            import torch

            out = torch.empty((n, 2), dtype=torch.int32, device=rays.device)
        else:
            out = np.zeros((n, 2), np.uint32)
    po = ctypes.c_void_p(out.data_ptr()) if dev else out.ctypes.data_as(ctypes.c_void_p)
    ctx.check(ctx.lib.obvhs_ray_traverse_multi(ctx.h, ctypes.cast(arr, ctypes.c_void_p), len(bvhs), pb, pr, n, po, dev))
    if dev:
        ctx.synchronize()
        return out
    del keep, keepb
    return out[:, 0].copy(), out[:, 1].copy().view(np.float32)


def ray_traverse_batches(bvhs, batch_bvh, rays, outs=None, ctx: Context | None = None):
    """Closest hits of several host ray batches in one launch: batch b traced
    in bvhs[batch_bvh[b]].  Returns one (n_b, 2) uint32 array per batch
    (primitive id, t bits), or fills `outs` (preallocated, e.g. in pinned
    memory).  Equal to CwBvh.ray_traverse of each batch alone."""
    ctx = _ctx(ctx)
    nb = len(rays)
    arrs = [np.ascontiguousarray(r, dtype=np.float32).reshape(-1, 8) for r in rays]
    if outs is None:
        outs = [np.zeros((len(a), 2), np.uint32) for a in arrs]
    for a, o in zip(arrs, outs):
        if o.shape != (len(a), 2) or o.dtype != np.uint32 or not o.flags.c_contiguous:
            raise ValueError("each output must be a contiguous (n, 2) uint32 array")
    harr = (ctypes.c_void_p * max(len(bvhs), 1))(*[b.h.value if isinstance(b.h, ctypes.c_void_p) else b.h for b in bvhs])
    idx = np.ascontiguousarray(batch_bvh, dtype=np.uint32)
    if len(idx) != nb:
        raise ValueError("one BVH index per batch")
    counts = np.array([len(a) for a in arrs], np.uint32)
    rp = (ctypes.c_void_p * max(nb, 1))(*[a.ctypes.data for a in arrs])
    op = (ctypes.c_void_p * max(nb, 1))(*[o.ctypes.data for o in outs])
    ctx.check(ctx.lib.obvhs_ray_traverse_batches(ctx.h, ctypes.cast(harr, ctypes.c_void_p), len(bvhs), nb,
                                                 idx.ctypes.data_as(ctypes.c_void_p), ctypes.cast(rp, ctypes.c_void_p),
                                                 counts.ctypes.data_as(ctypes.c_void_p),
                                                 ctypes.cast(op, ctypes.c_void_p)))
    return outs


def _query(obj, fn, kind, queries, prim_aabbs, extra):
    """Two calls of an obvhs_*_query entry (sizes, then ids): a list of uint32
    arrays of original primitive ids, one per query."""
    k = 0 if kind == "aabb" else 1
    q = np.ascontiguousarray(queries, dtype=np.float32).reshape(-1, 6 if k == 0 else 3)
    pa = None if prim_aabbs is None else np.ascontiguousarray(prim_aabbs, dtype=np.float32).reshape(-1, 6)
    n = len(q)
    off = np.zeros(n + 1, np.uint32)
    args = [obj.ctx.h, obj.h, k, q.ctypes.data_as(ctypes.c_void_p), n,
            None if pa is None else pa.ctypes.data_as(ctypes.c_void_p), 0 if pa is None else len(pa)] + extra
    obj.ctx.check(fn(*args, off.ctypes.data_as(ctypes.c_void_p), None, 0, 0))
    ids = np.zeros(max(int(off[n]), 1), np.uint32)
    obj.ctx.check(fn(*args, off.ctypes.data_as(ctypes.c_void_p), ids.ctypes.data_as(ctypes.c_void_p), len(ids), 0))
    return [ids[int(off[i]):int(off[i + 1])].copy() for i in range(n)]


def _params(p: BvhBuildParams) -> N.BuildParams:
    return N.BuildParams(int(bool(p.pre_split)), int(p.ploc_search_distance), int(p.search_depth_threshold),
                         float(p.reinsertion_batch_ratio), float(p.post_collapse_reinsertion_batch_ratio_multiplier),
                         int(p.sort_precision), int(p.max_prims_per_leaf), float(p.collapse_traversal_cost))


def build_cwbvh_from_tris(triangles, config: BvhBuildParams, ctx: Context | None = None) -> CwBvh:
    """src/cwbvh/builder.rs:20-85.  The result carries `stats.core_build_ms`
    (the reference returns it through `&mut Duration`)."""
    ctx = _ctx(ctx)
    p, n, dev, keep = _prep(triangles, np.float32, 9)
    h = ctypes.c_void_p()
    st = N.BuildStats()
    prm = _params(config)
    ctx.check(ctx.lib.obvhs_build_cwbvh_from_tris(ctx.h, p, n, ctypes.byref(prm), dev, ctypes.byref(h),
                                                  ctypes.byref(st)))
    if dev:
        ctx.synchronize()
    del keep
    return CwBvh(ctx, h, BuildStats.from_c(st))


def build_bvh2_from_tris(triangles, config: BvhBuildParams, ctx: Context | None = None) -> Bvh2:
    """src/bvh2/builder.rs:16-91: pre-splits, PLOC, reinsertion, collapse,
    reinsertion; the triangles attached for Bvh2.ray_traverse."""
    ctx = _ctx(ctx)
    p, n, dev, keep = _prep(triangles, np.float32, 9)
    h = ctypes.c_void_p()
    st = N.BuildStats()
    prm = _params(config)
    ctx.check(ctx.lib.obvhs_build_bvh2_from_tris(ctx.h, p, n, ctypes.byref(prm), dev, ctypes.byref(h),
                                                 ctypes.byref(st)))
    del keep
    return Bvh2(ctx, h, BuildStats.from_c(st))


def build_bvh2(aabbs, config: BvhBuildParams, ctx: Context | None = None) -> Bvh2:
    """src/bvh2/builder.rs:103-138 (pre_split is ignored)."""
    ctx = _ctx(ctx)
    p, n, dev, keep = _prep(aabbs, np.float32, 6)
    h = ctypes.c_void_p()
    st = N.BuildStats()
    prm = _params(config)
    ctx.check(ctx.lib.obvhs_build_bvh2(ctx.h, p, n, ctypes.byref(prm), dev, ctypes.byref(h), ctypes.byref(st)))
    del keep
    return Bvh2(ctx, h, BuildStats.from_c(st))


def build_cwbvh(aabbs, config: BvhBuildParams, ctx: Context | None = None) -> CwBvh:
    """src/cwbvh/builder.rs:97-123 (pre_split is ignored)."""
    ctx = _ctx(ctx)
    p, n, dev, keep = _prep(aabbs, np.float32, 6)
    h = ctypes.c_void_p()
    st = N.BuildStats()
    prm = _params(config)
    ctx.check(ctx.lib.obvhs_build_cwbvh(ctx.h, p, n, ctypes.byref(prm), dev, ctypes.byref(h), ctypes.byref(st)))
    if dev:
        ctx.synchronize()
    del keep
    return CwBvh(ctx, h, BuildStats.from_c(st))


def morton_sort(aabbs, sort_precision=SortPrecision.U64, ctx: Context | None = None):
    """Morton codes of the leaf centres (input order, (lo, hi) u64) and the
    stable sorted order (src/ploc/mod.rs:771-847)."""
    ctx = _ctx(ctx)
    a = np.ascontiguousarray(aabbs, dtype=np.float32).reshape(-1, 6)
    codes = np.zeros((len(a), 2), np.uint64)
    order = np.zeros(len(a), np.uint32)
    ctx.check(ctx.lib.obvhs_morton_sort(ctx.h, a.ctypes.data_as(ctypes.c_void_p), len(a), int(sort_precision),
                                        codes.ctypes.data_as(ctypes.c_void_p), order.ctypes.data_as(ctypes.c_void_p)))
    return codes, order
