"""ctypes wrapper around the C++ oracle (obvhs_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check in
__graft_entry__.py and by bench.py's CPU-baseline leg.  The product package
obvhs_gb300 never imports this module.

Array conventions (all numpy, C-contiguous):
  aabbs  float32 (n, 6)  min xyz, max xyz
  tris   float32 (n, 9)  v0 xyz, v1 xyz, v2 xyz
  rays   float32 (n, 8)  origin xyz, tmin, dir xyz, tmax
  bvh2   uint8   (m, 32) min xyz f32, prim_count u32, max xyz f32, first_index u32
  cwbvh  uint8   (m, 80) CwBvhNode byte layout of src/cwbvh/node.rs:12-54
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "obvhs_oracle.cpp")
_LIB = os.path.join(_HERE, "_build", "libobvhs_oracle.so")

CXXFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-std=c++17", "-fPIC", "-shared"]


def compile_lib(force: bool = False) -> str:
    """Compile the oracle with g++ (host compiler, either architecture)."""
    if not force and os.path.exists(_LIB) and os.path.getmtime(_LIB) >= os.path.getmtime(_SRC):
        return _LIB
    os.makedirs(os.path.dirname(_LIB), exist_ok=True)
    tmp = _LIB + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", *CXXFLAGS, "-o", tmp, _SRC, "-lpthread"])
    os.replace(tmp, _LIB)
    return _LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(compile_lib())
        _declare(_lib)
    return _lib


P = ctypes.c_void_p
U64 = ctypes.c_uint64
U32 = ctypes.c_uint32
I32 = ctypes.c_int32
F32 = ctypes.c_float


class OrcParams(ctypes.Structure):
    _fields_ = [
        ("pre_split", I32),
        ("search_distance", U32),
        ("search_depth_threshold", U32),
        ("reinsertion_batch_ratio", F32),
        ("sort_precision", U32),
        ("max_prims_per_leaf", U32),
    ]


def _declare(L):
    L.orc_tri_aabbs.argtypes = [P, U64, P]
    L.orc_morton.argtypes = [P, U64, U32, P, P]
    L.orc_ploc.argtypes = [P, P, U64, U32, U32, U32, I32, P, P, P]
    L.orc_ploc.restype = ctypes.c_int64
    L.orc_reinsertion.argtypes = [P, U64, P, U64, U32, F32, P, U64, I32, P]
    L.orc_reinsertion.restype = I32
    L.orc_bvh2_to_cwbvh.argtypes = [P, U64, P, U64, U32, I32, P, P, P]
    L.orc_bvh2_to_cwbvh.restype = I32
    L.orc_bvh2_collapse.argtypes = [P, U64, P, U64, U32, ctypes.c_float, P]
    L.orc_bvh2_collapse.restype = I32
    L.orc_bvh2_rebuild.argtypes = [P, U64, P, ctypes.c_int64, U32, U32, U32]
    L.orc_bvh2_rebuild.restype = ctypes.c_int64
    L.orc_query.argtypes = [I32, I32, P, U64, P, U64, P, U64, P, U64, P, P, P, U64]
    L.orc_query.restype = None
    L.orc_bvh2_refit_all.argtypes = [P, U64]
    L.orc_bvh2_refit_all.restype = None
    L.orc_bvh2_traverse.argtypes = [I32, P, U64, P, U64, P, U64, P, U64, P, I32, P]
    L.orc_bvh2_traverse.restype = None
    L.orc_build_bvh2.argtypes = [P, P, U64, P, ctypes.c_float, ctypes.c_float, I32, P]
    L.orc_build_bvh2.restype = P
    L.orc_bvh2_to_cwbvh_exact.argtypes = [P, U64, P, U64, U32, I32, P, P, P, P]
    L.orc_bvh2_to_cwbvh_exact.restype = I32
    L.orc_cwbvh_order_children.argtypes = [P, U64, P, U64, P, P, U64, I32, ctypes.c_int64]
    L.orc_cwbvh_order_children.restype = I32
    L.orc_presplit.argtypes = [P, U64]
    L.orc_presplit.restype = P
    L.orc_presplit_count.argtypes = [P]
    L.orc_presplit_count.restype = U64
    L.orc_presplit_get.argtypes = [P, P, P]
    L.orc_build.argtypes = [P, P, U64, ctypes.POINTER(OrcParams), I32, ctypes.POINTER(I32)]
    L.orc_build.restype = P
    L.orc_free.argtypes = [P]
    L.orc_build_sizes.argtypes = [P, P]
    L.orc_build_times.argtypes = [P, P]
    L.orc_build_search_stats.argtypes = [P, P]
    L.orc_build_get_cwbvh.argtypes = [P, P, P]
    L.orc_build_get_bvh2.argtypes = [P, I32, P, P]
    L.orc_build_get_leaves.argtypes = [P, P, P, P, P]
    L.orc_traverse.argtypes = [I32, P, U64, P, P, U64, P, U64, P, P, I32, P]
    L.orc_traverse_tlas.argtypes = [P, U64, P, U32, P, P, P, P, P, P, U64, P, I32]
    L.orc_compress_tris.argtypes = [P, U64, P, U64, P]
    L.orc_traverse_compressed.argtypes = [I32, P, U64, P, P, P, U64, P, I32]
    L.orc_tri_intersect.argtypes = [P, P]
    L.orc_tri_intersect.restype = F32
    L.orc_validate_bvh2.argtypes = [P, U64, P, U64, U32, P, U64, I32, I32, P]
    L.orc_validate_bvh2.restype = I32
    L.orc_validate_cwbvh.argtypes = [P, U64, P, U64, P, U64, I32, P]
    L.orc_validate_cwbvh.restype = I32
    L.orc_sah_bvh2.argtypes = [P, U64]
    L.orc_sah_bvh2.restype = ctypes.c_double
    L.orc_sah_cwbvh.argtypes = [P, U64]
    L.orc_sah_cwbvh.restype = ctypes.c_double


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _f32(a, cols):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a.reshape(-1, cols)


def tri_aabbs(tris):
    tris = _f32(tris, 9)
    out = np.empty((len(tris), 6), np.float32)
    lib().orc_tri_aabbs(_p(tris), len(tris), _p(out))
    return out


def morton(aabbs, precision: int):
    """Morton codes (input order, (lo, hi) u64 pairs) and the stable sorted order."""
    aabbs = _f32(aabbs, 6)
    n = len(aabbs)
    codes = np.zeros((n, 2), np.uint64)
    order = np.zeros(n, np.uint32)
    lib().orc_morton(_p(aabbs), n, precision, _p(codes), _p(order))
    return codes, order


def ploc(aabbs, indices=None, search_distance=14, sort_precision=0, search_depth_threshold=0, nthreads=1):
    aabbs = _f32(aabbs, 6)
    n = len(aabbs)
    if indices is None:
        indices = np.arange(n, dtype=np.uint32)
    indices = np.ascontiguousarray(indices, dtype=np.uint32)
    nodes = np.zeros((max(2 * n - 1, 0), 32), np.uint8)
    pidx = np.zeros(n, np.uint32)
    stats = np.zeros(2, np.uint64)
    md = lib().orc_ploc(_p(aabbs), _p(indices), n, search_distance, sort_precision, search_depth_threshold,
                        nthreads, _p(nodes), _p(pidx), _p(stats))
    return nodes, pidx, int(md), stats


def reinsertion(nodes, pidx, max_depth, ratio, seq=None, nthreads=1):
    nodes = np.array(nodes, dtype=np.uint8, copy=True).reshape(-1, 32)
    pidx = np.ascontiguousarray(pidx, dtype=np.uint32)
    s = None if seq is None else np.ascontiguousarray(seq, dtype=np.float32)
    stats = np.zeros(2, np.uint64)
    r = lib().orc_reinsertion(_p(nodes), len(nodes), _p(pidx), len(pidx), max_depth, ratio, _p(s),
                              0 if s is None else len(s), nthreads, _p(stats))
    if r != 0:
        raise RuntimeError(f"oracle reinsertion failed: {r}")
    return nodes, stats


def bvh2_to_cwbvh(nodes, pidx, max_prims_per_leaf=3, order_children=True):
    nodes = np.ascontiguousarray(nodes, dtype=np.uint8).reshape(-1, 32)
    pidx = np.ascontiguousarray(pidx, dtype=np.uint32)
    out_n = np.zeros((max(len(nodes), 1), 80), np.uint8)
    out_p = np.zeros(max(len(pidx), 1), np.uint32)
    counts = np.zeros(2, np.uint64)
    r = lib().orc_bvh2_to_cwbvh(_p(nodes), len(nodes), _p(pidx), len(pidx), max_prims_per_leaf,
                                int(order_children), _p(out_n), _p(out_p), _p(counts))
    if r != 0:
        raise RuntimeError(f"oracle bvh2_to_cwbvh failed: {r}")
    return out_n[: int(counts[0])].copy(), out_p[: int(counts[1])].copy()


def bvh2_to_cwbvh_exact(nodes, pidx, max_prims_per_leaf=3, order_children=True):
    """bvh2_to_cwbvh with include_exact_node_aabbs: (nodes80, primitive
    indices, exact AABB (min xyz, max xyz) per CWBVH node)."""
    nodes = np.ascontiguousarray(nodes, dtype=np.uint8).reshape(-1, 32)
    pidx = np.ascontiguousarray(pidx, dtype=np.uint32)
    out_n = np.zeros((max(len(nodes), 1), 80), np.uint8)
    out_p = np.zeros(max(len(pidx), 1), np.uint32)
    out_e = np.zeros((max(len(nodes), 1), 6), np.float32)
    counts = np.zeros(2, np.uint64)
    r = lib().orc_bvh2_to_cwbvh_exact(_p(nodes), len(nodes), _p(pidx), len(pidx), max_prims_per_leaf,
                                      int(order_children), _p(out_n), _p(out_p), _p(out_e), _p(counts))
    if r != 0:
        raise RuntimeError(f"oracle bvh2_to_cwbvh failed: {r}")
    k = int(counts[0])
    return out_n[:k].copy(), out_p[: int(counts[1])].copy(), out_e[:k].copy()


def cwbvh_order_children(nodes80, pidx, prim_aabbs, direct_layout=False, exact=None, node_index=-1):
    """CwBvh::order_children (node_index < 0) or order_node_children: returns
    the reordered nodes (and exact boxes when given)."""
    nodes = np.ascontiguousarray(nodes80, dtype=np.uint8).reshape(-1, 80).copy()
    pidx = np.ascontiguousarray(pidx, dtype=np.uint32)
    prims = _f32(prim_aabbs, 6)
    ex = None if exact is None else np.ascontiguousarray(exact, dtype=np.float32).reshape(-1, 6).copy()
    r = lib().orc_cwbvh_order_children(_p(nodes), len(nodes), _p(pidx), len(pidx), _p(ex) if ex is not None else None,
                                       _p(prims), len(prims), int(direct_layout), int(node_index))
    if r != 0:
        raise RuntimeError(f"oracle order_children failed: {r}")
    return nodes if ex is None else (nodes, ex)


def collapse(nodes, pidx, max_prims, traversal_cost):
    """collapse (src/bvh2/leaf_collapser.rs): (nodes32, primitive_indices)."""
    nodes = np.ascontiguousarray(nodes, dtype=np.uint8).reshape(-1, 32).copy()
    pidx = np.ascontiguousarray(pidx, dtype=np.uint32).copy()
    counts = np.zeros(2, np.uint64)
    lib().orc_bvh2_collapse(_p(nodes), len(nodes), _p(pidx), len(pidx), int(max_prims), float(traversal_cost),
                            _p(counts))
    return nodes[: int(counts[0])].copy(), pidx[: int(counts[1])].copy()


def rebuild(nodes, leaves=None, search_distance=1, sort_precision=0, search_depth_threshold=0):
    """PlocBuilder::full_rebuild (leaves None) or partial_rebuild with the
    rebuild path flags of `leaves`: (nodes, max_depth)."""
    nodes = np.ascontiguousarray(nodes, dtype=np.uint8).reshape(-1, 32).copy()
    lv = None if leaves is None else np.ascontiguousarray(leaves, dtype=np.uint32)
    md = lib().orc_bvh2_rebuild(_p(nodes), len(nodes), _p(lv) if lv is not None else None,
                                -1 if lv is None else len(lv), int(search_distance), int(sort_precision),
                                int(search_depth_threshold))
    return nodes, int(md)


def query(nodes, pidx, queries, kind="aabb", prim_aabbs=None, direction=None):
    """Bvh2::aabb_traverse / point_traverse (32-byte nodes) or the traverse!
    loop with CwBvhNode::intersect_aabb / contains_point (80-byte nodes):
    per query the original ids of the reached leaves' primitives in traversal
    order (filtered by their boxes when prim_aabbs is given).  Returns a list
    of uint32 arrays."""
    nodes = np.ascontiguousarray(nodes, dtype=np.uint8)
    structure = 0 if nodes.shape[-1] == 32 else 1
    nodes = nodes.reshape(-1, 32 if structure == 0 else 80)
    pidx = np.ascontiguousarray(pidx, dtype=np.uint32)
    k = 0 if kind == "aabb" else 1
    q = _f32(queries, 6 if k == 0 else 3)
    pa = None if prim_aabbs is None else _f32(prim_aabbs, 6)
    d = None if direction is None else np.ascontiguousarray(direction, dtype=np.float32)
    n = len(q)
    off = np.zeros(n + 1, np.uint64)
    L = lib()
    L.orc_query(structure, k, _p(nodes), len(nodes), _p(pidx), len(pidx), _p(q), n, _p(pa),
                0 if pa is None else len(pa), _p(d), _p(off), None, 0)
    ids = np.zeros(max(int(off[n]), 1), np.uint32)
    L.orc_query(structure, k, _p(nodes), len(nodes), _p(pidx), len(pidx), _p(q), n, _p(pa),
                0 if pa is None else len(pa), _p(d), _p(off), _p(ids), len(ids))
    return [ids[int(off[i]):int(off[i + 1])].copy() for i in range(n)]


def refit_all(nodes):
    """Bvh2::refit_all (src/bvh2/mod.rs:527-570): returns the refit nodes."""
    nodes = np.ascontiguousarray(nodes, dtype=np.uint8).reshape(-1, 32).copy()
    lib().orc_bvh2_refit_all(_p(nodes), len(nodes))
    return nodes


def traverse_bvh2(nodes, pidx, tris, rays, mode=0, nthreads=1, counters=False):
    """Bvh2::ray_traverse (mode 0: (original ids, 0xffffffff = none), t) or
    ray_traverse_miss (mode 1: occluded flags) with Triangle::intersect."""
    nodes = np.ascontiguousarray(nodes, dtype=np.uint8).reshape(-1, 32)
    pidx = np.ascontiguousarray(pidx, dtype=np.uint32)
    tris = _f32(tris, 9)
    rays = _f32(rays, 8)
    hits = np.zeros((len(rays), 2), np.uint32)
    vis = np.zeros(1, np.uint64)
    lib().orc_bvh2_traverse(mode, _p(nodes), len(nodes), _p(pidx), len(pidx), _p(tris), len(tris), _p(rays),
                            len(rays), _p(hits), nthreads, _p(vis))
    out = (hits[:, 0].copy(), hits[:, 1].copy().view(np.float32)) if mode == 0 else hits[:, 0].astype(bool)
    return (out, int(vis[0])) if counters else out


def build_bvh2(tris=None, aabbs=None, params=None, nthreads=1):
    """build_bvh2_from_tris (tris) / build_bvh2 (aabbs), src/bvh2/builder.rs:
    returns (nodes32, primitive_indices, max_depth, reinsertions applied)."""
    from obvhs_gb300.params import BvhBuildParams

    params = params or BvhBuildParams.medium_build()
    p = OrcParams(int(params.pre_split) if tris is not None else 0, params.ploc_search_distance,
                  params.search_depth_threshold, params.reinsertion_batch_ratio, params.sort_precision,
                  params.max_prims_per_leaf)
    L = lib()
    st = I32(0)
    src = _f32(tris, 9) if tris is not None else _f32(aabbs, 6)
    h = L.orc_build_bvh2(_p(src) if tris is not None else None, _p(src) if tris is None else None, len(src),
                         ctypes.byref(p), float(params.post_collapse_reinsertion_batch_ratio_multiplier),
                         float(params.collapse_traversal_cost), nthreads, ctypes.byref(st))
    try:
        if st.value != 0:
            raise RuntimeError(f"oracle build_bvh2 failed: {st.value}")
        sz = np.zeros(8, np.uint64)
        L.orc_build_sizes(h, _p(sz))
        nodes = np.zeros((int(sz[2]), 32), np.uint8)
        bp = np.zeros(int(sz[3]), np.uint32)  # collapsing keeps every primitive slot
        L.orc_build_get_bvh2(h, 1, _p(nodes), _p(bp))
        return nodes, bp, int(sz[7]), int(sz[6])
    finally:
        L.orc_free(h)


def presplit(tris):
    tris = _f32(tris, 9)
    L = lib()
    h = L.orc_presplit(_p(tris), len(tris))
    try:
        m = L.orc_presplit_count(h)
        aabbs = np.zeros((m, 6), np.float32)
        idx = np.zeros(m, np.uint32)
        L.orc_presplit_get(h, _p(aabbs), _p(idx))
    finally:
        L.orc_free(h)
    return aabbs, idx


@dataclass
class OracleBuild:
    cw_nodes: np.ndarray
    cw_pidx: np.ndarray
    bvh2_nodes: np.ndarray
    bvh2_ploc_nodes: np.ndarray
    bvh2_pidx: np.ndarray
    leaf_aabbs: np.ndarray
    leaf_indices: np.ndarray
    codes: np.ndarray
    order: np.ndarray
    ploc_passes: int
    sum_counts: int
    reinsertions: int
    max_depth: int
    times_ms: np.ndarray
    searches: int = 0       # reinsertion searches (find_reinsertion calls)
    search_nodes: int = 0   # node records those searches read


def build(tris=None, aabbs=None, params=None, nthreads=1, keep_intermediate=True) -> OracleBuild:
    """build_cwbvh_from_tris (tris given) or build_cwbvh (aabbs given)."""
    from obvhs_gb300.params import BvhBuildParams  # plain dataclass, no CUDA

    params = params or BvhBuildParams.medium_build()
    p = OrcParams(int(params.pre_split), params.ploc_search_distance, params.search_depth_threshold,
                  params.reinsertion_batch_ratio, params.sort_precision, params.max_prims_per_leaf)
    L = lib()
    st = I32(0)
    if tris is not None:
        tris = _f32(tris, 9)
        n = len(tris)
        h = L.orc_build(_p(tris), None, n, ctypes.byref(p), nthreads, ctypes.byref(st))
    else:
        aabbs = _f32(aabbs, 6)
        n = len(aabbs)
        h = L.orc_build(None, _p(aabbs), n, ctypes.byref(p), nthreads, ctypes.byref(st))
    try:
        if st.value != 0:
            raise RuntimeError(f"oracle build failed: {st.value}")
        sz = np.zeros(8, np.uint64)
        L.orc_build_sizes(h, _p(sz))
        tm = np.zeros(4, np.float64)
        L.orc_build_times(h, _p(tm))
        ss = np.zeros(2, np.uint64)
        L.orc_build_search_stats(h, _p(ss))
        cwn = np.zeros((int(sz[0]), 80), np.uint8)
        cwp = np.zeros(int(sz[1]), np.uint32)
        L.orc_build_get_cwbvh(h, _p(cwn), _p(cwp))
        nb = int(sz[2])
        m = int(sz[3])
        b2 = np.zeros((nb, 32), np.uint8)
        b2p = np.zeros((nb, 32), np.uint8)
        bp = np.zeros(m, np.uint32)
        la = np.zeros((m, 6), np.float32)
        li = np.zeros(m, np.uint32)
        codes = np.zeros((m, 2), np.uint64)
        order = np.zeros(m, np.uint32)
        if keep_intermediate:
            L.orc_build_get_bvh2(h, 1, _p(b2), _p(bp))
            L.orc_build_get_bvh2(h, 0, _p(b2p), _p(bp))
            L.orc_build_get_leaves(h, _p(la), _p(li), _p(codes), _p(order))
        return OracleBuild(cwn, cwp, b2, b2p, bp, la, li, codes, order, int(sz[4]), int(sz[5]), int(sz[6]),
                           int(sz[7]), tm, int(ss[0]), int(ss[1]))
    finally:
        L.orc_free(h)


def traverse(cw_nodes, cw_pidx, tris, rays, mode=0, nthreads=1, counters=False):
    """mode 0 = closest hit (ray_traverse), 1 = occlusion (ray_traverse_miss).

    Returns (prim_ids (original ids, 0xffffffff = none), t float32, bvh-order ids[, counters]).
    """
    cw_nodes = np.ascontiguousarray(cw_nodes, dtype=np.uint8).reshape(-1, 80)
    cw_pidx = np.ascontiguousarray(cw_pidx, dtype=np.uint32)
    tris = _f32(tris, 9)
    rays = _f32(rays, 8)
    n = len(rays)
    hits = np.zeros((n, 2), np.uint32)
    ids = np.zeros(n, np.uint32)
    cnt = np.zeros(2, np.uint64)
    lib().orc_traverse(mode, _p(cw_nodes), len(cw_nodes), _p(cw_pidx), _p(tris), len(tris), _p(rays), n,
                       _p(hits), _p(ids), nthreads, _p(cnt) if counters else None)
    out = (hits[:, 0].copy(), hits[:, 1].copy().view(np.float32), ids)
    return out + (cnt,) if counters else out


def compress_tris(tris, pidx):
    """RtCompressedTriangle::new (src/rt_triangle.rs:31-47) of tris (original
    order) laid out in pidx order: (n, 24) bytes."""
    tris = _f32(tris, 9)
    pidx = np.ascontiguousarray(pidx, dtype=np.uint32)
    out = np.zeros((len(pidx), 24), np.uint8)
    lib().orc_compress_tris(_p(tris), len(tris), _p(pidx), len(pidx), _p(out))
    return out


def traverse_compressed(cw_nodes, cw_pidx, ctris24, rays, mode=0, nthreads=1):
    """ray_traverse (mode 0) / ray_traverse_miss (mode 1) with
    RtCompressedTriangle::intersect; ctris24 in primitive_indices order.
    Returns (original ids or 0xffffffff, t)."""
    cw_nodes = np.ascontiguousarray(cw_nodes, dtype=np.uint8).reshape(-1, 80)
    cw_pidx = np.ascontiguousarray(cw_pidx, dtype=np.uint32)
    ctris24 = np.ascontiguousarray(ctris24, dtype=np.uint8).reshape(-1, 24)
    rays = _f32(rays, 8)
    hits = np.zeros((len(rays), 2), np.uint32)
    lib().orc_traverse_compressed(mode, _p(cw_nodes), len(cw_nodes), _p(cw_pidx), _p(ctris24), _p(rays), len(rays),
                                  _p(hits), nthreads)
    return hits[:, 0].copy(), hits[:, 1].copy().view(np.float32)


def traverse_tlas(tlas_nodes, tlas_pidx, blas, rays, nthreads=1):
    """CwBvh::ray_traverse_tlas_blas (src/cwbvh/mod.rs:342-491) with
    Triangle::intersect.  `blas` is a list of (cwbvh nodes, primitive_indices,
    triangles in original order).  Returns (geometry id, BVH-order primitive
    id, original primitive id, t) arrays; ids 0xffffffff and t +inf on a miss."""
    tlas_nodes = np.ascontiguousarray(tlas_nodes, dtype=np.uint8).reshape(-1, 80)
    tlas_pidx = np.ascontiguousarray(tlas_pidx, dtype=np.uint32)
    keep = []
    nodes_p, nn, pidx_p, tris_p, nt = [], [], [], [], []
    for nodes, pidx, tris in blas:
        nodes = np.ascontiguousarray(nodes, dtype=np.uint8).reshape(-1, 80)
        pidx = np.ascontiguousarray(pidx, dtype=np.uint32)
        tris = _f32(tris, 9)
        keep += [nodes, pidx, tris]
        nodes_p.append(nodes.ctypes.data)
        pidx_p.append(pidx.ctypes.data)
        tris_p.append(tris.ctypes.data)
        nn.append(len(nodes))
        nt.append(len(tris))
    arr = lambda v, t: (t * max(len(v), 1))(*v)
    rays = _f32(rays, 8)
    n = len(rays)
    hits = np.zeros((n, 4), np.uint32)
    lib().orc_traverse_tlas(_p(tlas_nodes), len(tlas_nodes), _p(tlas_pidx), len(blas),
                            ctypes.cast(arr(nodes_p, ctypes.c_void_p), ctypes.c_void_p),
                            ctypes.cast(arr(nn, ctypes.c_uint64), ctypes.c_void_p),
                            ctypes.cast(arr(pidx_p, ctypes.c_void_p), ctypes.c_void_p),
                            ctypes.cast(arr(tris_p, ctypes.c_void_p), ctypes.c_void_p),
                            ctypes.cast(arr(nt, ctypes.c_uint64), ctypes.c_void_p), _p(rays), n, _p(hits), nthreads)
    return hits[:, 0].copy(), hits[:, 1].copy(), hits[:, 2].copy(), hits[:, 3].copy().view(np.float32)


def tri_intersect(tri9, ray8) -> float:
    t = _f32(tri9, 9)
    r = _f32(ray8, 8)
    return float(lib().orc_tri_intersect(_p(t), _p(r)))


def validate_bvh2(nodes, pidx, max_depth, prim_aabbs, tight=False, splits=False):
    nodes = np.ascontiguousarray(nodes, dtype=np.uint8).reshape(-1, 32)
    pidx = np.ascontiguousarray(pidx, dtype=np.uint32)
    pa = _f32(prim_aabbs, 6)
    d = U32(0)
    r = lib().orc_validate_bvh2(_p(nodes), len(nodes), _p(pidx), len(pidx), max_depth, _p(pa), len(pa),
                                int(tight), int(splits), ctypes.byref(d))
    return r, d.value


def validate_cwbvh(nodes, pidx, prim_aabbs, splits=False):
    nodes = np.ascontiguousarray(nodes, dtype=np.uint8).reshape(-1, 80)
    pidx = np.ascontiguousarray(pidx, dtype=np.uint32)
    pa = _f32(prim_aabbs, 6)
    d = U32(0)
    r = lib().orc_validate_cwbvh(_p(nodes), len(nodes), _p(pidx), len(pidx), _p(pa), len(pa), int(splits),
                                 ctypes.byref(d))
    return r, d.value


def sah_bvh2(nodes):
    nodes = np.ascontiguousarray(nodes, dtype=np.uint8).reshape(-1, 32)
    return lib().orc_sah_bvh2(_p(nodes), len(nodes))


def sah_cwbvh(nodes):
    nodes = np.ascontiguousarray(nodes, dtype=np.uint8).reshape(-1, 80)
    return lib().orc_sah_cwbvh(_p(nodes), len(nodes))
