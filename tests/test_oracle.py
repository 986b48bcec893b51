"""The oracle against the reference's own golden values and tests (CPU only).

Pins reproduced here (each names the reference test it restates):
  * traverse! doctest, src/cwbvh/traverse_macro.rs:17-57 -> original prim 62
  * check_flat_subdivided_plane_normals, tests/mod.rs:104-124 -> 65,536 +Y hits
  * obj_cwbvh test, examples/obj_cwbvh.rs:142-181 -> hash 1343358762, 5 presets
  * degenerate builds, tests/mod.rs:34-88 -> build and miss
  * build_bvh_with_varying_prim_counts, tests/mod.rs:90-102 -> validate
  * test_reinsertion, src/bvh2/reinsertion.rs:394-438 -> validate
"""
import numpy as np
import pytest

from oracle import oracle as O
from obvhs_gb300 import test_util as T
from obvhs_gb300.params import PRESETS, BvhBuildParams, SortPrecision

import helpers as H

ALL = list(PRESETS)
F32_MAX = np.float32(3.4028235e38)


def _interleave_ref(x, y, z, bits):
    code = 0
    for b in range(bits):
        code |= ((x >> b) & 1) << (3 * b)
        code |= ((y >> b) & 1) << (3 * b + 1)
        code |= ((z >> b) & 1) << (3 * b + 2)
    return code


@pytest.mark.parametrize("precision,bits", [(0, 21), (1, 42)])
def test_morton_matches_bit_interleave(precision, bits):
    """morton_encode_u64/u128_unorm (src/ploc/morton.rs:55-89) equal a plain
    bit interleave of the truncated, masked grid coordinates."""
    rng = np.random.default_rng(7)
    n = 300
    c = rng.uniform(-3, 5, size=(n, 3)).astype(np.float32)
    aabbs = np.concatenate([c, c], 1)
    codes, order = O.morton(aabbs, precision)
    mn = aabbs[:, :3].min(0)
    mx = aabbs[:, 3:].max(0)
    # Aabb::diagonal() is an f32 subtraction, widened afterwards (ploc/mod.rs:287)
    scale = 1.0 / (mx - mn).astype(np.float64)
    offset = -mn.astype(np.float64) * scale
    for i in range(n):
        p = c[i].astype(np.float64) * scale + offset
        q = [int(v * float(1 << bits)) if v > 0 else 0 for v in p]
        q = [min(v, (1 << 64) - 1) & ((1 << bits) - 1) for v in q]
        want = _interleave_ref(q[0], q[1], q[2], bits)
        got = int(codes[i, 0]) | (int(codes[i, 1]) << 64)
        assert got == want, i
    keys = [(int(codes[i, 0]) | (int(codes[i, 1]) << 64), i) for i in range(n)]
    assert [k[1] for k in sorted(keys)] == list(order)


def test_morton_edge_cases():
    """unorm 1.0 -> 2^21 masks to 0; NaN/negative saturate to 0 (Rust `as`)."""
    aabbs = np.array([[0, 0, 0, 0, 0, 0], [1, 1, 1, 1, 1, 1]], np.float32)
    codes, _ = O.morton(aabbs, 0)
    assert int(codes[0, 0]) == 0 and int(codes[1, 0]) == 0
    codes, _ = O.morton(aabbs, 1)
    assert int(codes[1, 0]) == 0 and int(codes[1, 1]) == 0
    inf = np.array([[-np.inf] * 3 + [np.inf] * 3] * 4, np.float32)
    codes, order = O.morton(inf, 0)
    assert not codes.any() and list(order) == [0, 1, 2, 3]


@pytest.mark.parametrize("preset", ALL)
def test_doctest_hit_prim_62(preset):
    tris, ray = H.doctest_scene()
    b = O.build(tris=tris, params=PRESETS[preset]())
    ids, t, _ = O.traverse(b.cw_nodes, b.cw_pidx, tris, ray)
    assert ids[0] == H.DOCTEST_PRIM
    assert np.isfinite(t[0])


def test_flat_plane_normals():
    tris, rays = H.plane_scene()
    b = O.build(tris=tris, params=BvhBuildParams.medium_build())
    _, _, bid = O.traverse(b.cw_nodes, b.cw_pidx, tris, rays)
    assert (bid != 0xFFFFFFFF).all()
    # tests/mod.rs:110 indexes the ORIGINAL tris by the BVH-order id.
    n = T.compute_normal(tris[bid])
    assert np.all(n == np.array([0, 1, 0], np.float32))


@pytest.mark.parametrize("preset", ["fastest", "fast", "medium", "slow", "very_slow"])
def test_kitchen_hash(preset):
    tris = H.kitchen_tris()
    rays = H.kitchen_rays()
    b = O.build(tris=tris, params=PRESETS[preset](), nthreads=4)
    _, _, bid = O.traverse(b.cw_nodes, b.cw_pidx, tris, rays)
    assert H.kitchen_hash(tris, b.cw_pidx, bid, rays) == H.KITCHEN_HASH


EMPTY = np.array([[F32_MAX] * 3 + [-F32_MAX] * 3], np.float32)
INF10 = np.array([[-np.inf] * 3 + [np.inf] * 3] * 10, np.float32)
MAX10 = np.array([[-F32_MAX] * 3 + [F32_MAX] * 3] * 10, np.float32)
NOTHING = np.zeros((0, 6), np.float32)


@pytest.mark.parametrize("preset", ALL)
@pytest.mark.parametrize("aabbs", [EMPTY, INF10, MAX10, NOTHING], ids=["empty", "inf", "max", "nothing"])
def test_degenerate_bvh2_builds(preset, aabbs):
    """build_bvh2_with_{empty_aabb,many_inf,many_max,nothing} (tests/mod.rs:34-78):
    PLOC + reinsertion build and produce a structurally valid tree."""
    p = PRESETS[preset]()
    nodes, pidx, md, _ = O.ploc(aabbs, search_distance=p.ploc_search_distance, sort_precision=p.sort_precision,
                                search_depth_threshold=p.search_depth_threshold)
    assert len(nodes) == max(2 * len(aabbs) - 1, 0)
    if len(nodes):
        nodes, _ = O.reinsertion(nodes, pidx, md, p.reinsertion_batch_ratio)
        assert O.validate_bvh2(nodes, pidx, md, aabbs)[0] == 0


@pytest.mark.parametrize("preset", ALL)
@pytest.mark.parametrize("aabbs", [EMPTY, NOTHING], ids=["empty", "nothing"])
def test_degenerate_cwbvh_builds_miss(preset, aabbs):
    """build_cwbvh_with_{empty_aabb,nothing} (tests/mod.rs:61-88)."""
    b = O.build(aabbs=aabbs, params=PRESETS[preset]())
    if len(aabbs) == 0:
        assert len(b.cw_nodes) == 0
    ray = T.make_rays([[0, 0, 1]], [[0, 0, -1]])
    dummy = np.zeros((max(len(aabbs), 1), 9), np.float32)  # triangles that never hit
    ids, _, _ = O.traverse(b.cw_nodes, b.cw_pidx, dummy, ray)
    assert ids[0] == 0xFFFFFFFF


def test_cwbvh_of_infinite_boxes_is_an_error():
    """With infinite half areas every distribution cost is inf, no split is
    chosen and the reference would index decisions out of range
    (src/cwbvh/bvh2_to_cwbvh.rs:281-291,361-369); the oracle reports it."""
    with pytest.raises(RuntimeError):
        O.build(aabbs=INF10, params=BvhBuildParams.medium_build())


def test_varying_prim_counts_validate():
    tris_all = T.height_to_triangles(T.flat_heights(4, 4), 4, 4)
    for n in range(len(tris_all) - 1, 0, -1):
        tris = tris_all[:n]
        aabbs = T.tri_aabbs(tris)
        for preset in ALL:
            p = PRESETS[preset]()
            b = O.build(tris=tris, params=p)
            r, _ = O.validate_bvh2(b.bvh2_nodes, b.bvh2_pidx, b.max_depth, aabbs, tight=not p.pre_split,
                                   splits=p.pre_split)
            assert r == 0, (n, preset, "bvh2", r)
            r, _ = O.validate_cwbvh(b.cw_nodes, b.cw_pidx, aabbs, splits=p.pre_split)
            assert r == 0, (n, preset, "cwbvh", r)


def test_reinsertion_validates_demoscene():
    tris = T.demoscene(32, 0)
    aabbs = T.tri_aabbs(tris)
    nodes, pidx, md, _ = O.ploc(aabbs, search_distance=2, sort_precision=SortPrecision.U64,
                                search_depth_threshold=1)
    assert O.validate_bvh2(nodes, pidx, md, aabbs)[0] == 0
    nodes2, stats = O.reinsertion(nodes, pidx, md, 0.25)
    assert stats[0] > 0
    assert O.validate_bvh2(nodes2, pidx, md, aabbs, tight=True)[0] == 0
    nodes3, _ = O.reinsertion(nodes2, pidx, md, 0.5)
    assert O.validate_bvh2(nodes3, pidx, md, aabbs, tight=True)[0] == 0
    assert O.sah_bvh2(nodes3) <= O.sah_bvh2(nodes) * 1.0001


def test_tri_aabbs_match_numpy():
    tris = T.demoscene(16, 3)
    assert np.array_equal(O.tri_aabbs(tris).view(np.uint32), T.tri_aabbs(tris).view(np.uint32))


def test_triangle_intersect_kats():
    """Triangle::intersect (src/triangle.rs:35-76): hit, miss, and tmin/tmax."""
    tri = np.array([[-1, -1, 0, 1, -1, 0, 0, 1, 0]], np.float32)
    assert O.tri_intersect(tri, T.make_rays([[0, 0, -2]], [[0, 0, 1]])) == 2.0
    assert O.tri_intersect(tri, T.make_rays([[5, 0, -2]], [[0, 0, 1]])) == np.inf
    assert O.tri_intersect(tri, T.make_rays([[0, 0, -2]], [[0, 0, 1]], tmax=1.5)) == np.inf
    assert O.tri_intersect(tri, T.make_rays([[0, 0, -2]], [[0, 0, 1]], tmin=2.5)) == np.inf


# --- instance traversal (CwBvh::ray_traverse_tlas_blas) ---------------------

import instances as I


def test_tlas_with_one_instance_equals_plain_traversal():
    blas_tris = I.instanced_scene(1, seed=2)
    tl, blas = I.oracle_scene(blas_tris, 3)
    rays = I.incoherent_rays(4000)
    g, p, orig, t = O.traverse_tlas(tl.cw_nodes, tl.cw_pidx, blas, rays)
    nodes, pidx, tris = blas[0]
    oid, ot, bvh_ids = O.traverse(nodes, pidx, tris, rays, 0)
    hit = oid != 0xFFFFFFFF
    assert hit.any()
    assert np.array_equal(orig, oid) and np.array_equal(p, bvh_ids)
    assert np.array_equal(t.view(np.uint32), ot.view(np.uint32))
    assert np.array_equal(g[hit], np.zeros(hit.sum(), np.uint32))


def test_tlas_hits_are_the_closest_hit_of_the_reported_instance():
    """Each reported hit is the closest hit of its own BLAS (the instance was
    entered with a tmax no smaller than that hit), and never nearer than the
    closest over all instances.  The reference does not visit every instance
    a ray reaches: after the first instance of a TLAS node's leaf group it
    pushes the rest as a primitive group, which its loop clears when popped,
    so the nearest instance can be skipped (misses below)."""
    blas_tris = I.instanced_scene(8, seed=3)
    tl, blas = I.oracle_scene(blas_tris, 1)
    rays = I.incoherent_rays(4000, seed=4)
    g, p, orig, t = O.traverse_tlas(tl.cw_nodes, tl.cw_pidx, blas, rays)
    per = [O.traverse(nodes, pidx, tris, rays, 0) for nodes, pidx, tris in blas]
    best_t = np.min(np.stack([x[1] for x in per]), axis=0)
    hit = g != 0xFFFFFFFF
    assert hit.sum() > 100
    assert np.all(t[hit] >= best_t[hit])
    for b in range(len(blas)):
        sel = g == b
        oid, ot, bvh = per[b]
        assert np.array_equal(t[sel].view(np.uint32), ot[sel].view(np.uint32))
        assert np.array_equal(orig[sel], oid[sel]) and np.array_equal(p[sel], bvh[sel])
    assert np.all(np.isinf(t[~hit]))
    assert (t > best_t).any()  # instances skipped as in the reference


# --- RtCompressedTriangle ------------------------------------------------------


def test_compressed_triangle_halves_round_to_nearest_even():
    """Edges go to IEEE halves with round-to-nearest-even (f16::from_f32),
    checked against numpy's float16 conversion: normal, subnormal, overflow,
    and exact halfway values."""
    rng = np.random.default_rng(1)
    vals = np.concatenate([
        rng.normal(size=20000).astype(np.float32) * np.float32(10.0) ** rng.integers(-8, 6, 20000).astype(np.float32),
        np.float32([0.0, -0.0, 65504.0, 65520.0, 65519.99, 1e6, -1e6, 6.1e-5, 5.96e-8, 2.98e-8, 2.9802326e-08,
                    1e-9, 1.0 + 2.0 ** -11, 1.0 + 3 * 2.0 ** -11, 2048.0 + 1.0, 2048.0 + 3.0]),
        (np.arange(1, 2048, dtype=np.float32) + np.float32(0.5)) * np.float32(2.0 ** -24),  # subnormal halfway
    ]).astype(np.float32)
    n = (len(vals) + 2) // 3 * 3
    v = np.zeros(n, np.float32)
    v[: len(vals)] = vals
    e1 = v.reshape(-1, 3)
    tris = np.zeros((len(e1), 9), np.float32)
    tris[:, 3:6] = e1  # v0 = 0, v1 = e1, so the stored e1 is the value itself
    ct = O.compress_tris(tris, np.arange(len(tris), dtype=np.uint32))
    halves = ct[:, 12:24].copy().view(np.uint16).reshape(-1, 6)[:, 0::2]  # e1x, e1y, e1z
    with np.errstate(over="ignore"):
        expect = e1.astype(np.float16).view(np.uint16)
    assert np.array_equal(halves, expect)


def test_compressed_traversal_hits_large_flat_quads():
    """Exact-in-half geometry (a 16x16 grid of unit quads at z = 0): rays straight
    down hit the quad under them, as with full-precision triangles."""
    qs = []
    for i in range(16):
        for j in range(16):
            a, b, c, d = (i, j, 0), (i + 1, j, 0), (i + 1, j + 1, 0), (i, j + 1, 0)
            qs += [a + b + c, a + c + d]
    tris = np.asarray(qs, np.float32)
    ob = O.build(tris=tris, params=BvhBuildParams.medium_build(), keep_intermediate=False)
    ct = O.compress_tris(tris, ob.cw_pidx)
    xs = np.float32(0.3) + np.arange(16, dtype=np.float32)
    o = np.stack(np.meshgrid(xs, xs, indexing="ij"), -1).reshape(-1, 2)
    o = np.concatenate([o, np.full((len(o), 1), 5, np.float32)], 1)
    d = np.tile(np.float32([0, 0, -1]), (len(o), 1))
    rays = T.make_rays(o.astype(np.float32), d, 0.0, np.inf)
    cid, ct_t = O.traverse_compressed(ob.cw_nodes, ob.cw_pidx, ct, rays)
    fid, ft, _ = O.traverse(ob.cw_nodes, ob.cw_pidx, tris, rays)
    assert np.all(cid != 0xFFFFFFFF) and np.array_equal(cid, fid)
    assert np.allclose(ct_t, 5.0) and np.allclose(ft, 5.0)


# --- CWBVH post-passes: exact node AABBs and order_children -----------------


def _very_fast_demoscene():
    """The set-up of order_children_cwbvh / exact_aabbs_cwbvh
    (tests/mod.rs:350-451): demoscene(100, 0), very_fast_build's PLOC, then
    bvh2_to_cwbvh(max_prims 8 clamped to 3, order_children = true)."""
    from obvhs_gb300.params import BvhBuildParams

    tris = T.demoscene(100, 0)
    aabbs = T.tri_aabbs(tris)
    p = BvhBuildParams.very_fast_build()
    nodes, pidx, _, _ = O.ploc(aabbs, None, int(p.ploc_search_distance), int(p.sort_precision),
                               int(p.search_depth_threshold))
    return tris, aabbs, nodes, pidx


def test_order_children_keeps_a_valid_tree():
    """order_children_cwbvh (tests/mod.rs:351-385): every node reordered one
    at a time, then the whole pass: the CWBVH stays valid each time."""
    tris, aabbs, nodes, pidx = _very_fast_demoscene()
    cn, cp = O.bvh2_to_cwbvh(nodes, pidx, 3, True)
    assert O.validate_cwbvh(cn, cp, aabbs)[0] == 0
    one = cn
    for i in range(len(cn)):
        one = O.cwbvh_order_children(one, cp, aabbs, node_index=i)
    assert O.validate_cwbvh(one, cp, aabbs)[0] == 0
    whole = O.cwbvh_order_children(one, cp, aabbs)
    assert O.validate_cwbvh(whole, cp, aabbs)[0] == 0
    # node-by-node in index order is the whole pass
    assert np.array_equal(O.cwbvh_order_children(cn, cp, aabbs), one)


def test_exact_aabbs_contained_in_the_compressed_boxes():
    """exact_aabbs_cwbvh (tests/mod.rs:387-451): each inner child's exact box
    lies inside its quantised box in the parent and inside its own node's
    (p, e) box; order_children with the exact boxes keeps the tree valid."""
    tris, aabbs, nodes, pidx = _very_fast_demoscene()
    cn, cp, ex = O.bvh2_to_cwbvh_exact(nodes, pidx, 3, True)
    ref_n, ref_p = O.bvh2_to_cwbvh(nodes, pidx, 3, True)
    assert np.array_equal(cn, ref_n) and np.array_equal(cp, ref_p)
    rec = cn.view(np.uint8)

    def node_box(i):
        p = rec[i, 0:12].view(np.float32)
        e = (rec[i, 12:15].astype(np.uint32) << 23).view(np.float32)
        return p, p + e * np.float32(255.0)

    for i in range(len(cn)):
        p = rec[i, 0:12].view(np.float32)
        e = (rec[i, 12:15].astype(np.uint32) << 23).view(np.float32)
        imask = int(rec[i, 15])
        base = int(rec[i, 16:20].view(np.uint32)[0])
        for ch in range(8):
            meta = int(rec[i, 24 + ch])
            if meta == 0 or not (imask >> ch) & 1:
                continue
            slot = (meta & 31) - 24
            k = base + bin(imask & ~(0xFFFFFFFF << slot) & 0xFF).count("1")
            lo = np.array([rec[i, 32 + ch], rec[i, 48 + ch], rec[i, 64 + ch]], np.float32) * e + p
            hi = np.array([rec[i, 40 + ch], rec[i, 56 + ch], rec[i, 72 + ch]], np.float32) * e + p
            smin, smax = node_box(k)
            assert np.all(ex[k, :3] >= lo) and np.all(ex[k, 3:] <= hi)
            assert np.all(ex[k, :3] >= smin) and np.all(ex[k, 3:] <= smax)
    n1, e1 = O.cwbvh_order_children(cn, cp, aabbs, exact=ex)
    assert O.validate_cwbvh(n1, cp, aabbs)[0] == 0
    n2, e2 = O.cwbvh_order_children(n1, cp, aabbs, exact=e1)
    assert O.validate_cwbvh(n2, cp, aabbs)[0] == 0
    # the exact boxes move with their nodes: each still lies in its node's box
    for i in range(len(n2)):
        smin, smax = (lambda r: (r[0:12].view(np.float32),
                                 r[0:12].view(np.float32) + (r[12:15].astype(np.uint32) << 23).view(np.float32)
                                 * np.float32(255.0)))(n2.view(np.uint8)[i])
        assert np.all(e2[i, :3] >= smin - 1e-5) and np.all(e2[i, 3:] <= smax + 1e-5)


# --- the BVH2 product: collapse, build_bvh2, Bvh2 traversal ---------------------


@pytest.mark.parametrize("preset", ALL)
@pytest.mark.parametrize("aabbs", [EMPTY, INF10, MAX10, NOTHING], ids=["empty", "inf", "max", "nothing"])
def test_degenerate_build_bvh2_misses(preset, aabbs):
    """build_bvh2_with_{empty_aabb,many_inf,many_max,nothing} (tests/mod.rs:34-78)
    through the whole builder (reinsertion, collapse, reinsertion): valid,
    and the ray of the test misses."""
    nodes, pidx, md, _ = O.build_bvh2(aabbs=aabbs, params=PRESETS[preset]())
    if len(nodes):
        assert O.validate_bvh2(nodes, pidx, md, aabbs)[0] == 0
    ray = T.make_rays([[0, 0, 1]], [[0, 0, -1]])
    dummy = np.zeros((max(len(aabbs), 1), 9), np.float32)  # triangles that never hit
    ids, _ = O.traverse_bvh2(nodes, pidx, dummy, ray)
    assert ids[0] == 0xFFFFFFFF
    assert not O.traverse_bvh2(nodes, pidx, dummy, ray, mode=1)[0]


def test_varying_prim_counts_build_bvh2_validate():
    """build_bvh_with_varying_prim_counts (tests/mod.rs:90-102), the BVH2
    half: build_bvh2_from_tris for every prefix of a 32-triangle grid and
    every preset validates (tight boxes unless pre-split)."""
    tris_all = T.height_to_triangles(T.flat_heights(4, 4), 4, 4)
    for n in range(len(tris_all) - 1, 0, -1):
        tris = tris_all[:n]
        aabbs = T.tri_aabbs(tris)
        for preset in ALL:
            p = PRESETS[preset]()
            nodes, pidx, md, _ = O.build_bvh2(tris=tris, params=p)
            r, _ = O.validate_bvh2(nodes, pidx, md, aabbs, tight=not p.pre_split, splits=p.pre_split)
            assert r == 0, (n, preset, r)


@pytest.mark.parametrize("max_prims", [2, 3, 8, 255])
def test_collapse_keeps_every_primitive(max_prims):
    tris = T.demoscene(32, 0)
    aabbs = T.tri_aabbs(tris)
    nodes, pidx, md, _ = O.ploc(aabbs, search_distance=14)
    cn, cp = O.collapse(nodes, pidx, max_prims, 1.0)
    assert sorted(cp.tolist()) == sorted(pidx.tolist())
    assert len(cn) < len(nodes)
    counts = cn[:, 12:16].copy().view(np.uint32).ravel()
    assert counts.max() <= max_prims
    assert O.validate_bvh2(cn, cp, md, aabbs)[0] == 0


def test_bvh2_and_cwbvh_traversal_agree():
    """The same scene through build_bvh2_from_tris + Bvh2::ray_traverse and
    build_cwbvh_from_tris + CwBvh::ray_traverse: the same closest t for every
    ray (ids agree wherever the closest hit is unique), the same occlusion."""
    tris = T.demoscene(64, 3)
    rng = np.random.default_rng(4)
    v = tris.reshape(-1, 3)
    o = rng.uniform(v.min(0), v.max(0), size=(4000, 3)).astype(np.float32)
    o[:, 1] = v[:, 1].max() + 1.0
    d = T.normalize3(rng.uniform(-1, 1, size=(4000, 3)).astype(np.float32) * np.float32([0.3, 1, 0.3]) -
                     np.float32([0, 1, 0]))
    rays = T.make_rays(o, d, 0.0, np.inf)
    p = BvhBuildParams.medium_build()
    nodes, pidx, _, _ = O.build_bvh2(tris=tris, params=p)
    b2_ids, b2_t = O.traverse_bvh2(nodes, pidx, tris, rays)
    cw = O.build(tris=tris, params=p)
    cw_ids, cw_t, _ = O.traverse(cw.cw_nodes, cw.cw_pidx, tris, rays)
    assert (b2_ids != 0xFFFFFFFF).mean() > 0.5
    assert np.array_equal(b2_t.view(np.uint32), cw_t.view(np.uint32))
    assert (b2_ids == cw_ids).mean() > 0.999
    occ = O.traverse_bvh2(nodes, pidx, tris, rays, mode=1)
    assert np.array_equal(occ, b2_ids != 0xFFFFFFFF)


# --- dynamic updates: full / partial rebuild, refit ------------------------------


def _leaf_ids(nodes):
    return np.nonzero(nodes[:, 12:16].copy().view(np.uint32).ravel() != 0)[0].astype(np.uint32)


def _rebuild_scenes():
    sm = T.demoscene(5, 0)
    return [T.demoscene(31, 0), sm, sm[:1], sm[:2], sm[:3]]


@pytest.mark.parametrize("which", ["full", "partial_all", "partial_one", "partial_random"])
def test_rebuilds_validate(which):
    """test_full_rebuild, test_partial_rebuild_with_{all_leaves,one_leaf,
    random_leaves} (src/ploc/rebuild.rs:193-366)."""
    scenes = [T.demoscene(8, 0)] if which == "partial_one" else _rebuild_scenes()
    for tris in scenes:
        aabbs = T.tri_aabbs(tris)
        thr = 0 if which in ("partial_one", "partial_random") else 1
        nodes, pidx, md, _ = O.ploc(aabbs, search_distance=1, sort_precision=0, search_depth_threshold=thr)
        assert O.validate_bvh2(nodes, pidx, md, aabbs)[0] == 0
        leaves = _leaf_ids(nodes)
        if which == "full":
            out, md2 = O.rebuild(nodes, None, 1, 0, 1)
        else:
            if which == "partial_one":
                pick = leaves[:1]
            elif which == "partial_random":
                pick = np.array([i for i in leaves if T.hash_noise(0, 0, int(i)) > 0.5][:1], np.uint32)
            else:
                pick = leaves
            out, md2 = O.rebuild(nodes, pick, 1, 0, thr)
        assert len(out) == len(nodes)
        assert O.validate_bvh2(out, pidx, md2, aabbs)[0] == 0


def test_partial_rebuild_after_moving_leaves():
    """Leaves given new boxes, their paths rebuilt: a valid, tight tree over
    the moved boxes; untouched subtrees keep their nodes."""
    tris = T.demoscene(32, 0)
    aabbs = T.tri_aabbs(tris)
    nodes, pidx, md, _ = O.ploc(aabbs, search_distance=14)
    leaves = _leaf_ids(nodes)
    rng = np.random.default_rng(3)
    moved = np.sort(rng.choice(leaves, size=len(leaves) // 20, replace=False)).astype(np.uint32)
    shift = np.float32(0.3)
    new_aabbs = aabbs.copy()
    nn = nodes.copy()
    for i in moved:
        f = nn[i].view(np.float32)
        f[[0, 1, 2, 4, 5, 6]] += shift
        prim = pidx[nn[i, 28:32].view(np.uint32)[0]]
        new_aabbs[prim] += shift
    out, md2 = O.rebuild(nn, moved, 14, 0, 0)
    assert O.validate_bvh2(out, pidx, md2, new_aabbs)[0] == 0
    # refit_all of a tree whose leaves moved in place gives tight boxes again
    refit = O.refit_all(nn)
    assert O.validate_bvh2(refit, pidx, md, new_aabbs)[0] == 0


# --- AABB and point queries -----------------------------------------------------------


def _brute(tris, q, kind):
    a = T.tri_aabbs(tris)
    if kind == "aabb":
        hit = ~((a[:, 0] > q[3]) | (a[:, 1] > q[4]) | (a[:, 2] > q[5]) | (a[:, 3] < q[0]) | (a[:, 4] < q[1]) |
                (a[:, 5] < q[2]))
    else:
        hit = (q[0] >= a[:, 0]) & (q[1] >= a[:, 1]) & (q[2] >= a[:, 2]) & (q[0] <= a[:, 3]) & (q[1] <= a[:, 4]) & \
              (q[2] <= a[:, 5])
    return np.nonzero(hit)[0]


def test_traverse_aabb():
    """traverse_aabb (tests/mod.rs:180-247): demoscene(201, 0), fast_build, the
    query box; BVH2 and CWBVH traversal with exact filtering find the same
    primitives (count and id sum) as testing every triangle."""
    tris = T.demoscene(201, 0)
    q = np.array([0.511, -1.0, 0.511, 0.611, 1.0, 0.611], np.float32)
    ref = _brute(tris, q, "aabb")
    assert len(ref) > 0
    p = BvhBuildParams.fast_build()
    aabbs = T.tri_aabbs(tris)
    nodes, pidx, _, _ = O.build_bvh2(tris=tris, params=p)
    got = O.query(nodes, pidx, q[None], "aabb", aabbs)[0]
    assert len(got) == len(ref) and int(got.astype(np.uint64).sum()) == int(ref.sum())
    cw = O.build(tris=tris, params=p)
    got = O.query(cw.cw_nodes, cw.cw_pidx, q[None], "aabb", aabbs)[0]
    assert len(got) == len(ref) and int(got.astype(np.uint64).sum()) == int(ref.sum())


def test_traverse_point():
    """traverse_point (tests/mod.rs:249-323): icosphere(0), fast_build, 512
    points on the unit sphere (uniform_sample_sphere of hash_noise)."""
    tris = T.icosphere(0)
    aabbs = T.tri_aabbs(tris)
    p = BvhBuildParams.fast_build()
    nodes, pidx, _, _ = O.build_bvh2(tris=tris, params=p)
    cw = O.build(tris=tris, params=p)
    u0 = np.array([T.hash_noise(0, 0, i) for i in range(512)], np.float32)
    u1 = np.array([T.hash_noise(0, 1, i) for i in range(512)], np.float32)
    pts = T.uniform_sample_sphere(u0, u1)
    b2 = O.query(nodes, pidx, pts, "point", aabbs)
    c8 = O.query(cw.cw_nodes, cw.cw_pidx, pts, "point", aabbs)
    total = 0
    for i in range(512):
        ref = _brute(tris, pts[i], "point")
        total += len(ref)
        for got in (b2[i], c8[i]):
            assert len(got) == len(ref) and int(got.astype(np.uint64).sum()) == int(ref.sum())
    assert total > 0
