"""The BVH2 product on the GPU (leaf collapsing, build_bvh2_from_tris /
build_bvh2, Bvh2::ray_traverse / ray_traverse_miss) against the oracle, bit
for bit."""
import numpy as np
import pytest

from oracle import oracle as O
from obvhs_gb300 import scenes as S
from obvhs_gb300 import test_util as T
from obvhs_gb300.params import PRESETS, BvhBuildParams

pytestmark = pytest.mark.gpu

F32_MAX = np.finfo(np.float32).max
EMPTY = np.array([[F32_MAX] * 3 + [-F32_MAX] * 3], np.float32)
INF10 = np.array([[-np.inf] * 3 + [np.inf] * 3] * 10, np.float32)
MAX10 = np.array([[-F32_MAX] * 3 + [F32_MAX] * 3] * 10, np.float32)
NOTHING = np.zeros((0, 6), np.float32)


@pytest.fixture(scope="module")
def G():
    import obvhs_gb300 as g

    return g


def _same(a, b):
    return np.ascontiguousarray(a).tobytes() == np.ascontiguousarray(b).tobytes()


def _rays(tris, n, seed):
    v = tris.reshape(-1, 3)
    rng = np.random.default_rng(seed)
    o = rng.uniform(v.min(0), v.max(0), size=(n, 3)).astype(np.float32)
    d = T.uniform_sample_sphere(rng.random(n).astype(np.float32), rng.random(n).astype(np.float32))
    return T.make_rays(o, d, 0.0, np.inf)


@pytest.mark.parametrize("max_prims,cost", [(2, 1.0), (3, 3.0), (8, 3.0), (255, 1.0), (4, 0.0)])
def test_collapse_matches_oracle(G, max_prims, cost):
    tris = T.demoscene(64, 1)
    aabbs = T.tri_aabbs(tris)
    b2 = G.PlocBuilder().build_ploc(14, aabbs, None, 0, 0)
    nodes, pidx = b2.download()
    b2.collapse(max_prims, cost)
    gn, gp = b2.download()
    on, op = O.collapse(nodes, pidx, max_prims, cost)
    assert _same(gn, on) and _same(gp, op)


@pytest.mark.parametrize("preset", list(PRESETS))
def test_build_bvh2_from_tris_matches_oracle(G, preset):
    tris = S.scene2_tris(30_000, offset=5)
    p = PRESETS[preset]()
    b = G.build_bvh2_from_tris(tris, p)
    gn, gp = b.download()
    on, op, md, applied = O.build_bvh2(tris=tris, params=p, nthreads=8)
    assert _same(gn, on) and _same(gp, op)
    assert b.max_depth == md
    assert b.stats.reinsertions == applied
    rays = _rays(tris, 20_000, 3)
    ids, t = b.ray_traverse(rays)
    oid, ot = O.traverse_bvh2(on, op, tris, rays, nthreads=8)
    assert np.array_equal(ids, oid)
    assert np.array_equal(t.view(np.uint32), ot.view(np.uint32))
    assert np.array_equal(b.ray_traverse_miss(rays), ~O.traverse_bvh2(on, op, tris, rays, mode=1, nthreads=8))


@pytest.mark.parametrize("preset", ["fastest", "medium", "very_slow"])
@pytest.mark.parametrize("aabbs", [EMPTY, INF10, MAX10, NOTHING], ids=["empty", "inf", "max", "nothing"])
def test_degenerate_build_bvh2_misses(G, preset, aabbs):
    """build_bvh2_with_{empty_aabb,many_inf,many_max,nothing} (tests/mod.rs:34-78)."""
    p = PRESETS[preset]()
    b = G.build_bvh2(aabbs, p)
    gn, gp = b.download()
    on, op, _, _ = O.build_bvh2(aabbs=aabbs, params=p)
    assert _same(gn, on) and _same(gp, op)
    b.set_triangles(np.zeros((len(aabbs), 9), np.float32))  # triangles that never hit
    ids, _ = b.ray_traverse(T.make_rays([[0, 0, 1]], [[0, 0, -1]]))
    assert ids[0] == 0xFFFFFFFF


def test_varying_prim_counts_build_bvh2(G):
    """build_bvh_with_varying_prim_counts (tests/mod.rs:90-102), BVH2 half."""
    tris_all = T.height_to_triangles(T.flat_heights(4, 4), 4, 4)
    for n in range(len(tris_all) - 1, 0, -4):
        tris = tris_all[:n]
        for preset in PRESETS:
            p = PRESETS[preset]()
            gn, gp = G.build_bvh2_from_tris(tris, p).download()
            on, op, _, _ = O.build_bvh2(tris=tris, params=p)
            assert _same(gn, on) and _same(gp, op), (n, preset)


def test_large_bvh2_build_and_traversal(G):
    tris = S.scene2_tris(1_000_000)
    p = BvhBuildParams.medium_build()
    b = G.build_bvh2_from_tris(tris, p)
    on, op, _, _ = O.build_bvh2(tris=tris, params=p, nthreads=16)
    gn, gp = b.download()
    assert _same(gn, on) and _same(gp, op)
    rays = _rays(tris, 100_000, 8)
    ids, t = b.ray_traverse(rays)
    oid, ot = O.traverse_bvh2(on, op, tris, rays, nthreads=16)
    assert np.array_equal(ids, oid) and np.array_equal(t.view(np.uint32), ot.view(np.uint32))


# --- dynamic updates: refit_all, full / partial rebuild ------------------------------


def _leaf_ids(nodes):
    return np.nonzero(nodes[:, 12:16].copy().view(np.uint32).ravel() != 0)[0].astype(np.uint32)


def _moved(nodes, pidx, aabbs, frac, seed, shift=0.3):
    """A copy of the tree with `frac` of its leaves shifted (and the boxes)."""
    leaves = _leaf_ids(nodes)
    rng = np.random.default_rng(seed)
    moved = np.sort(rng.choice(leaves, size=max(1, int(len(leaves) * frac)), replace=False)).astype(np.uint32)
    nn = nodes.copy()
    boxes = np.zeros((len(moved), 6), np.float32)
    for k, i in enumerate(moved):
        f = nn[i].view(np.float32)
        f[[0, 1, 2, 4, 5, 6]] += np.float32(shift)
        boxes[k] = f[[0, 1, 2, 4, 5, 6]]
    return nn, moved, boxes


def test_refit_all_matches_oracle(G):
    tris = S.scene2_tris(200_000, offset=2)
    b = G.build_bvh2_from_tris(tris, BvhBuildParams.medium_build())
    nodes, pidx = b.download()
    nn, moved, boxes = _moved(nodes, pidx, None, 0.05, 1)
    b.set_node_aabbs(moved, boxes)
    assert _same(b.download()[0], nn)
    b.refit_all()
    assert _same(b.download()[0], O.refit_all(nn))


@pytest.mark.parametrize("radius,thr", [(1, 1), (14, 0), (24, 2)])
def test_full_rebuild_matches_oracle(G, radius, thr):
    tris = S.scene2_tris(100_000, offset=3)
    b = G.build_bvh2_from_tris(tris, BvhBuildParams.slow_build())  # collapsed, multi-primitive leaves
    nodes, _ = b.download()
    b.full_rebuild(radius, 0, thr)
    on, omd = O.rebuild(nodes, None, radius, 0, thr)
    assert _same(b.download()[0], on)
    assert b.max_depth == omd


@pytest.mark.parametrize("which", ["all", "one", "random", "moved"])
def test_partial_rebuild_matches_oracle(G, which):
    tris = S.scene2_tris(60_000, offset=4)
    aabbs = T.tri_aabbs(tris)
    b = G.PlocBuilder().build_ploc(14, aabbs, None, 0, 0)
    nodes, pidx = b.download()
    leaves = _leaf_ids(nodes)
    if which == "all":
        pick = leaves
    elif which == "one":
        pick = leaves[:1]
    elif which == "random":
        pick = np.array([i for i in leaves[:5000] if T.hash_noise(0, 0, int(i)) > 0.5], np.uint32)
    else:
        nodes, pick, boxes = _moved(nodes, pidx, aabbs, 0.05, 7)
        b.set_node_aabbs(pick, boxes)
        aabbs = aabbs.copy()  # the moved leaves' primitives moved with them
        for i, box in zip(pick, boxes):
            aabbs[pidx[nodes[i, 28:32].view(np.uint32)[0]]] = box
    b.partial_rebuild(pick, 14, 0, 0)
    on, omd = O.rebuild(nodes, pick, 14, 0, 0)
    assert _same(b.download()[0], on)
    assert b.max_depth == omd
    assert O.validate_bvh2(on, pidx, omd, aabbs)[0] == 0


def test_partial_rebuild_large(G):
    """Every leaf of a 1M-leaf tree through the partial rebuild (the largest
    collection the top-down walk can meet)."""
    tris = S.scene2_tris(1_000_000)
    aabbs = T.tri_aabbs(tris)
    b = G.PlocBuilder().build_ploc(14, aabbs, None, 0, 0)
    nodes, pidx = b.download()
    nn, moved, boxes = _moved(nodes, pidx, aabbs, 0.01, 9)
    b.set_node_aabbs(moved, boxes)
    b.partial_rebuild(moved, 14, 0, 0)
    on, _ = O.rebuild(nn, moved, 14, 0, 0)
    assert _same(b.download()[0], on)


# --- AABB and point queries -------------------------------------------------------


def _query_inputs(tris, n, seed):
    v = tris.reshape(-1, 3)
    lo, hi = v.min(0), v.max(0)
    rng = np.random.default_rng(seed)
    c = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    h = (rng.random((n, 1)) * 0.05 * (hi - lo).max()).astype(np.float32)
    boxes = np.concatenate([c - h, c + h], 1)
    # triangle centroids: inside their own boxes, so the filtered lists are not empty
    t = tris.reshape(-1, 3, 3)[rng.integers(0, len(tris), size=n)]
    pts = ((t[:, 0] + t[:, 1] + t[:, 2]) / np.float32(3)).astype(np.float32)
    return boxes, pts


@pytest.mark.parametrize("filtered", [False, True])
def test_queries_match_oracle(G, filtered):
    """Per query the same primitive ids in the same order as the oracle's
    restatement of aabb_traverse / point_traverse and of the traverse! loop
    with the node query tests; with the exact filter, the same sets as testing
    every triangle."""
    tris = S.scene2_tris(200_000, offset=6)
    aabbs = T.tri_aabbs(tris)
    p = BvhBuildParams.fast_build()
    b2 = G.build_bvh2_from_tris(tris, p)
    cw = G.build_cwbvh_from_tris(tris, p)
    n2, p2 = b2.download()
    n8, p8 = cw.download()
    boxes, pts = _query_inputs(tris, 3000, 2)
    pa = aabbs if filtered else None
    d = np.array([0.3, -0.5, 0.8], np.float32)
    for kind, q in (("aabb", boxes), ("point", pts)):
        g2 = b2.aabb_query(q, pa) if kind == "aabb" else b2.point_query(q, pa)
        o2 = O.query(n2, p2, q, kind, pa)
        g8 = cw.aabb_query(q, pa, d) if kind == "aabb" else cw.point_query(q, pa, d)
        o8 = O.query(n8, p8, q, kind, pa, d)
        assert all(np.array_equal(a, b) for a, b in zip(g2, o2))
        assert all(np.array_equal(a, b) for a, b in zip(g8, o8))
        assert sum(len(a) for a in g2) > 0
        if filtered:
            for a, b in zip(g2, g8):
                assert np.array_equal(np.sort(a), np.sort(b))
