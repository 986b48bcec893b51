"""CUDA path vs the oracle, stage by stage, bit for bit (needs a GPU).

Every comparison is exact (np.array_equal on raw bytes): Morton codes and
sorted order, the PLOC BVH2 nodes, the tree after reinsertion, the 80-byte
CWBVH nodes and primitive indices, and closest-hit ids / t / occlusion
flags.  The reference's own pins (prim 62, 65,536 plane hits, kitchen hash
1343358762) are also run end to end on the GPU.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from obvhs_gb300 import scenes as S
from obvhs_gb300 import test_util as T
from obvhs_gb300.params import PRESETS, BvhBuildParams, SortPrecision

import helpers as H

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import obvhs_gb300 as g

    return g


def _random_aabbs(n, seed, spread=5.0, size=0.05):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-spread, spread, size=(n, 3))
    e = rng.uniform(0, size, size=(n, 3))
    return np.concatenate([c - e, c + e], 1).astype(np.float32)


def _eq(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    return a.shape == b.shape and a.tobytes() == b.tobytes()


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("n", [1, 2, 7, 1000, 100_003])
def test_morton_and_order(G, n, precision):
    a = _random_aabbs(n, 10 + n)
    codes, order = G.morton_sort(a, precision)
    ocodes, oorder = O.morton(a, precision)
    assert _eq(codes, ocodes)
    assert _eq(order, oorder)


def _edge_scene(kind, seed=31):
    """Boxes whose Morton inputs reach the conversions' edge cases."""
    rng = np.random.default_rng(seed)
    f = np.float32
    if kind == "edges":  # centres on the scene's min and max corners, at 0 and -0
        a = _random_aabbs(3000, seed)
        lo, hi = a[:, :3].min(0), a[:, 3:].max(0)
        pts = [lo, hi, np.array([lo[0], hi[1], 0], f), np.zeros(3, f), np.full(3, -0.0, f)]
        extra = np.array([np.concatenate([p, p]) for p in pts] + [[-1, -1, -1, 1, 1, 1]], f)
        return np.concatenate([a, extra]).astype(f)
    if kind == "subnormal":  # centres that are subnormal floats
        c = rng.uniform(-2e-38, 2e-38, size=(3000, 3)).astype(f)
        c[::5] = (rng.integers(-50, 50, size=c[::5].shape) * 1e-45).astype(f)
        c[::11] = 0.0
        return np.concatenate([c, c], 1).astype(f)
    if kind == "huge":  # centres near the float maximum, some of them inf
        c = rng.uniform(1e38, 3.0e38, size=(3000, 3)).astype(f)
        a = np.concatenate([c, c], 1)
        a[::17, :3] = 3.3e38
        a[::17, 3:] = 3.4e38  # centre (a + b) * 0.5 overflows to inf
        return a.astype(f)
    if kind == "huge-extent":  # the scene's extent overflows to inf: zero scale
        c = rng.uniform(-3.3e38, 3.3e38, size=(3000, 3)).astype(f)
        return np.concatenate([c, c], 1).astype(f)
    if kind == "flat":  # one axis of zero extent: infinite scale, NaN products
        a = _random_aabbs(3000, seed)
        a[:, 2] = a[:, 5] = 2.5
        return a
    if kind == "flat-zero":
        a = _random_aabbs(3000, seed)
        a[:, 1] = a[:, 4] = 0.0
        return a
    raise ValueError(kind)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("kind", ["edges", "subnormal", "huge", "huge-extent", "flat", "flat-zero"])
def test_morton_edge_values(G, kind, precision):
    """Codes equal the oracle's where the float->double widening and the
    saturating double->integer conversions meet zeros, subnormals, infinities,
    NaN and the exact top of the grid."""
    a = _edge_scene(kind)
    with np.errstate(over="ignore", invalid="ignore"):
        codes, order = G.morton_sort(a, precision)
        ocodes, oorder = O.morton(a, precision)
    assert _eq(codes, ocodes)
    assert _eq(order, oorder)


def test_morton_duplicates_keep_input_order(G):
    a = np.repeat(_random_aabbs(50, 3), 40, axis=0)  # equal keys in runs
    codes, order = G.morton_sort(a, 0)
    _, oorder = O.morton(a, 0)
    assert _eq(order, oorder)


def test_morton_exact_duplicates_u128(G):
    a = np.repeat(_random_aabbs(40, 5), 50, axis=0)  # runs longer than the high-digit fix-up takes
    codes, order = G.morton_sort(a, 1)
    ocodes, oorder = O.morton(a, 1)
    assert _eq(codes, ocodes) and _eq(order, oorder)


@pytest.mark.parametrize("precision", [0, 1])
def test_morton_runs_of_equal_high_digits(G, precision):
    """Clumps of 1-32 boxes whose centres differ only below the high digits
    the sort runs on: each run is put in order by the low bits (stably)."""
    rng = np.random.default_rng(21 + precision)
    base = rng.uniform(-50, 50, size=(3000, 3))
    reps = rng.integers(1, 33, size=len(base))
    c = np.repeat(base, reps, axis=0)
    jitter = 2e-3 if precision == 0 else 1e-5
    c = c + rng.uniform(-jitter, jitter, size=c.shape)
    c[::7] = np.repeat(base, reps, axis=0)[::7]  # some exact duplicates inside runs too
    perm = rng.permutation(len(c))
    c = c[perm]
    a = np.concatenate([c - 1e-6, c + 1e-6], 1).astype(np.float32)
    codes, order = G.morton_sort(a, precision)
    ocodes, oorder = O.morton(a, precision)
    assert _eq(codes, ocodes) and _eq(order, oorder)
    # the runs exist: many neighbours in sorted order share their high digits
    srt = ocodes[oorder]
    hi = srt[:, 1] if precision else srt[:, 0] >> np.uint64(24)
    assert (hi[1:] == hi[:-1]).sum() > 1000


@pytest.mark.parametrize("radius,threshold,precision", [(1, 0, 0), (2, 1, 0), (6, 2, 0), (14, 3, 0), (16, 0, 0),
                                                        (24, 2, 1), (32, 0, 1)])
@pytest.mark.parametrize("n", [2, 3, 17, 2048, 2049, 50_000])
def test_ploc_bitexact(G, n, radius, threshold, precision):
    a = _random_aabbs(n, n * 7 + radius)
    b = G.PlocBuilder().build_ploc(radius, a, None, precision, threshold)
    nodes, pidx = b.download()
    on, op, omd, _ = O.ploc(a, None, radius, precision, threshold)
    assert _eq(nodes, on)
    assert _eq(pidx, op)
    assert b.max_depth == omd


def _clumps(seed):
    """Clumps of 1-32 boxes whose centres share their high Morton digits."""
    rng = np.random.default_rng(seed)
    base = rng.uniform(-50, 50, size=(1500, 3))
    c = np.repeat(base, rng.integers(1, 33, size=len(base)), axis=0)
    c = c + rng.uniform(-2e-3, 2e-3, size=c.shape)
    c = c[rng.permutation(len(c))]
    return np.concatenate([c - 1e-6, c + 1e-6], 1).astype(np.float32)


@pytest.mark.parametrize("kind", ["dup3", "dup40", "clumps"])
def test_ploc_u64_runs_of_equal_high_digits(G, kind):
    """U64 builds whose Morton order has runs of equal high digits: runs of up
    to 32 put in order as the leaves are gathered (equal codes by input
    order), a longer run of equal codes sorting all the bits instead."""
    if kind == "clumps":
        a = _clumps(4)
    else:
        a = np.repeat(_random_aabbs(2000, 77), 3 if kind == "dup3" else 40, axis=0)
    b = G.PlocBuilder().build_ploc(14, a, None, 0, 0)
    nodes, pidx = b.download()
    on, op, omd, _ = O.ploc(a, None, 14, 0, 0)
    assert _eq(nodes, on) and _eq(pidx, op)
    assert b.max_depth == omd


def test_ploc_single_and_empty(G):
    a = _random_aabbs(1, 1)
    nodes, pidx = G.PlocBuilder().build_ploc(14, a).download()
    on, op, _, _ = O.ploc(a)
    assert _eq(nodes, on) and _eq(pidx, op)
    b = G.PlocBuilder().build_ploc(14, np.zeros((0, 6), np.float32))
    assert b.info()[:2] == (0, 0)


def test_ploc_rejects_bad_radius(G):
    with pytest.raises(ValueError):
        G.PlocBuilder().build(16, _random_aabbs(10, 1))  # PlocSearchDistance::from(16) panics


def test_ploc_nan_is_an_error(G):
    a = _random_aabbs(100, 2)
    a[17, 2] = np.nan
    with pytest.raises(G.ObvhsError):
        G.PlocBuilder().build_ploc(14, a)


@pytest.mark.parametrize("ratio", [0.05, 0.25, 1.0])
def test_reinsertion_bitexact(G, ratio):
    tris = T.demoscene(64, 1)
    a = T.tri_aabbs(tris)
    on, op, md, _ = O.ploc(a, None, 2, 0, 1)
    want, stats = O.reinsertion(on, op, md, ratio)
    b = G.Bvh2.upload(on, op, md)
    applied = G.ReinsertionOptimizer().run(b, ratio)
    got, _ = b.download()
    assert applied == int(stats[0])
    assert _eq(got, want)


def test_reinsertion_custom_sequence(G):
    a = _random_aabbs(20_000, 5)
    on, op, md, _ = O.ploc(a, None, 6, 0, 0)
    seq = [0.5, 0.2, 0.1]
    want, _ = O.reinsertion(on, op, md, 0.3, seq)
    b = G.Bvh2.upload(on, op, md)
    G.ReinsertionOptimizer().run(b, 0.3, seq)
    assert _eq(b.download()[0], want)


@pytest.mark.parametrize("max_prims", [1, 2, 3])
@pytest.mark.parametrize("order", [True, False])
def test_cwbvh_bitexact(G, max_prims, order):
    tris = T.demoscene(48, 2)
    a = T.tri_aabbs(tris)
    on, op, md, _ = O.ploc(a, None, 14, 0, 3)
    on, _ = O.reinsertion(on, op, md, 0.1)
    wn, wp = O.bvh2_to_cwbvh(on, op, max_prims, order)
    cw = G.bvh2_to_cwbvh(G.Bvh2.upload(on, op, md), max_prims, order)
    gn, gp = cw.download()
    assert _eq(gn, wn)
    assert _eq(gp, wp)


def test_presplit_bitexact(G):
    tris, _ = S.scene1(3000)
    tris = tris.copy()
    tris[::97] *= 40.0  # some large triangles to split
    ga, gi = G.split_aabbs_preset(tris)
    oa, oi = O.presplit(tris)
    assert len(ga) > len(tris)
    assert _eq(ga, oa) and _eq(gi, oi)


@pytest.mark.parametrize("preset", list(PRESETS))
def test_full_build_bitexact(G, preset):
    tris = T.demoscene(40, 3)
    tris[::53] *= 3.0
    p = PRESETS[preset]()
    cw = G.build_cwbvh_from_tris(tris, p)
    gn, gp = cw.download()
    ob = O.build(tris=tris, params=p)
    assert _eq(gn, ob.cw_nodes)
    assert _eq(gp, ob.cw_pidx)


@pytest.mark.parametrize("preset", list(PRESETS))
def test_doctest_pin_gpu(G, preset):
    tris, ray = H.doctest_scene()
    cw = G.build_cwbvh_from_tris(tris, PRESETS[preset]())
    ids, t = cw.ray_traverse(ray)
    assert ids[0] == H.DOCTEST_PRIM and np.isfinite(t[0])


def test_flat_plane_pin_gpu(G):
    tris, rays = H.plane_scene()
    cw = G.build_cwbvh_from_tris(tris, BvhBuildParams.medium_build())
    ids, _ = cw.ray_traverse(rays)
    assert (ids != 0xFFFFFFFF).all()
    n = T.compute_normal(tris[ids])
    assert np.all(n == np.array([0, 1, 0], np.float32))


@pytest.mark.parametrize("preset", ["fastest", "fast", "medium", "slow", "very_slow"])
def test_kitchen_hash_gpu(G, preset):
    tris = H.kitchen_tris()
    rays = H.kitchen_rays()
    cw = G.build_cwbvh_from_tris(tris, PRESETS[preset]())
    ids, t = cw.ray_traverse(rays)
    # kitchen_hash works on BVH-order ids; map the original ids back through
    # identity (tris are indexed by original id)
    hit = ids != 0xFFFFFFFF
    normals = np.zeros((len(rays), 3), np.float32)
    n = T.compute_normal(tris[ids[hit]])
    dd = T.dot3(n, -rays[hit, 4:7])
    sgn = np.where(np.isnan(dd), dd, np.where(np.signbit(dd), np.float32(-1), np.float32(1))).astype(np.float32)
    normals[hit] = n * sgn[:, None]
    assert T.hash_f32_bits(normals) == H.KITCHEN_HASH


EMPTY = np.array([[3.4028235e38] * 3 + [-3.4028235e38] * 3], np.float32)


@pytest.mark.parametrize("preset", list(PRESETS))
def test_degenerate_gpu(G, preset):
    p = PRESETS[preset]()
    for a in (EMPTY, np.zeros((0, 6), np.float32)):
        cw = G.build_cwbvh(a, p)
        nn, npr, _ = cw.info()
        on = O.build(aabbs=a, params=p)
        assert nn == len(on.cw_nodes) and npr == len(on.cw_pidx)
    inf10 = np.array([[-np.inf] * 3 + [np.inf] * 3] * 10, np.float32)
    nodes, pidx = G.PlocBuilder().build(p.ploc_search_distance, inf10, None, p.sort_precision,
                                        p.search_depth_threshold).download()
    on, op, _, _ = O.ploc(inf10, None, p.ploc_search_distance, p.sort_precision, p.search_depth_threshold)
    assert _eq(nodes, on)
    with pytest.raises(G.ObvhsError):
        G.build_cwbvh(inf10, BvhBuildParams.medium_build())


@pytest.mark.parametrize("preset", ["fastest", "slow"])
def test_full_build_nan_is_an_error_and_context_recovers(G, preset):
    tris = T.demoscene(20, 3)
    bad = tris.copy()
    # the last vertex: min/max with the SSE semantics (a < b ? a : b) keep a
    # NaN only in the second operand, so the box is NaN and the build must fail
    bad[len(bad) // 2, 6] = np.nan
    p = PRESETS[preset]()
    with pytest.raises(G.ObvhsError) as e:
        G.build_cwbvh_from_tris(bad, p)
    assert e.value.code == -4
    cw = G.build_cwbvh_from_tris(tris, p)
    gn, gp = cw.download()
    ob = O.build(tris=tris, params=p)
    assert _eq(gn, ob.cw_nodes) and _eq(gp, ob.cw_pidx)


def test_traversal_bitexact_scene1(G):
    tris, rays = S.scene1()
    ob = O.build(tris=tris, params=BvhBuildParams.fastest_build())
    cw = G.CwBvh.upload(ob.cw_nodes, ob.cw_pidx).set_triangles(tris)
    ids, t = cw.ray_traverse(rays)
    oids, ot, _ = O.traverse(ob.cw_nodes, ob.cw_pidx, tris, rays, 0, nthreads=4)
    assert (oids != 0xFFFFFFFF).sum() > 1000
    assert _eq(ids, oids)
    assert _eq(t.view(np.uint32), ot.view(np.uint32))


def test_traversal_incoherent_and_occlusion(G):
    tris = S.scene2_tris(60_000)
    rng = np.random.default_rng(3)
    o = rng.uniform(-12, 12, size=(40_000, 3)).astype(np.float32)
    d = T.uniform_sample_sphere(rng.random(40_000).astype(np.float32), rng.random(40_000).astype(np.float32))
    tmax = rng.uniform(0.5, 30, size=40_000).astype(np.float32)
    tmax[::3] = np.inf
    rays = T.make_rays(o, d, 0.0, tmax)
    cw = G.build_cwbvh_from_tris(tris, BvhBuildParams.medium_build())
    gn, gp = cw.download()
    ids, t = cw.ray_traverse(rays)
    oids, ot, _ = O.traverse(gn, gp, tris, rays, 0, nthreads=4)
    assert _eq(ids, oids) and _eq(t.view(np.uint32), ot.view(np.uint32))
    miss = cw.ray_traverse_miss(rays)
    omiss, _, _ = O.traverse(gn, gp, tris, rays, 1, nthreads=4)
    assert _eq(miss, omiss == 0xFFFFFFFF)
    assert miss.any() and (~miss).any()


def test_traversal_outside_the_fast_slab_bounds(G):
    """Rays and nodes outside the bounds of the hardware min/max slab test
    (infinite, NaN or huge origins and directions, NaN tmax; needle triangles
    whose nodes have exponent bytes above 200 and |p| above 2^80) take the
    reference's select min/max; one warp holds both kinds of rays."""
    rng = np.random.default_rng(5)
    tris, _ = S.scene1()
    needles = np.zeros((6, 9), np.float32)
    needles[:, 0] = -3e25
    needles[:, 3] = 3e25
    needles[:, 6] = rng.uniform(-1, 1, 6)
    needles[:, [1, 4, 7]] = rng.uniform(-1, 1, (6, 1))
    needles[:, [2, 5, 8]] = rng.uniform(-1, 1, (6, 1))
    tris = np.concatenate([tris, needles]).astype(np.float32)
    n = 24_000
    o = rng.uniform(-1.2, 1.2, size=(n, 3)).astype(np.float32)
    d = T.uniform_sample_sphere(rng.random(n).astype(np.float32), rng.random(n).astype(np.float32))
    tmax = np.where(np.arange(n) % 2 == 0, np.inf, rng.uniform(0.5, 3, n)).astype(np.float32)
    k = np.arange(0, n, 5)
    kind = (k // 5) % 7
    o[k[kind == 0], 0] = np.inf
    d[k[kind == 1], 0] = 0.0
    d[k[kind == 1], 1] = 0.0
    o[k[kind == 2]] = np.float32(2e24)
    d[k[kind == 3], 2] = np.nan
    tmax[k[kind == 4]] = np.nan
    d[k[kind == 5], 1] = -np.inf
    o[k[kind == 6], 1] = np.nan
    rays = T.make_rays(o, d, 0.0, tmax)
    cw = G.build_cwbvh_from_tris(tris, BvhBuildParams.medium_build())
    gn, gp = cw.download()
    ids, t = cw.ray_traverse(rays)
    oids, ot, _ = O.traverse(gn, gp, tris, rays, 0, nthreads=4)
    assert (oids != 0xFFFFFFFF).sum() > 1000
    assert _eq(ids, oids) and _eq(t.view(np.uint32), ot.view(np.uint32))
    miss = cw.ray_traverse_miss(rays)
    omiss, _, _ = O.traverse(gn, gp, tris, rays, 1, nthreads=4)
    assert _eq(miss, omiss == 0xFFFFFFFF)


def test_device_pointer_path(G):
    torch = pytest.importorskip("torch")
    tris, rays = S.scene1()
    dt = torch.from_numpy(tris).cuda()
    dr = torch.from_numpy(rays).cuda()
    cw = G.build_cwbvh_from_tris(dt, BvhBuildParams.fast_build())
    out = cw.ray_traverse(dr).cpu().numpy().view(np.uint32)
    ids, t = cw.ray_traverse(rays)
    assert _eq(out[:, 0], ids) and _eq(out[:, 1], t.view(np.uint32))


# --- CWBVH post-passes -----------------------------------------------------------


def _demoscene_bvh2(G, preset="very_fast"):
    """tests/mod.rs:351-451 set-up: demoscene(100, 0) boxes, the preset's PLOC."""
    tris = T.demoscene(100, 0)
    aabbs = T.tri_aabbs(tris)
    p = PRESETS[preset]()
    b2 = G.PlocBuilder().build_ploc(int(p.ploc_search_distance), aabbs, None, int(p.sort_precision),
                                    int(p.search_depth_threshold))
    return tris, aabbs, b2


@pytest.mark.parametrize("order", [True, False])
def test_exact_node_aabbs_match_oracle(G, order):
    tris, aabbs, b2 = _demoscene_bvh2(G)
    nodes, pidx = b2.download()
    cw = G.bvh2_to_cwbvh(b2, 3, order, include_exact_node_aabbs=True)
    on, op, oe = O.bvh2_to_cwbvh_exact(nodes, pidx, 3, order)
    gn, gp = cw.download()
    assert gn.tobytes() == on.tobytes() and gp.tobytes() == op.tobytes()
    assert cw.exact_node_aabbs().tobytes() == oe.tobytes()
    assert G.bvh2_to_cwbvh(b2, 3, order).exact_node_aabbs() is None


@pytest.mark.parametrize("preset,order,exact,direct", [("very_fast", True, False, False),
                                                       ("very_fast", False, False, False),
                                                       ("very_fast", True, True, False),
                                                       ("medium", True, False, True),
                                                       ("slow", False, True, True)])
def test_order_children_post_pass_matches_oracle(G, preset, order, exact, direct):
    """CwBvh::order_children on the GPU, twice (the second pass starts from
    the reordered tree), against the oracle's sequential pass, node bytes and
    exact boxes bit for bit."""
    tris, aabbs, b2 = _demoscene_bvh2(G, preset)
    nodes, pidx = b2.download()
    cw = G.bvh2_to_cwbvh(b2, 3, order, include_exact_node_aabbs=exact)
    cn, cp = cw.download()
    prims = aabbs[cp] if direct else aabbs  # direct layout: boxes in primitive_indices order
    ex = cw.exact_node_aabbs() if exact else None
    for _ in range(2):
        cw.order_children(prims, direct_layout=direct)
        r = O.cwbvh_order_children(cn, cp, prims, direct_layout=direct, exact=ex)
        cn, ex = (r if exact else (r, None))
        gn, gp = cw.download()
        assert gn.tobytes() == cn.tobytes()
        assert gp.tobytes() == cp.tobytes()
        if exact:
            assert cw.exact_node_aabbs().tobytes() == ex.tobytes()
        assert O.validate_cwbvh(gn, gp, aabbs)[0] == 0


def test_order_node_children_one_at_a_time(G):
    tris, aabbs, b2 = _demoscene_bvh2(G)
    cw = G.bvh2_to_cwbvh(b2, 3, True)
    cn, cp = cw.download()
    for i in (0, 1, 7, len(cn) // 2, len(cn) - 1):
        cw.order_node_children(aabbs, i)
        cn = O.cwbvh_order_children(cn, cp, aabbs, node_index=i)
        assert cw.download()[0].tobytes() == cn.tobytes()


def test_order_children_large_scene(G):
    """The post-pass on a 1M-triangle clustered CWBVH: many warps in the
    queue at once."""
    from obvhs_gb300 import scenes as S

    tris = S.scene2_tris(1_000_000)
    aabbs = T.tri_aabbs(tris)
    cw = G.build_cwbvh_from_tris(tris, BvhBuildParams.medium_build())
    cn, cp = cw.download()
    cw.order_children(aabbs)
    on = O.cwbvh_order_children(cn, cp, aabbs)
    assert cw.download()[0].tobytes() == on.tobytes()


def test_dependent_launches_off_gives_the_same_tree(G, tmp_path):
    """OBVHS_PDL=0 (plain stream launches) builds the same bytes as the
    default programmatic dependent launches (read once per process, so the
    other form runs in a child process)."""
    import subprocess
    import sys

    tris = S.scene2_tris(120_000)
    p = BvhBuildParams.slow_build()
    nodes, pidx = G.build_cwbvh_from_tris(tris, p).download()
    np.save(tmp_path / "tris.npy", tris)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys, numpy as np; sys.path.insert(0, %r); import obvhs_gb300 as G; "
            "from obvhs_gb300.params import BvhBuildParams as P; "
            "n, i = G.build_cwbvh_from_tris(np.load(%r), P.slow_build()).download(); "
            "np.save(%r, n); np.save(%r, i)") % (root, str(tmp_path / "tris.npy"), str(tmp_path / "n.npy"),
                                                 str(tmp_path / "i.npy"))
    env = dict(os.environ, OBVHS_PDL="0")
    subprocess.run([sys.executable, "-c", code], env=env, check=True, timeout=300)
    assert _eq(np.load(tmp_path / "n.npy"), nodes) and _eq(np.load(tmp_path / "i.npy"), pidx)


@pytest.mark.parametrize("preset", ["slow_build", "very_slow_build"])
def test_reinsertion_global_forms_give_the_same_tree(G, tmp_path, preset):
    """OBVHS_RESOLVE_TABLES=0: the one-block reinsertion passes resolve on the
    global claim arrays and the global mark and refit (the forms used when the
    shared-memory tables overflow) and build the same bytes as the default
    (read once per process, so that form runs in a child process)."""
    import subprocess
    import sys

    tris = S.scene2_tris(200_000)
    nodes, pidx = G.build_cwbvh_from_tris(tris, getattr(BvhBuildParams, preset)()).download()
    np.save(tmp_path / "tris.npy", tris)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys, numpy as np; sys.path.insert(0, %r); import obvhs_gb300 as G; "
            "from obvhs_gb300.params import BvhBuildParams as P; "
            "n, i = G.build_cwbvh_from_tris(np.load(%r), P.%s()).download(); "
            "np.save(%r, n); np.save(%r, i)") % (root, str(tmp_path / "tris.npy"), preset, str(tmp_path / "n.npy"),
                                                 str(tmp_path / "i.npy"))
    env = dict(os.environ, OBVHS_RESOLVE_TABLES="0")
    subprocess.run([sys.executable, "-c", code], env=env, check=True, timeout=300)
    assert _eq(np.load(tmp_path / "n.npy"), nodes) and _eq(np.load(tmp_path / "i.npy"), pidx)
