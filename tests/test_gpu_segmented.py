"""Segmented builds (every stage once for a whole batch of scenes): each
scene's CWBVH byte-identical to building it alone, which the parity tests pin
to the oracle; traversal of the results identical to per-scene traversal."""
import numpy as np
import pytest

from oracle import oracle as O
from obvhs_gb300 import scenes as S
from obvhs_gb300 import test_util as T
from obvhs_gb300.params import PRESETS, BvhBuildParams

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import obvhs_gb300 as g

    return g


def _same(a, b):
    return a[0].tobytes() == b[0].tobytes() and a[1].tobytes() == b[1].tobytes()


def _rays_for(tris, n, seed):
    v = tris.reshape(-1, 3)
    lo, hi = v.min(0), v.max(0)
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    d = T.uniform_sample_sphere(rng.random(n).astype(np.float32), rng.random(n).astype(np.float32))
    return T.make_rays(o, d, 0.0, np.inf)


def _ragged(seed):
    """Empty, one-, two- and three-triangle scenes beside larger ones."""
    rng = np.random.default_rng(seed)
    sizes = [0, 1, 2, 3, 17, 100, 1000, 5000, 20_000, 2, 0, 60_000, 7]
    out = []
    for i, n in enumerate(sizes):
        if n >= 1000:
            out.append(S.scene2_tris(n, offset=100 + i))
        else:
            c = rng.uniform(-1, 1, size=(n, 1, 3))
            out.append((c + rng.uniform(-0.1, 0.1, size=(n, 3, 3))).reshape(-1, 9).astype(np.float32))
    return out


@pytest.mark.parametrize("preset", ["fastest", "very_fast", "fast", "medium", "slow", "very_slow"])
def test_segmented_equals_single_builds(G, preset):
    scenes = _ragged(7)
    p = PRESETS[preset]()
    seg = G.build_cwbvh_from_tris_segmented(scenes, p)
    for tris, cw in zip(scenes, seg):
        one = G.build_cwbvh_from_tris(tris, p)
        assert _same(cw.download(), one.download())
        assert cw.stats.leaf_count == one.stats.leaf_count
        assert cw.stats.ploc_passes == one.stats.ploc_passes
        assert np.array_equal(np.asarray(cw.total_aabb), np.asarray(one.total_aabb))
        one.free()


def test_segmented_matches_the_oracle(G):
    scenes = _ragged(8)
    p = BvhBuildParams.medium_build()
    seg = G.build_cwbvh_from_tris_segmented(scenes, p)
    for tris, cw in zip(scenes, seg):
        if len(tris) == 0:
            assert cw.download()[0].shape[0] == 0
            continue
        ob = O.build(tris=tris, params=p, nthreads=8, keep_intermediate=False)
        nodes, prims = cw.download()
        assert nodes.tobytes() == ob.cw_nodes.tobytes()
        assert prims.tobytes() == ob.cw_pidx.tobytes()


def test_many_scenes_and_device_inputs(G):
    """300 scenes (two scene-key digits) from device tensors; closest hits of
    all scenes in one multi-BVH launch equal per-scene traversal."""
    import torch

    rng = np.random.default_rng(11)
    sizes = np.exp(rng.uniform(np.log(50), np.log(30_000), size=300)).astype(int)
    scenes = [S.scene2_tris(int(n), offset=i) for i, n in enumerate(sizes)]
    p = BvhBuildParams.medium_build()
    seg = G.build_cwbvh_from_tris_segmented([torch.from_numpy(t).cuda() for t in scenes], p)
    pick = [0, 1, 2, 57, 150, 299] + list(np.argsort(sizes)[-3:])
    for i in pick:
        one = G.build_cwbvh_from_tris(scenes[i], p)
        assert _same(seg[i].download(), one.download())
        one.free()
    rays, owner, eid, et = [], [], [], []
    for i in pick:
        r = _rays_for(scenes[i], 2000, i)
        ids, t = seg[i].ray_traverse(r)
        rays.append(r)
        owner.append(np.full(len(r), i, np.uint32))
        eid.append(ids)
        et.append(t)
    ids, t = G.ray_traverse_multi(seg, np.concatenate(owner), np.concatenate(rays))
    assert np.array_equal(ids, np.concatenate(eid))
    assert np.array_equal(t.view(np.uint32), np.concatenate(et).view(np.uint32))


def test_results_outlive_their_batch_mates(G):
    """Results share one allocation: freeing some leaves the others intact."""
    scenes = [S.scene2_tris(n, offset=i) for i, n in enumerate([3000, 4000, 5000, 6000])]
    p = BvhBuildParams.fast_build()
    seg = G.build_cwbvh_from_tris_segmented(scenes, p)
    keep = seg[2]
    expect = keep.download()
    r = _rays_for(scenes[2], 4000, 5)
    ids0, t0 = keep.ray_traverse(r)
    for k in (0, 1, 3):
        seg[k].free()
    del seg
    assert _same(keep.download(), expect)
    ids, t = keep.ray_traverse(r)
    assert np.array_equal(ids, ids0) and np.array_equal(t.view(np.uint32), t0.view(np.uint32))


def test_nan_scene_fails_the_batch_and_the_context_recovers(G):
    scenes = [S.scene2_tris(2000, offset=1), S.scene2_tris(3000, offset=2)]
    bad = scenes[1].copy()
    bad[17, 7] = np.nan  # v2.y: a NaN in v0 or v1 is dropped by the min/max order
    p = BvhBuildParams.medium_build()
    ctx = G.Context(0)
    try:
        with pytest.raises(G.ObvhsError):
            G.build_cwbvh_from_tris_segmented([scenes[0], bad], p, ctx=ctx)
        seg = G.build_cwbvh_from_tris_segmented(scenes, p, ctx=ctx)
        one = G.build_cwbvh_from_tris(scenes[1], p, ctx=ctx)
        assert _same(seg[1].download(), one.download())
    finally:
        ctx.close()


def test_segmented_while_other_contexts_are_live(G):
    """With several contexts on the GPU the cooperative launches go through
    the shared stream; results are unchanged."""
    scenes = _ragged(9)
    p = BvhBuildParams.slow_build()
    others = [G.Context(0) for _ in range(2)]
    try:
        seg = G.build_cwbvh_from_tris_segmented(scenes, p)
        for tris, cw in zip(scenes, seg):
            one = G.build_cwbvh_from_tris(tris, p)
            assert _same(cw.download(), one.download())
            one.free()
    finally:
        for c in others:
            c.close()


def _deep_chain(n=220):
    """Triangles along the x axis with gaps growing by 8% each: nearest
    neighbours point back along the chain, so PLOC merges only a few pairs per
    pass (115 passes for 220 triangles with slow_build's search: more than 95,
    the unclamped reinsertion search stack)."""
    x = np.cumsum(1.08 ** np.arange(n)).astype(np.float32)
    t = np.zeros((n, 3, 3), np.float32)
    t[:, 0, 0] = x
    t[:, 1, 0] = x + 0.01
    t[:, 2, 0] = x
    t[:, 2, 1] = 0.01
    return t.reshape(-1, 9)


def test_deep_scene_alone_and_in_a_batch(G):
    """A scene whose PLOC needs more than 95 passes (reinsertion with the
    unclamped search stack), alone against the oracle, and in a segmented
    batch beside ordinary scenes (per-scene stack modes in one launch)."""
    deep = _deep_chain()
    p = BvhBuildParams.slow_build()
    p.pre_split = False  # keep the chain exact: pre-splits would add leaves
    one = G.build_cwbvh_from_tris(deep, p)
    assert one.stats.ploc_passes > 95
    ob = O.build(tris=deep, params=p, nthreads=4, keep_intermediate=False)
    nodes, prims = one.download()
    assert nodes.tobytes() == ob.cw_nodes.tobytes() and prims.tobytes() == ob.cw_pidx.tobytes()
    assert one.stats.reinsertions == ob.reinsertions
    scenes = [S.scene2_tris(3000, offset=1), deep, S.scene2_tris(20_000, offset=2)]
    seg = G.build_cwbvh_from_tris_segmented(scenes, p)
    for tris, cw in zip(scenes, seg):
        alone = G.build_cwbvh_from_tris(tris, p)
        assert _same(cw.download(), alone.download())
        alone.free()
