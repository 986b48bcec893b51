"""Batched builds (many scenes, several contexts at once) and multi-BVH
traversal: every result identical to its one-scene counterpart."""
import numpy as np
import pytest

from obvhs_gb300 import scenes as S
from obvhs_gb300 import test_util as T
from obvhs_gb300.params import BvhBuildParams

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import obvhs_gb300 as g

    return g


def _scenes(k, seed, clustered=False):
    """k scenes of 1k-60k triangles (log-uniform): the clustered generator, or
    triangles of edge up to ~0.6 in a cube of side 6 (many ray hits)."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(1000), np.log(60_000), size=k)).astype(int)
    if clustered:
        return [S.scene2_tris(int(n), offset=i) for i, n in enumerate(sizes)]
    out = []
    for n in sizes:
        c = rng.uniform(-3, 3, size=(int(n), 1, 3))
        out.append((c + rng.uniform(-0.3, 0.3, size=(int(n), 3, 3))).reshape(-1, 9).astype(np.float32))
    return out


def _rays_for(tris, n, seed):
    v = tris.reshape(-1, 3)
    lo, hi = v.min(0), v.max(0)
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    d = T.uniform_sample_sphere(rng.random(n).astype(np.float32), rng.random(n).astype(np.float32))
    return T.make_rays(o, d, 0.0, np.inf)


@pytest.mark.parametrize("preset,n_ctx", [("medium_build", 4), ("slow_build", 3)])
def test_batched_builds_equal_single_builds(G, preset, n_ctx):
    scenes = _scenes(24, 1 if n_ctx == 4 else 2, clustered=True)
    p = getattr(BvhBuildParams, preset)()
    ctxs = [G.Context(0) for _ in range(n_ctx)]
    try:
        batch = G.build_cwbvh_from_tris_batch(scenes, p, ctxs)
        for tris, cw in zip(scenes, batch):
            one = G.build_cwbvh_from_tris(tris, p, ctx=ctxs[0])
            a, b = cw.download(), one.download()
            assert a[0].tobytes() == b[0].tobytes() and a[1].tobytes() == b[1].tobytes()
            assert cw.stats.leaf_count == one.stats.leaf_count
            cw.free()
            one.free()
    finally:
        for c in ctxs:
            c.close()


def test_multi_bvh_traversal_equals_per_bvh(G):
    scenes = _scenes(16, 3)
    p = BvhBuildParams.medium_build()
    ctxs = [G.Context(0) for _ in range(2)]
    request_cleanup = ctxs
    bvhs = G.build_cwbvh_from_tris_batch(scenes, p, ctxs)
    rays, owner, expect_id, expect_t = [], [], [], []
    for i, (tris, cw) in enumerate(zip(scenes, bvhs)):
        r = _rays_for(tris, 3000 + 500 * i, i)
        ids, t = cw.ray_traverse(r)
        rays.append(r)
        owner.append(np.full(len(r), i, np.uint32))
        expect_id.append(ids)
        expect_t.append(t)
    rays = np.concatenate(rays)
    owner = np.concatenate(owner)
    perm = np.random.default_rng(4).permutation(len(rays))  # interleaved BVHs
    ids, t = G.ray_traverse_multi(bvhs, owner[perm], rays[perm], ctx=ctxs[0])
    assert np.array_equal(ids, np.concatenate(expect_id)[perm])
    assert np.array_equal(t.view(np.uint32), np.concatenate(expect_t)[perm].view(np.uint32))
    assert (ids != 0xFFFFFFFF).sum() > 1000
    for b in bvhs:
        b.free()
    for c in request_cleanup:
        c.close()


def test_batched_build_error_frees_everything_and_contexts_recover(G):
    scenes = _scenes(8, 5)
    bad = scenes[3].copy()
    bad[7, 6] = np.nan
    scenes[3] = bad
    ctxs = [G.Context(0) for _ in range(3)]
    with pytest.raises(G.ObvhsError) as e:
        G.build_cwbvh_from_tris_batch(scenes, BvhBuildParams.medium_build(), ctxs)
    assert e.value.code == -4
    ok = G.build_cwbvh_from_tris_batch(scenes[:3], BvhBuildParams.medium_build(), ctxs)
    assert len(ok) == 3 and all(b.info()[0] > 0 for b in ok)
    for b in ok:
        b.free()
    for c in ctxs:
        c.close()


def test_shared_gpu_paths_match_the_oracle(G):
    """On a context marked as sharing the GPU (the form builds take while
    several are in flight), PLOC and conflict resolution run as single blocks
    with normal launches; the result is the same tree as the whole-GPU
    cooperative forms and the oracle."""
    from oracle import oracle as O

    tris = S.scene2_tris(200_000, offset=9)
    p = BvhBuildParams.slow_build()
    extra, other = G.Context(0), G.Context(0)  # two live contexts: cooperative launches take the shared stream
    extra.set_shared_gpu(True)
    try:
        cw = G.build_cwbvh_from_tris(tris, p, ctx=extra)
        nodes, prims = cw.download()
        ob = O.build(tris=tris, params=p, nthreads=8, keep_intermediate=False)
        assert nodes.tobytes() == ob.cw_nodes.tobytes() and prims.tobytes() == ob.cw_pidx.tobytes()
        assert cw.stats.reinsertions == ob.reinsertions
        cw.free()
    finally:
        extra.close()
        other.close()
