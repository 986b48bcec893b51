"""The serving loop on the GPU: every ray batch's hits, served in the mix
(continuous batching, evictions and rebuilds under a small HBM budget), equal
the hits of its scene built and traced alone."""
import numpy as np
import pytest

from obvhs_gb300 import serve
from obvhs_gb300.params import BvhBuildParams

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import obvhs_gb300 as g

    return g


@pytest.fixture(scope="module")
def pools():
    return serve.clustered_pools(3, 60_000, 30_000, seed=17)


def _stream(pools, seed):
    tris, rays = pools
    rng = np.random.default_rng(seed)
    reqs, scene_of = serve.make_stream(160, 4000.0, tris, rays, rng, tri_range=(2000, 60_000),
                                       ray_range=(1000, 30_000), preloaded=2)
    pre = [(i, tris[scene_of[i]][:20_000]) for i in range(2)]
    return reqs, pre


def _check_alone(G, reqs, pre, p):
    src = dict(pre)
    src.update({r.bvh_id: r.tris for r in reqs if r.kind == "build"})
    alone = {}
    for r in reqs:
        assert r.done is not None
        if r.kind != "rays":
            continue
        if r.bvh_id not in alone:
            alone[r.bvh_id] = G.build_cwbvh_from_tris(src[r.bvh_id], p)
        ids, t = alone[r.bvh_id].ray_traverse(r.rays)
        assert np.array_equal(r.result[0], ids)
        assert np.array_equal(r.result[1].view(np.uint32), t.view(np.uint32))
    for b in alone.values():
        b.free()


@pytest.mark.parametrize("server", ["continuous", "plain"])
def test_served_hits_equal_alone(G, pools, server):
    p = BvhBuildParams.medium_build()
    reqs, pre = _stream(pools, 3)
    be = serve.GpuBackend(p)
    budget = 16 << 20  # a few scenes: forces evictions and rebuilds
    try:
        s = serve.ContinuousServer(be, budget) if server == "continuous" else serve.PlainServer(be, budget)
        s.run(reqs, preload=pre)
        assert s.store.evictions > 0
        assert s.store.bytes <= budget
        _check_alone(G, reqs, pre, p)
        if server == "continuous":
            n_rays = sum(r.kind == "rays" for r in reqs)
            assert s.steps["rays"] < n_rays  # batches were coalesced
        summ = serve.summarize(reqs)
        assert summ["latency_rays"]["p99_ms"] > 0
    finally:
        for k in list(s.store.items):
            s.store.items.pop(k)[0].free()
        be.close()


def test_traverse_batches_equals_alone(G, pools):
    """Host ray batches of several BVHs (repeated BVHs, an empty batch) in one
    launch: each batch's hits equal its BVH's traversal alone."""
    tris, rays = pools
    p = BvhBuildParams.fast_build()
    bvhs = [G.build_cwbvh_from_tris(tris[k][: 10_000 * (k + 1)], p) for k in range(3)]
    rng = np.random.default_rng(9)
    batch_bvh, batches = [], []
    for j in range(7):
        k = int(rng.integers(3))
        src = rays[k][j % 2]
        n = 0 if j == 3 else int(rng.integers(500, 20_000))
        batch_bvh.append(k)
        batches.append(np.ascontiguousarray(src[:n]))
    outs = G.ray_traverse_batches(bvhs, batch_bvh, batches)
    for k, r, o in zip(batch_bvh, batches, outs):
        ids, t = bvhs[k].ray_traverse(r)
        assert np.array_equal(o[:, 0], ids)
        assert np.array_equal(o[:, 1], t.view(np.uint32))
    for b in bvhs:
        b.free()


def test_large_traverse_batches_pipelined_equal_alone(G):
    """A call of more than 2M rays (copies pipelined with the traversal in
    runs of batches on separate streams) gives each batch the hits of its BVH
    traversed alone, from pinned and from pageable host memory."""
    import torch
    from obvhs_gb300 import scenes as S
    from obvhs_gb300 import test_util as T

    p = BvhBuildParams.fast_build()
    bvhs = [G.build_cwbvh_from_tris(S.scene2_tris(n, offset=k), p) for k, n in enumerate((40_000, 120_000))]
    rng = np.random.default_rng(21)
    batch_bvh, batches = [], []
    for j, n in enumerate((900_000, 3, 0, 700_000, 650_000, 1, 400_000)):
        o = rng.uniform(-12, 12, size=(n, 3)).astype(np.float32)
        d = T.uniform_sample_sphere(rng.random(n).astype(np.float32), rng.random(n).astype(np.float32))
        r = T.make_rays(o, d, 0.0, np.inf)
        if j % 2:
            pinned = torch.empty((n, 8), dtype=torch.float32).pin_memory().numpy()
            pinned[:] = r
            r = pinned
        batch_bvh.append(j % 2)
        batches.append(r)
    outs = G.ray_traverse_batches(bvhs, batch_bvh, batches)
    for k, r, o in zip(batch_bvh, batches, outs):
        ids, t = bvhs[k].ray_traverse(r)
        assert np.array_equal(o[:, 0], ids)
        assert np.array_equal(o[:, 1], t.view(np.uint32))
    for b in bvhs:
        b.free()
